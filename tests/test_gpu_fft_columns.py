"""Column FFT kernels of the j and i passes (csrc/fft2.cu) through
fftgal_fft_columns_f32, against numpy.fft in FP64: every power-of-two length
from 4 to 2048 (2048 = 32 x 64 with paired second-step lanes) and other
tuned shapes, both signs, ragged column counts, batch and element strides of
the grid's j and i passes in small form."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fg():
    from fftgal_gb300 import build
    build.build()
    import fftgal_gb300
    return fftgal_gb300


CASES = [(N, -1) for N in (4, 8, 32, 64, 128, 512, 1024, 2048)] + [(1024, 3), (1024, 4), (1024, 2), (2048, 2)]


@pytest.mark.parametrize("N,shape", CASES)
@pytest.mark.parametrize("sign", [-1, 1])
def test_columns_against_numpy(fg, N, shape, sign):
    import torch
    rng = np.random.default_rng(N + (sign > 0))
    nbatch, ncols, pitch = 3, 37, 41  # ragged: not a multiple of the columns per CTA
    a = (rng.standard_normal((nbatch, N, pitch)) + 1j * rng.standard_normal((nbatch, N, pitch))).astype(np.complex64)
    d = torch.from_numpy(a.view(np.float32)).cuda()
    torch.cuda.synchronize()
    st = fg.lib().fftgal_fft_columns_f32(N, d.data_ptr(), ncols, pitch, N * pitch, nbatch, sign, shape, None)
    assert st == 0, fg.lib().fftgal_last_error()
    got = d.cpu().numpy().view(np.complex64)
    x = a.astype(np.complex128)[:, :, :ncols]
    want = np.fft.fft(x, axis=1) if sign < 0 else np.fft.ifft(x, axis=1) * N
    err = np.linalg.norm(got[:, :, :ncols] - want) / np.linalg.norm(want)
    assert err <= 3e-7 * np.log2(N) + 1e-7, err
    np.testing.assert_array_equal(got[:, :, ncols:], a[:, :, ncols:])  # columns past ncols untouched


def test_columns_reject_unsupported_lengths(fg):
    import torch
    d = torch.zeros(2 * 96 * 8, dtype=torch.float32, device="cuda")
    assert fg.lib().fftgal_fft_columns_f32(96, d.data_ptr(), 8, 8, 96 * 8, 1, -1, -1, None) == -4
    assert fg.lib().fftgal_fft_columns_f32(4096, d.data_ptr(), 8, 8, 96 * 8, 1, -1, -1, None) == -4
    assert fg.lib().fftgal_fft_columns_f32(512, d.data_ptr(), 8, 8, 96 * 8, 1, -1, 9, None) == -1
