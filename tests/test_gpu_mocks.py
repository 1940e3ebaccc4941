"""The GPU lognormal mock generator (fftgal_gb300/mocks.py) against the numpy
one of tests/golden/lognormal.py (same algorithm, different random streams):
particle count within Poisson scatter, the measured P_0(k) and the velocity
dispersion within the scatter of a few seeds."""
import numpy as np
import pytest

from lognormal import lognormal_catalog as np_catalog

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fg():
    from fftgal_gb300 import build
    build.build()
    import fftgal_gb300
    return fftgal_gb300


def test_mocks_match_numpy_generator(fg):
    import torch
    from fftgal_gb300 import mocks
    n, L, Np, Ng = 64, 1000.0, 4e5, 64
    dK = 2 * np.pi / L
    g = fg.Grid(Ng, L, precision="f32", host_view="lazy")
    p_gpu, p_np, v_gpu, v_np = [], [], [], []
    for seed in range(1, 5):
        x, y, z, vx, vy, vz = mocks.lognormal_catalog(n, L, Np, seed)
        assert abs(x.numel() - Np) < 5 * np.sqrt(Np) + 0.02 * Np
        assert float(x.min()) >= 0 and float(x.max()) <= L
        r = g.power_f32(x.cpu().numpy(), y.cpu().numpy(), z.cpu().numpy(), L ** 3, (0, 0, 1), dK)
        p_gpu.append(r["P"][:, 0])
        v_gpu.append(float(torch.sqrt((vz.double() ** 2).mean())))
        xn, yn, zn, vxn, vyn, vzn = np_catalog(100 + seed, n, L, Np)
        r = g.power_f32(xn, yn, zn, L ** 3, (0, 0, 1), dK)
        p_np.append(r["P"][:, 0])
        v_np.append(float(np.sqrt((vzn ** 2).mean())))
        K = r["K"]
    sel = (K > 0.03) & (K < 0.15)
    ratio = np.mean(p_gpu, axis=0)[sel] / np.mean(p_np, axis=0)[sel]
    assert np.all(np.abs(ratio - 1) < 0.2), ratio
    assert abs(np.mean(v_gpu) / np.mean(v_np) - 1) < 0.1


def test_device_catalog_ordered_after_torch_stream(fg):
    """A catalog written by torch kernels and measured through device pointers
    on a grid bound to torch's current stream (handle 0, the legacy default
    stream), with no synchronisation in between, gives the host-path result."""
    import torch
    from fftgal_gb300 import mocks
    n, L, Np = 64, 1000.0, 4e5
    dK = 2 * np.pi / L
    g = fg.Grid(n, L, precision="f32", host_view="lazy")
    g.set_stream(torch.cuda.current_stream().cuda_stream)
    for seed in (11, 12):
        x, y, z, vx, vy, vz = mocks.lognormal_catalog(n, L, Np, seed, axes=(2,))
        zr = (z + vz).contiguous()
        rd = g.power_f32(x.data_ptr(), y.data_ptr(), zr.data_ptr(), L ** 3, (0, 0, 1), dK, Nmu=3,
                         where=fg.MEM_DEVICE, Np=int(x.numel()))
        rh = g.power_f32(x.cpu().numpy(), y.cpu().numpy(), zr.cpu().numpy(), L ** 3, (0, 0, 1), dK, Nmu=3)
        ok = rh["N"] > 0
        # errors in units of |P_0| + Pshot: the bin sums' atomic order varies
        # between runs, and P_6 near a zero crossing cancels terms ~1e4 larger
        den = np.abs(rh["P"][ok][:, :1]) + L ** 3 / x.numel()
        assert (np.abs(rd["P"][ok] - rh["P"][ok]) / den).max() <= 1e-6
