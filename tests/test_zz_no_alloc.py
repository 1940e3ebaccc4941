"""fftgal_power_bins_noalloc (allocation-free binning of a k-space grid in GPU
memory, for callers whose framework owns all device memory) through the C
ABI: against fftgal_power_f32's own binning of the same grid on two calls in
a row, against the FP64 oracle, at the documented limits, and without any
change of the device's free memory after the first call.  Named to be
collected last, so it runs both alone and after the rest.

Tolerances: mode counts bit-exact; mean K per bin 1e-12 relative; P_l and
wedges within 1e-5 of (|P_0(k)| + Pshot) of power_f32 -- both sides sum FP32
powers into FP64 per block, in different orders; against the oracle the
parity criterion of the FP32 path (tests/golden/parity.py).
"""
import numpy as np
import pytest

import parity
from catalogs import uniform_box

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fg():
    from fftgal_gb300 import build
    build.build()
    import fftgal_gb300
    return fftgal_gb300


def _close(got, want, Pshot):
    P0 = want["P"][:, :1]
    den = np.where(np.isfinite(P0), np.abs(P0), 0.0) + Pshot  # empty bins are NaN
    np.testing.assert_array_equal(got["N"], want["N"])
    np.testing.assert_array_equal(got["Nmu"], want["Nmu"])
    np.testing.assert_allclose(got["K"], want["K"], rtol=1e-12)
    np.testing.assert_allclose(got["Kmu"], want["Kmu"], rtol=1e-12)
    ok = np.isfinite(want["P"])
    assert np.array_equal(ok, np.isfinite(got["P"]))
    err = np.abs(got["P"] - want["P"])[ok] / np.broadcast_to(den, want["P"].shape)[ok]
    assert err.max() <= 1e-5, f"P_l error {err.max():.2e}"
    errw = np.abs(got["Pmu"] - want["Pmu"]) / np.broadcast_to(den, want["Pmu"].shape)
    assert errw.max() <= 1e-5, f"P_mu error {errw.max():.2e}"


def _kspace(fg, Ng, L, x, y, z):
    """An FP32 grid holding the deconvolved interlaced k-space field of the
    catalog (fft_p2k through the drop-in API) and its device pointer."""
    g = fg.Grid(Ng, L, precision="f32", host_view="lazy")
    cat = fg.Catalog(x, y, z, L ** 3)
    g.p2k(cat)
    g.synchronize()
    return g, fg.lib().fftgal_device_grid(g.p)


@pytest.mark.parametrize("Ng,L,n,los,dKf,Nmu", [(64, 500.0, 60_000, (0.0, 1.0, 1.0), 1.0, 3),
                                               (48, 300.0, 30_000, (0.0, 0.0, 1.0), 1.5, 10),
                                               (1024, 1000.0, 2_000_000, (0.0, 0.0, 1.0), 1.0, 10)])
def test_noalloc_matches_power_f32(fg, Ng, L, n, los, dKf, Nmu):
    """Two calls in a row give power_f32's tables: the second call must not
    see the first one's sums.  Ng = 1024 with 10 wedges (NK = 887) is inside
    the documented shared-memory bound."""
    x, y, z = uniform_box(11, n, L)
    dK = dKf * 2 * np.pi / L
    want = fg.Grid(Ng, L, precision="f32", host_view="lazy").power_f32(x, y, z, L ** 3, los, dK, Nmu=Nmu)
    g, fk = _kspace(fg, Ng, L, x, y, z)
    Pshot = L ** 3 / n
    for _ in range(2):
        got = fg.power_bins_noalloc(fk, Ng, L, L ** 3, n, los, dK, Nmu=Nmu)
        _close(got, want, Pshot)


def test_noalloc_matches_oracle(fg, oracle_lib):
    Ng, L, n, los, Nmu = 64, 400.0, 80_000, (1.0, 1.0, 0.0), 4
    x, y, z = uniform_box(12, n, L)
    x, y, z = (np.asarray(a, dtype=np.float32).astype(np.float64) for a in (x, y, z))
    dK = 2 * np.pi / L
    g, fk = _kspace(fg, Ng, L, x, y, z)
    got = fg.power_bins_noalloc(fk, Ng, L, L ** 3, n, los, dK, Nmu=Nmu)
    want = oracle_lib.power_spectrum(Ng, L, x, y, z, los, dK, Nmu=Nmu)
    e = parity.errors(got, want, L ** 3 / n, Ng, L)
    # k < 0.8 k_Nyq: the parity bound; the corner bins, where the window
    # deconvolution amplifies FP32 rounding and the 256-row FP32 chunk sums add
    # their own, within 2e-3 at this size
    assert parity.passes(e, tol_all=2e-3), e


def test_noalloc_allocates_nothing(fg):
    """After a first call on the device, later calls leave the device's free
    memory unchanged (no cudaMalloc, no library pool growth)."""
    import torch
    Ng, L, n = 128, 600.0, 200_000
    x, y, z = uniform_box(13, n, L)
    g, fk = _kspace(fg, Ng, L, x, y, z)
    args = (fk, Ng, L, L ** 3, n, (0.0, 0.0, 1.0), 2 * np.pi / L)
    first = fg.power_bins_noalloc(*args, Nmu=3)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for nmu in (3, 10, 16, 3):
        got = fg.power_bins_noalloc(*args, Nmu=nmu)
        assert torch.cuda.mem_get_info()[0] == free0
    # the same tables again, up to the order of the atomic additions
    _close(got, first, L ** 3 / n)


def test_noalloc_limits(fg):
    """The documented limits: NK <= 2048, Nmu <= 16, and
    NK * (36 + 16 Nmu) + 8 <= 225280 bytes of shared accumulators."""
    g = fg.Grid(16, 100.0, precision="f32", host_view="lazy")
    fk = fg.lib().fftgal_device_grid(g.p)
    with pytest.raises(fg.FftgalError, match="Nmu"):
        fg.power_bins_noalloc(fk, 16, 100.0, 1e6, 10, (0, 0, 1), 0.1, Nmu=17)
    with pytest.raises(fg.FftgalError, match="fixed scratch"):
        fg.power_bins_noalloc(fk, 16, 100.0, 1e6, 10, (0, 0, 1), 2 * np.pi / 100.0 / 300, Nmu=3)
    # Ng = 1024, dK = 2 pi / L: NK = 887 fits up to Nmu = 13 (887 * 244 + 8 bytes)
    # and not at Nmu = 16 (887 * 292 + 8 > 225280); rejected before any grid access
    KF = 2 * np.pi / 1000.0
    with pytest.raises(fg.FftgalError, match="shared"):
        fg.power_bins_noalloc(fk, 1024, 1000.0, 1e9, 10, (0, 0, 1), KF, Nmu=16)
    # Ng = 2048, dK = 2 pi / L: NK = 1774 fits for Nmu <= 5 and not at Nmu = 10
    with pytest.raises(fg.FftgalError, match="shared"):
        fg.power_bins_noalloc(fk, 2048, 1000.0, 1e9, 10, (0, 0, 1), KF, Nmu=10)


def test_noalloc_ng2048_geometry(fg):
    """NK = 1774 (Ng = 2048, dK = 2 pi / L, 3 wedges) runs on a real 34 GB
    grid of zeros: every mode's power is -Pshot, the mode counts add up to
    Ng^3 - 1 (checked inside the call) and match the wedge counts."""
    import torch
    Ng, L, V, Np = 2048, 1000.0, 1e9, 10 ** 8
    free = torch.cuda.mem_get_info()[0]
    nbytes = Ng * Ng * (Ng + 2) * 4
    if free < nbytes + (4 << 30):
        pytest.skip(f"needs {nbytes / 2 ** 30:.0f} GiB of free device memory")
    fk = torch.zeros(Ng * Ng * (Ng + 2), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    got = fg.power_bins_noalloc(fk.data_ptr(), Ng, L, V, Np, (0.0, 0.0, 1.0), 2 * np.pi / L, Nmu=3)
    del fk
    torch.cuda.empty_cache()
    assert len(got["N"]) == 1774
    assert int(got["N"].sum()) == Ng ** 3 - 1
    np.testing.assert_array_equal(got["Nmu"].sum(axis=1), got["N"])
    Pshot = V / Np
    full = got["N"] > 0  # bin 0 holds no mode at dK = 2 pi / L: NaN, as the reference prints it
    assert not full[0] and full[1:].all() and np.isnan(got["P"][0]).all()
    np.testing.assert_allclose(got["P"][full, 0], -Pshot, rtol=1e-5)
    filled = got["Nmu"] > 0
    np.testing.assert_allclose(got["Pmu"][filled], -Pshot, rtol=1e-5)
    assert np.all(np.isfinite(got["P"][full]))
