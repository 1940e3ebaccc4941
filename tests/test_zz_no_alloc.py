"""fftgal_power_bins_noalloc (allocation-free binning of a k-space grid in GPU
memory) against fftgal_power_f32's own binning of the same grid, through the
C ABI.  Named to be collected last, so it runs both alone and after the rest.

Tolerances: mode counts bit-exact; mean K per bin 1e-12 relative; P_l and
wedges within 1e-5 of (|P_0(k)| + Pshot) -- both sides sum FP32 powers into
FP64 per block, in different orders.
"""
import numpy as np
import pytest

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


@pytest.mark.parametrize("Ng,L,n,los,dKf,Nmu", [(64, 500.0, 60_000, (0.0, 1.0, 1.0), 1.0, 3),
                                               (48, 300.0, 30_000, (0.0, 0.0, 1.0), 1.5, 10)])
def test_noalloc_matches_power_f32(fg, Ng, L, n, los, dKf, Nmu):
    x, y, z = uniform_box(11, n, L)
    dK = dKf * 2 * np.pi / L
    g = fg.Grid(Ng, L, precision="f32", host_view="lazy")
    want = g.power_f32(x, y, z, L ** 3, los, dK, Nmu=Nmu)
    fk = fg.lib().fftgal_device_grid(g.p)
    Pshot = L ** 3 / n
    # two calls in a row: the second must not see the first one's sums
    for _ in range(2):
        got = fg.power_bins_noalloc(fk, Ng, L, L ** 3, n, los, dK, Nmu=Nmu)
        _close(got, want, Pshot)


def test_noalloc_limits(fg):
    g = fg.Grid(16, 100.0, precision="f32", host_view="lazy")
    fk = fg.lib().fftgal_device_grid(g.p)
    with pytest.raises(fg.FftgalError, match="Nmu"):
        fg.power_bins_noalloc(fk, 16, 100.0, 1e6, 10, (0, 0, 1), 0.1, Nmu=17)
    with pytest.raises(fg.FftgalError, match="fixed scratch"):
        fg.power_bins_noalloc(fk, 16, 100.0, 1e6, 10, (0, 0, 1), 2 * np.pi / 100.0 / 300, Nmu=3)
