"""Clustered catalogs (lognormal field, Zel'dovich velocities, z-RSD) through
the fused FP32 call, against the FP64 oracle: folds 1 and 4 (the reference's
P.c paints on a box of L/fold and lets the cell index wrap, src/app/P.c:35-66),
Nmu = 10 wedges.  Strong clustering drives the paint's per-block fixed-point
bound below its maximum, which uniform catalogs never reach.

The redshift-space displacement is applied either by the oracle's gal_rsd
before painting or, through fftgal_power_rsd_f32, inside the paint itself.

Tolerances: mode counts bit-exact; mean K 1e-12; P_0,2,4 and every wedge within
1e-4 of (|P_0(k)| + Pshot) for k < 0.8 k_Nyq, every bin within 1e-3.
"""
import numpy as np
import pytest

from lognormal import lognormal_catalog

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fg():
    from fftgal_gb300 import build
    build.build()
    import fftgal_gb300
    return fftgal_gb300


def _f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


@pytest.fixture(scope="module")
def real_space():
    L = 1000.0
    return L, [_f32(a) for a in lognormal_catalog(7, 128, L, 1e6)]


@pytest.fixture(scope="module")
def catalog(oracle_lib, real_space):
    L, (x, y, z, vx, vy, vz) = real_space
    # redshift space along z through the oracle's gal_rsd (aH = 1)
    xs, ys, zs = oracle_lib.Oracle.rsd(x, y, z, vx, vy, vz, (0.0, 0.0, 1.0), 1.0)
    # both sides see the same FP32 positions
    return L, [_f32(a) for a in (xs, ys, zs)]


def _check(got, want, Pshot, kmax):
    np.testing.assert_array_equal(got["N"], want["N"])
    np.testing.assert_array_equal(got["Nmu"], want["Nmu"])
    np.testing.assert_allclose(got["K"], want["K"], rtol=1e-12)
    P0 = want["P"][:, :1]
    den = np.where(np.isfinite(P0), np.abs(P0), 0.0) + Pshot
    sel = want["K"] < kmax
    for key, cols in (("P", slice(0, 3)), ("Pmu", slice(None))):
        g, w = got[key][:, cols], want[key][:, cols]
        ok = np.isfinite(w)
        assert np.array_equal(ok, np.isfinite(g)), key
        err = np.abs(g - w) / np.broadcast_to(den, w.shape)
        err_lo = err[sel][ok[sel]]
        assert err_lo.max() <= 1e-4, f"{key}: {err_lo.max():.2e} for k < 0.8 k_Nyq"
        assert err[ok].max() <= 1e-3, f"{key}: {err[ok].max():.2e} over all bins"


@pytest.mark.parametrize("fold", [1, 4])
def test_lognormal_rsd_folded(fg, oracle_lib, catalog, fold):
    L, (x, y, z) = catalog
    Ng, Lfd, Nmu = 128, L / fold, 10
    los, dK, V = (0.0, 0.0, 1.0), 2 * np.pi / Lfd, L ** 3
    g = fg.Grid(Ng, Lfd, precision="f32", host_view="lazy")
    got = g.power_f32(x, y, z, V, los, dK, Nmu=Nmu)
    want = oracle_lib.power_spectrum(Ng, Lfd, x, y, z, los, dK, Nmu=Nmu, V=V)
    assert want["status"] == (0, 0)
    _check(got, want, V / len(x), 0.8 * np.pi * Ng / Lfd)


@pytest.mark.parametrize("los,aH", [((0.0, 0.0, 1.0), 1.0), ((1.0, 1.0, 0.0), 0.7)])
def test_rsd_fused_into_paint(fg, oracle_lib, real_space, los, aH):
    """fftgal_power_rsd_f32 (displacement inside the paint, FP32) against the
    oracle's gal_rsd (FP64, src/gal.c:63-77) followed by the P.c sequence;
    the displaced positions differ only by FP32 rounding (~1e-4 of a cell)."""
    L, (x, y, z, vx, vy, vz) = real_space
    Ng, fold, Nmu = 128, 2, 10
    Lfd = L / fold
    dK, V = 2 * np.pi / Lfd, L ** 3
    g = fg.Grid(Ng, Lfd, precision="f32", host_view="lazy")
    got = g.power_rsd_f32(x, y, z, vx, vy, vz, V, los, aH, dK, Nmu=Nmu)
    xs, ys, zs = oracle_lib.Oracle.rsd(x, y, z, vx, vy, vz, los, aH)
    want = oracle_lib.power_spectrum(Ng, Lfd, xs, ys, zs, los, dK, Nmu=Nmu, V=V)
    _check(got, want, V / len(x), 0.8 * np.pi * Ng / Lfd)


@pytest.mark.parametrize("fold", [1, 4])
def test_single_paint_against_oracle(fg, oracle_lib, catalog, fold):
    """fftgal_power_single_f32 (no interlacing) against the oracle's
    fft_p2g -> fft_x2k -> fft_deconv -> P -> Pl -> Pmu on the clustered catalog."""
    L, (x, y, z) = catalog
    Ng, Lfd, Nmu = 128, L / fold, 10
    los, dK, V = (0.0, 0.0, 1.0), 2 * np.pi / Lfd, L ** 3
    g = fg.Grid(Ng, Lfd, precision="f32", host_view="lazy")
    got = g.power_f32(x, y, z, V, los, dK, Nmu=Nmu, interlace=False)
    want = oracle_lib.power_spectrum(Ng, Lfd, x, y, z, los, dK, Nmu=Nmu, V=V, interlace=False)
    assert want["status"] == (0, 0)
    _check(got, want, V / len(x), 0.8 * np.pi * Ng / Lfd)


def test_single_paint_lazy_and_sync_views_agree(fg):
    """The lazy host view bins the single paint's deconvolved field without
    storing it, the sync view stores it first: the same multipoles."""
    from catalogs import uniform_box
    Ng, L = 64, 500.0
    x, y, z = uniform_box(77, 150_000, L)
    dK = 2 * np.pi / L
    out = []
    for view in ("lazy", "sync"):
        g = fg.Grid(Ng, L, precision="f32", host_view=view)
        out.append(g.power_f32(x, y, z, L ** 3, (0, 0, 1), dK, Nmu=3, interlace=False))
    np.testing.assert_array_equal(out[0]["N"], out[1]["N"])
    den = np.abs(np.nan_to_num(out[1]["P"][:, :1])) + L ** 3 / len(x)
    ok = np.isfinite(out[1]["P"])
    assert (np.abs(out[0]["P"] - out[1]["P"]) / den)[ok].max() <= 1e-6
