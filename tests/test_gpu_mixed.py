"""fftgal_power_mixed_f32: catalogs of mixed grid sizes (powers of two and
not), fold factors (box L / fold, src/app/P.c:35-36), bin widths and uneven
particle counts in one call.  Every catalog's tables equal fftgal_power_f32's
on a grid of its own up to the order in which the binning adds its sums (the
FP32 shared-memory run sums and the FP64 global sums are atomic: 1e-6 of
|P_0| + Pshot; mode counts exact), a subset matches the FP64 oracle under the
parity criterion, and a second call reuses the kept grids."""
import numpy as np
import pytest

import parity
from catalogs import clustered_box, uniform_box

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fg():
    from fftgal_gb300 import build
    build.build()
    import fftgal_gb300
    return fftgal_gb300


def _list():
    rng = np.random.default_rng(3)
    L0 = 300.0
    cats, Ng, L, dK = [], [], [], []
    for q, (ng, fold) in enumerate([(32, 1), (48, 2), (64, 4), (32, 2), (48, 1), (64, 1), (32, 4), (48, 4)]):
        n = int(10 ** rng.uniform(4.3, 5.3))
        if q % 2:
            p = clustered_box(40 + q, n, L0, max(50, n // 40), 1.5)
        else:
            p = uniform_box(40 + q, n, L0)
        cats.append(tuple(np.asarray(a, dtype=np.float32) for a in p))
        Ng.append(ng)
        L.append(L0 / fold)
        dK.append((1.0 + 0.5 * (q % 3)) * 2 * np.pi / (L0 / fold))
    return cats, Ng, L, dK, L0 ** 3


def _close(got, want, Pshot, rel):
    np.testing.assert_array_equal(got["N"], want["N"])
    np.testing.assert_array_equal(got["Nmu"], want["Nmu"])
    P0 = want["P"][:, :1]
    den = np.where(np.isfinite(P0), np.abs(P0), 0.0) + Pshot  # empty bins are NaN
    ok = np.isfinite(want["P"])
    assert np.array_equal(ok, np.isfinite(got["P"]))
    assert (np.abs(got["P"] - want["P"]) / den)[ok].max() <= rel
    okm = np.isfinite(want["Pmu"])
    assert (np.abs(got["Pmu"] - want["Pmu"]) / den)[okm].max() <= rel


def test_mixed_matches_single_calls(fg, oracle_lib):
    cats, Ng, L, dK, V = _list()
    los, Nmu = (0.0, 0.3, 1.0), 4
    res = fg.power_mixed_f32(cats, V, Ng, L, los, dK, Nmu=Nmu)
    assert len(res) == len(cats)
    for c, (x, y, z) in enumerate(cats):
        g = fg.Grid(Ng[c], L[c], precision="f32", host_view="lazy")
        want = g.power_f32(x, y, z, V, los, dK[c], Nmu=Nmu)
        _close(res[c], want, V / len(x), 1e-6)
    for c in (0, 1, 6):  # a power of two and not, folds 1, 2 and 4
        x, y, z = (a.astype(np.float64) for a in cats[c])
        want = oracle_lib.power_spectrum(Ng[c], L[c], x, y, z, los, dK[c], Nmu=Nmu, V=V)
        e = parity.errors(res[c], want, V / len(x), Ng[c], L[c])
        assert parity.passes(e), (c, e)
    again = fg.power_mixed_f32(cats[::-1], V, Ng[::-1], L[::-1], los, dK[::-1], Nmu=Nmu)
    for c in range(len(cats)):
        _close(again[len(cats) - 1 - c], res[c], V / len(cats[c][0]), 1e-6)
    fg.power_mixed_release()


def test_mixed_rejects_bad_catalogs(fg):
    cats, Ng, L, dK, V = _list()
    Ng[2] = 1
    with pytest.raises(fg.FftgalError, match="catalog 2"):
        fg.power_mixed_f32(cats, V, Ng, L, (0, 0, 1), dK)
