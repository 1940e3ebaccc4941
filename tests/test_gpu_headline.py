"""Parity at the benchmarked sizes, against FP64 answers on the same FP32
positions.

* Ng = 1024, Np = 1e8 (the benchmark workload): a uniform and a clustered
  catalog, regenerated bit for bit from their splitmix64 seeds
  (tests/golden/catalogs.py), through fftgal_power_f32 and through the drop-in
  sequence fft_p2k -> P -> Pl -> Pmu (src/app/P.c:55-66), against
  tests/golden/headline_ng1024.npz: the reference's own fft_p2k / P / Pl / Pmu
  (src/fft.c:257-276, src/power.c:12-178) run in FP64 on those positions
  (tests/golden/make_headline_golden.py), 3 lines of sight, 3 and 10 wedges.
* The lognormal redshift-space configuration at full size: Ng = 512, about
  1e7 galaxies, folds 1 and 4 (src/app/P.c:35-36), 10 wedges, against the FP64
  oracle run on this host.
* A deep fold: Ng = 128 on a box folded 256 times, so x Ng / L_fold reaches
  32768 (the scale of Ng = 2048 with fold 16), against the FP64 oracle.

Criterion (tests/golden/parity.py): mode counts bit-exact, P_0,2,4 and every
wedge within 1e-4 of |P_0| + Pshot for k < 0.8 k_Nyq, every bin within 1e-3.
"""
import os

import numpy as np
import pytest

import parity
from catalogs import clustered_box, uniform_box_f32

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "headline_ng1024.npz")


@pytest.fixture(scope="module")
def fg():
    from fftgal_gb300 import build
    build.build()
    import fftgal_gb300
    return fftgal_gb300


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def _catalog(z, name):
    Np, L = int(z["Np"]), float(z["L"])
    if name == "uniform":
        p = uniform_box_f32(int(z["uniform_seed"]), Np, L)
    else:
        p = clustered_box(int(z["clustered_seed"]), Np, L, int(z["clustered_nclusters"]),
                          float(z["clustered_sigma"]))
    return tuple(np.ascontiguousarray(a, dtype=np.float32) for a in p)


@pytest.fixture(scope="module")
def grid1024(fg):
    return fg.Grid(1024, 1000.0, precision="f32", host_view="lazy")


def _assert_parity(got, want, Pshot, Ng, L, what):
    e = parity.errors(got, want, Pshot, Ng, L)
    assert parity.passes(e), f"{what}: {e}"
    return e


@pytest.mark.parametrize("name", ["uniform", "clustered"])
def test_headline_fused_call(fg, golden, grid1024, name):
    x, y, z = _catalog(golden, name)
    Ng, L = int(golden["Ng"]), float(golden["L"])
    V, dK, Pshot = L ** 3, float(golden["dK"]), L ** 3 / len(x)
    for il, los in enumerate(golden["los_set"]):
        for nmu in (3, 10):
            got = grid1024.power_f32(x, y, z, V, los, dK, Nmu=nmu)
            e = _assert_parity(got, parity.golden_result(golden, name, il, nmu), Pshot, Ng, L,
                               f"{name} los{il} Nmu={nmu}")
            print(f"{name} los{il} Nmu={nmu}: {e}")


def test_headline_dropin_sequence(fg, golden):
    """The P.c call sequence on an FP32 grid (fft_p2k, P, Pl, Pmu with the
    reference's text output; the k-space grid is painted again per line of
    sight instead of restored from an 8.6 GB fft_exportf snapshot), against
    the reference's own text tables."""
    import tempfile
    name = "clustered"
    x, y, z = _catalog(golden, name)
    Ng, L = int(golden["Ng"]), float(golden["L"])
    dK, Pshot = float(golden["dK"]), L ** 3 / len(x)
    cat = fg.Catalog(x, y, z, L ** 3)
    del x, y, z
    g = fg.Grid(Ng, L, precision="f32", host_view="lazy")
    with tempfile.TemporaryDirectory() as d:
        fpl, fmu = os.path.join(d, "pl.txt"), os.path.join(d, "pmu.txt")
        for il, los in enumerate(golden["los_set"]):
            g.p2k(cat)
            g.power(cat)
            g.pl(cat, np.array(los), dK, fpl)
            g.pmu(cat, np.array(los), dK, fmu)
            tpl, tmu = fg.read_table(fpl), fg.read_table(fmu)
            ref_pl = _table(golden[f"{name}_los{il}_pl_text"])
            ref_mu = _table(golden[f"{name}_los{il}_pmu_text"])
            got = dict(K=tpl[:, 0], N=tpl[:, 1].astype(np.int64), P=tpl[:, 2:6],
                       Kmu=tmu[:, 0::3], Nmu=tmu[:, 1::3].astype(np.int64), Pmu=tmu[:, 2::3])
            want = dict(K=ref_pl[:, 0], N=ref_pl[:, 1].astype(np.int64), P=ref_pl[:, 2:6],
                        Kmu=ref_mu[:, 0::3], Nmu=ref_mu[:, 1::3].astype(np.int64), Pmu=ref_mu[:, 2::3])
            _assert_parity(got, want, Pshot, Ng, L, f"drop-in los{il}")


def _table(text) -> np.ndarray:
    rows = [[float(t) for t in ln.split()] for ln in str(text).splitlines() if ln and not ln.startswith("#")]
    return np.array(rows)


@pytest.fixture(scope="module")
def lognormal_512(fg):
    """About 1e7 galaxies of the lognormal configuration (GPU generator, seed
    11): Poisson sampled on a 512^3 lognormal field, displaced by the
    Zel'dovich displacement, then shifted along z by f Psi_z (f = 0.8); FP32."""
    import torch
    from fftgal_gb300 import mocks
    f = 0.8
    x, y, z, vx, vy, vz = mocks.lognormal_catalog(512, 1000.0, 1e7, seed=11, f=f)
    # v = f Psi: real-space positions x + Psi, redshift space adds f Psi_z along z
    xs = (x + vx / f).cpu().numpy()
    ys = (y + vy / f).cpu().numpy()
    zs = (z + vz / f + vz).cpu().numpy()
    del x, y, z, vx, vy, vz
    torch.cuda.empty_cache()
    return tuple(np.ascontiguousarray(a, dtype=np.float32) for a in (xs, ys, zs))


@pytest.mark.parametrize("fold", [1, 4])
def test_lognormal_config_full_size(fg, oracle_lib, lognormal_512, fold):
    x, y, z = lognormal_512
    L, Ng, Nmu = 1000.0, 512, 10
    Lfd = L / fold
    los, dK, V = (0.0, 0.0, 1.0), 2 * np.pi / Lfd, L ** 3
    g = fg.Grid(Ng, Lfd, precision="f32", host_view="lazy")
    got = g.power_f32(x, y, z, V, los, dK, Nmu=Nmu)
    want = oracle_lib.power_spectrum(Ng, Lfd, x.astype(np.float64), y.astype(np.float64),
                                     z.astype(np.float64), los, dK, Nmu=Nmu, V=V)
    assert want["status"] == (0, 0)
    e = _assert_parity(got, want, V / len(x), Ng, Lfd, f"lognormal fold {fold}")
    print(f"fold {fold}, Np {len(x)}: {e}")


def test_deep_fold(fg, oracle_lib):
    """Fold 256 at Ng = 128: cell coordinates x Ng / L_fold up to 32768,
    where one FP32 unit in the last place of a position is about 1/500 of a
    cell; the clusters
    (sigma = 0.01 Mpc/h, a third of a folded cell) give the folded field
    power well above the shot noise at every k."""
    L, Ng, fold, Nmu = 1000.0, 128, 256, 3
    Lfd = L / fold
    x, y, z = (np.asarray(a, dtype=np.float32) for a in clustered_box(31, 1_000_000, L, 20_000, 0.01))
    assert float(x.max()) * Ng / Lfd > 32000
    los, dK, V = (1.0, 1.0, 1.0), 2 * np.pi / Lfd, L ** 3
    g = fg.Grid(Ng, Lfd, precision="f32", host_view="lazy")
    got = g.power_f32(x, y, z, V, los, dK, Nmu=Nmu)
    want = oracle_lib.power_spectrum(Ng, Lfd, x.astype(np.float64), y.astype(np.float64),
                                     z.astype(np.float64), los, dK, Nmu=Nmu, V=V)
    e = _assert_parity(got, want, V / len(x), Ng, Lfd, "fold 256")
    print(f"fold 256: {e}")
