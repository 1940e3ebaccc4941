"""Write tests/golden/headline_ng1024.npz: the FP64 reference answer for the
benchmarked workload, from the reference's OWN code.

Run in a checkout where the reference sources are present (see
oracle.reference_dir()), on a host with about 30 GB of free memory:

    make -C oracle ref && python tests/golden/make_headline_golden.py

Two seeded 1e8-particle catalogs in a 1000 Mpc/h box, both generated from
splitmix64 integers with plain IEEE arithmetic (tests/golden/catalogs.py), so
the GPU tests and bench.py regenerate bit-identical FP32 positions on any
machine:

  uniform    uniform_box_f32(seed 20240, 1e8, 1000): the catalog bench.py times;
  clustered  a Neyman-Scott process (1e6 centres, sigma = 2 Mpc/h, seed 20250),
             whose low-k power is ~100x the shot noise.

For each, the FP32 positions (widened exactly to FP64) go through the
reference's fft_init(1024, 1000) -> fft_p2k -> P -> Pl, Pmu
(src/app/P.c:55-66; oracle/_ref/librefgal.so, the reference's src/fft.c,
gal.c, power.c compiled unmodified against the shim FFTW whose FFT is the
project's FP64 FFT) for three lines of sight, dK = 2 pi / L.  Stored per
catalog and line of sight: the reference's Pl / Pmu text tables (7 digits),
and the full-precision arrays of the oracle (oracle/fftgal_oracle.c) binning
the same reference k-space grid, with 3 and with 10 mu wedges; the script
checks that both agree to the printed digits.  The wall times of the
reference's stages on this host are stored as well (single core).
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

from oracle import Oracle  # noqa: E402
from oracle.reflib import RefGal, RefGrid, RefLib, available, read_table, run_pl_pmu  # noqa: E402
from catalogs import clustered_box, uniform_box_f32  # noqa: E402

NG, L, NP = 1024, 1000.0, 100_000_000
LOS_SET = [(0.0, 0.0, 1.0), (1.0, 1.0, 0.0), (1.0, 1.0, 1.0)]
CATALOGS = {
    "uniform": dict(seed=20240),
    "clustered": dict(seed=20250, nclusters=1_000_000, sigma=2.0),
}


def catalog(name: str):
    """The FP32 positions of catalog `name` (three float32 arrays)."""
    c = CATALOGS[name]
    if name == "uniform":
        return uniform_box_f32(c["seed"], NP, L)
    x, y, z = clustered_box(c["seed"], NP, L, c["nclusters"], c["sigma"])
    return tuple(np.ascontiguousarray(a, dtype=np.float32) for a in (x, y, z))


def run(name: str, out: dict):
    lib = RefLib.lib()
    p32 = catalog(name)
    t = {}
    g = RefGrid(NG, L)
    gal = RefGal(*(a.astype(np.float64) for a in p32), L ** 3)
    del p32
    t0 = time.perf_counter()
    lib.fft_p2k(g.p, gal.p)
    t["p2k"] = time.perf_counter() - t0
    og = Oracle(NG, L)
    og.f[:] = g.f
    t0 = time.perf_counter()
    lib.P(g.p, gal.p)
    t["P"] = time.perf_counter() - t0
    og.power(NP, L ** 3)
    dK = 2 * np.pi / L
    for il, los in enumerate(LOS_SET):
        t0 = time.perf_counter()
        tpl, tmu = run_pl_pmu(g, gal, los, dK)
        t[f"Pl_Pmu_los{il}"] = time.perf_counter() - t0
        key = f"{name}_los{il}"
        out[key + "_pl_text"] = np.array(tpl)
        out[key + "_pmu_text"] = np.array(tmu)
        K, N, P, st, _ = og.pl(los, dK)
        assert st == 0
        out[key + "_K"], out[key + "_N"], out[key + "_P"] = K, N, P
        for nmu in (3, 10):
            Km, Nm, Pm, st, _ = og.pmu(los, dK, nmu)
            assert st == 0
            out[f"{key}_mu{nmu}_K"], out[f"{key}_mu{nmu}_N"], out[f"{key}_mu{nmu}_P"] = Km, Nm, Pm
        # the oracle's binning of the reference grid against the reference's printed tables
        _check_text(tpl, K, N, P, tmu, out[f"{key}_mu3_K"], out[f"{key}_mu3_N"], out[f"{key}_mu3_P"])
    out[name + "_seconds"] = np.array([t["p2k"], t["P"]] + [t[f"Pl_Pmu_los{i}"] for i in range(len(LOS_SET))])
    print(name, {k: round(v, 1) for k, v in t.items()}, flush=True)


def _write(path: str, text: str) -> str:
    with open(path, "w") as fh:
        fh.write(text)
    return path


def _check_text(tpl, K, N, P, tmu, Km, Nm, Pm):
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        a = read_table(_write(os.path.join(d, "pl"), tpl))
        b = read_table(_write(os.path.join(d, "pmu"), tmu))
    assert np.array_equal(a[:, 1].astype(np.int64), N)
    np.testing.assert_allclose(a[:, 0], K, rtol=1e-6)
    ok = np.isfinite(a[:, 2:])
    np.testing.assert_allclose(a[:, 2:][ok], P[ok], rtol=1e-6, atol=1e-12)
    for m in range(3):
        assert np.array_equal(b[:, 3 * m + 1].astype(np.int64), Nm[:, m])
        fin = np.isfinite(b[:, 3 * m + 2])
        np.testing.assert_allclose(b[fin, 3 * m + 2], Pm[fin, m], rtol=1e-6, atol=1e-12)


if __name__ == "__main__":
    if not available():
        sys.exit("reference build missing: run `make -C oracle ref` first")
    out = {"Ng": NG, "L": L, "Np": NP, "los_set": np.array(LOS_SET), "dK": 2 * np.pi / L,
           "host": os.uname().machine}
    for name, c in CATALOGS.items():
        for k, v in c.items():
            out[f"{name}_{k}"] = v
    for name in CATALOGS:
        run(name, out)
    np.savez_compressed(os.path.join(HERE, "headline_ng1024.npz"), **out)
    print("written", os.path.join(HERE, "headline_ng1024.npz"))
