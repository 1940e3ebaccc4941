"""Write the golden fixtures under tests/golden/ from the reference's OWN code.

Run in a checkout where the reference sources are present
(oracle.reference_dir(): FFTGAL_REFERENCE_DIR, or the checkout oracle/Makefile
builds from):

    make -C oracle ref && python tests/golden/make_golden.py

It drives oracle/_ref/librefgal.so -- src/fft.c, src/gal.c and src/power.c
compiled unmodified against the shim FFTW/GSL headers (the FFT backend is the
project's FP64 FFT, oracle/fft64.c, cross-checked against numpy.fft) -- and
stores its outputs:

  small_cases.npz    Ng in {2,3,4,5,6,8,12,16}: fft_p2g (offset 1/2, with and
                     without randoms), fft_x2k(phase on), fft_p2k, P, and the
                     Pl/Pmu tables for several lines of sight and bin widths.
  uniform_ng128.npz  the uniform-box configuration: 1e6 particles uniform in
                     [0,1000)^3 (splitmix64 seed 1, FP64), Ng=128, interlaced,
                     dK=2pi/L: the Pl and Pmu tables for 4 lines of sight.
  gal_rsd_wrap.npz   gal_rsd for 4 lines of sight (one not normalised) x 2
                     values of aH, and gal_wrap, on 400 particles spread over
                     three box lengths with Gaussian velocities.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

from oracle.reflib import RefGal, RefGrid, RefLib, available, run_pl_pmu  # noqa: E402
from catalogs import uniform_box  # noqa: E402

LOS_SET = [(0, 0, 1), (0, 1, 1), (1, 1, 0), (1, 1, 1), (0, 0, 0), (0.3, -0.2, 0.9)]


def small_cases():
    out = {}
    lib = RefLib.lib()
    for Ng in (2, 3, 4, 5, 6, 8, 12, 16):
        L = 50.0 + Ng
        n = 7 * Ng
        x, y, z = uniform_box(100 + Ng, n, 1.6 * L, lo=-0.3 * L)
        xr, yr, zr = uniform_box(200 + Ng, 3 * n, L)
        V = L ** 3
        key = f"ng{Ng}"
        out[key + "_L"] = L
        out[key + "_pos"] = np.stack([x, y, z])
        out[key + "_rand"] = np.stack([xr, yr, zr])
        # fft_p2g with an offset that remainder() must reduce
        g = RefGrid(Ng, L)
        gal = RefGal(x, y, z, V)
        off = np.array([0.5 + 3 * Ng, -1.5, 0.25])
        lib.fft_p2g(g.p, gal.p, off.ctypes.data_as(lib.fft_p2g.argtypes[2]))
        out[key + "_p2g_offset_in"] = np.array([0.5 + 3 * Ng, -1.5, 0.25])
        out[key + "_p2g_offset_out"] = off.copy()
        out[key + "_p2g"] = g.f.copy()
        lib.fft_x2k(g.p, 1)
        out[key + "_x2k_phase"] = g.f.copy()
        lib.fft_k2x(g.p, 1)
        out[key + "_k2x_phase"] = g.f.copy()
        # with randoms (alpha-weighted subtraction, src/fft.c:94-124)
        galr = RefGal(x, y, z, V, rand=(xr, yr, zr))
        off = np.array([0.0, 0.0, 0.0])
        lib.fft_p2g(g.p, galr.p, off.ctypes.data_as(lib.fft_p2g.argtypes[2]))
        out[key + "_p2g_rand"] = g.f.copy()
        # interlaced p2k, then P, then Pl/Pmu for several los and dK
        lib.fft_p2k(g.p, gal.p)
        out[key + "_p2k"] = g.f.copy()
        lib.P(g.p, gal.p)
        out[key + "_P"] = g.f.copy()
        KF = 2 * np.pi / L
        for il, los in enumerate(LOS_SET):
            for idk, dK in enumerate((KF, 0.7 * KF, 2.5 * KF)):
                tpl, tmu = run_pl_pmu(g, gal, los, dK)
                out[f"{key}_los{il}_dk{idk}_pl"] = np.array(tpl)
                out[f"{key}_los{il}_dk{idk}_pmu"] = np.array(tmu)
    out["los_set"] = np.array(LOS_SET, dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, "small_cases.npz"), **out)


def uniform_ng128():
    lib = RefLib.lib()
    L, Ng, n = 1000.0, 128, 1_000_000
    x, y, z = uniform_box(1, n, L)
    g = RefGrid(Ng, L)
    gal = RefGal(x, y, z, L ** 3)
    lib.fft_p2k(g.p, gal.p)
    fk = g.f.copy()
    out = {"L": L, "Ng": Ng, "Np": n, "seed": 1}
    out["fk_checksum"] = np.array([fk.sum(), np.abs(fk).sum(), (fk * fk).sum()])
    dK = 2 * np.pi / L
    for il, los in enumerate([(0, 0, 1), (0, 1, 1), (1, 1, 1), (1, 0, 0)]):
        g.f[:] = fk
        lib.P(g.p, gal.p)
        tpl, tmu = run_pl_pmu(g, gal, los, dK)
        out[f"los{il}"] = np.array(los, dtype=np.float64)
        out[f"los{il}_pl"] = np.array(tpl)
        out[f"los{il}_pmu"] = np.array(tmu)
    np.savez_compressed(os.path.join(HERE, "uniform_ng128.npz"), **out)


def gal_rsd_wrap():
    import ctypes as C
    lib = RefLib.lib()
    L, n = 100.0, 400
    x, y, z = uniform_box(7, n, 3 * L, lo=-L)
    rng = np.random.default_rng(7)  # velocities: any reproducible values do
    vx, vy, vz = (rng.standard_normal(n) * 40.0 for _ in range(3))
    out = {"L": L, "pos": np.stack([x, y, z]), "vel": np.stack([vx, vy, vz])}
    dp = C.POINTER(C.c_double)
    los_set = [(0.0, 0.0, 1.0), (1.0, 1.0, 0.0), (0.3, -0.2, 0.9), (2.0, 0.0, 0.0)]
    out["los_set"] = np.array(los_set)
    out["aH_set"] = np.array([1.0, 0.7])
    for il, los in enumerate(los_set):
        for ia, aH in enumerate((1.0, 0.7)):
            gal = RefGal(x, y, z, L ** 3, vel=(vx, vy, vz))
            l = np.array(los, dtype=np.float64)  # gal_rsd normalises it in place
            d = lib.gal_rsd(gal.p, l.ctypes.data_as(dp), aH)
            g = d.contents
            out[f"rsd_los{il}_ah{ia}"] = np.stack([np.ctypeslib.as_array(getattr(g, a), shape=(n,)).copy()
                                                   for a in ("x", "y", "z")])
            lib.gal_free(d)
    gal = RefGal(x, y, z, L ** 3)
    lib.gal_wrap(gal.p, L)
    g = gal.p.contents
    out["wrap"] = np.stack([np.ctypeslib.as_array(getattr(g, a), shape=(n,)).copy() for a in ("x", "y", "z")])
    np.savez_compressed(os.path.join(HERE, "gal_rsd_wrap.npz"), **out)


if __name__ == "__main__":
    if not available():
        sys.exit("reference build missing: run `make -C oracle ref` first")
    small_cases()
    uniform_ng128()
    gal_rsd_wrap()
    print("golden fixtures written to", HERE)
