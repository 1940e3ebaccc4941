"""ctypes binding of the reference's own C code, compiled unmodified from its
sources by ``make -C oracle ref`` into oracle/_ref/librefgal.so (TEST
INFRASTRUCTURE ONLY; present only where the reference sources were available
at build time).

Struct layouts follow the reference headers: ``fft_t`` (src/fft.h:16-24, with
the FFTW plan handles as pointers) and ``gal_t`` (src/gal.h:29-39).
"""
from __future__ import annotations

import ctypes as C
import os
import tempfile

import numpy as np

from . import REFLIB

_dp = C.POINTER(C.c_double)


class FFT_T(C.Structure):
    _fields_ = [("x2k", C.c_void_p), ("k2x", C.c_void_p), ("f", _dp),
                ("Ng", C.c_int), ("Ng_pad", C.c_int), ("Ng3_pad", C.c_long),
                ("L", C.c_double), ("offset", C.c_double * 3)]


class GAL_T(C.Structure):
    pass


GAL_T._fields_ = [("Np", C.c_long), ("V", C.c_double),
                  ("x", _dp), ("y", _dp), ("z", _dp),
                  ("vx", _dp), ("vy", _dp), ("vz", _dp),
                  ("rand", C.POINTER(GAL_T))]


def available() -> bool:
    return os.path.exists(REFLIB)


class RefLib:
    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            lib = C.CDLL(REFLIB)
            P_F, P_G = C.POINTER(FFT_T), C.POINTER(GAL_T)
            lib.fft_init.restype = P_F
            lib.fft_init.argtypes = [C.c_int, C.c_double, C.c_char_p]
            lib.fft_free.argtypes = [P_F]
            lib.fft_p2g.argtypes = [P_F, P_G, _dp]
            lib.fft_g2p.argtypes = [P_F, P_G]
            lib.fft_g2p.restype = _dp
            lib.fft_x2k.argtypes = [P_F, C.c_int]
            lib.fft_k2x.argtypes = [P_F, C.c_int]
            lib.fft_offset_phase.argtypes = [P_F, C.c_int]
            lib.fft_deconv.argtypes = [P_F]
            lib.fft_p2k.argtypes = [P_F, P_G]
            lib.gal_init.restype = P_G
            lib.gal_init.argtypes = [C.c_long, C.c_double]
            lib.gal_free.argtypes = [P_G]
            lib.P.argtypes = [P_F, P_G]
            lib.Pl.argtypes = [P_F, P_G, _dp, C.c_double, C.c_char_p]
            lib.Pmu.argtypes = [P_F, P_G, _dp, C.c_double, C.c_char_p]
            lib.gal_rsd.restype = P_G
            lib.gal_rsd.argtypes = [P_G, _dp, C.c_double]
            lib.gal_wrap.argtypes = [P_G, C.c_double]
            lib.gal_subbox.restype = P_G
            lib.gal_subbox.argtypes = [P_G, _dp, C.c_double]
            lib.gal_subsphere.restype = P_G
            lib.gal_subsphere.argtypes = [P_G, _dp, C.c_double]
            lib.gal_loadqpm_cubic.restype = P_G
            lib.gal_loadqpm_cubic.argtypes = [C.c_char_p, C.c_double]
            lib.free.argtypes = [C.c_void_p]
            cls._lib = lib
        return cls._lib


class RefGrid:
    """One reference ``fft_t`` driven through the reference's own functions."""

    def __init__(self, Ng: int, L: float):
        self.lib = RefLib.lib()
        self.p = self.lib.fft_init(int(Ng), float(L), b"FFTW_ESTIMATE")
        self.Ng = Ng
        self.Ng_pad = self.p.contents.Ng_pad

    def __del__(self):
        if getattr(self, "p", None):
            self.lib.fft_free(self.p)
            self.p = None

    @property
    def f(self) -> np.ndarray:
        n = self.p.contents.Ng3_pad
        return np.ctypeslib.as_array(self.p.contents.f, shape=(n,))

    @property
    def offset(self):
        return np.array(self.p.contents.offset[:])


class RefGal:
    def __init__(self, x, y, z, V, vel=None, rand=None):
        self.lib = RefLib.lib()
        n = len(x)
        self.p = self.lib.gal_init(n, float(V))
        g = self.p.contents
        for name, a in (("x", x), ("y", y), ("z", z)):
            dst = np.ctypeslib.as_array(getattr(g, name), shape=(n,))
            dst[:] = np.asarray(a, dtype=np.float64)
        self._rand = None
        if rand is not None:
            xr, yr, zr = rand
            self._rand = RefGal(xr, yr, zr, V)
            g.rand = self._rand.p
        if vel is not None:
            # velocities are malloc'd by the library owner in the reference
            # (src/io/qpm.c:20-22); keep numpy buffers alive here instead
            self._vel = [np.ascontiguousarray(v, dtype=np.float64) for v in vel]
            g.vx, g.vy, g.vz = (v.ctypes.data_as(_dp) for v in self._vel)

    def __del__(self):
        if getattr(self, "p", None):
            g = self.p.contents
            g.rand = None
            g.vx = g.vy = g.vz = None
            self.lib.gal_free(self.p)
            self.p = None


def read_table(path: str) -> np.ndarray:
    """Parse a Pl/Pmu text table (src/power.c:80-98,157-175); nan/-nan -> NaN."""
    rows = []
    with open(path) as fh:
        for line in fh:
            if line.startswith("#"):
                continue
            rows.append([float(t) for t in line.split()])
    return np.array(rows)


def run_pl_pmu(grid: RefGrid, gal: RefGal, los, dK):
    """Call the reference Pl and Pmu and return (text_pl, text_pmu)."""
    lib = RefLib.lib()
    with tempfile.TemporaryDirectory() as d:
        fpl, fmu = os.path.join(d, "pl.txt"), os.path.join(d, "pmu.txt")
        l1 = np.ascontiguousarray(los, dtype=np.float64).copy()
        lib.Pl(grid.p, gal.p, l1.ctypes.data_as(_dp), float(dK), fpl.encode())
        l2 = np.ascontiguousarray(los, dtype=np.float64).copy()
        lib.Pmu(grid.p, gal.p, l2.ctypes.data_as(_dp), float(dK), fmu.encode())
        with open(fpl) as a, open(fmu) as b:
            return a.read(), b.read()
