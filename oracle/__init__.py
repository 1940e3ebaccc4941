"""CPU oracle for the power-spectrum path (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this package, as the checker.  The shipped library (``fftgal_gb300``) never
imports, links or calls it.

Two oracles live here:

* ``Oracle``: ctypes wrapper of ``liboracle.so``, the project's FP64 C
  restatement of src/fft.c and src/power.c (oracle/fftgal_oracle.c) on the
  project's FP64 FFT (oracle/fft64.c).
* ``RefLib``: ctypes wrapper of ``_ref/librefgal.so``, the reference's own
  src/fft.c, src/gal.c, src/power.c compiled unmodified against shim
  FFTW/GSL headers (oracle/Makefile target ``ref``).  It exists only where the
  reference sources are present; it is used to pin ``Oracle`` and to write the
  golden fixtures under tests/golden/.

``oracle.mlp`` restates the learned-correction perceptron's forward pass and
gradient in FP64 (numpy) for the parity tests of the GPU kernels.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REFLIB = os.path.join(HERE, "_ref", "librefgal.so")

_dp = C.POINTER(C.c_double)
_lp = C.POINTER(C.c_long)


def build(ref: bool = False) -> None:
    """Compile liboracle.so (and the reference build when ``ref`` and the
    reference sources exist: FFTGAL_REFERENCE_DIR, else the location the
    build recipe oracle/Makefile names)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref and subprocess.run(["make", "-s", "-C", HERE, "have-ref"], capture_output=True).returncode == 0:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def reference_dir() -> str | None:
    """The reference checkout: FFTGAL_REFERENCE_DIR, else the one the
    reference build in oracle/_ref was compiled from, else None."""
    d = os.environ.get("FFTGAL_REFERENCE_DIR")
    if d:
        return d if os.path.isdir(d) else None
    try:
        with open(os.path.join(HERE, "_ref", "SOURCE_DIR")) as fh:
            d = fh.read().strip()
    except OSError:
        return None
    return d if os.path.isdir(d) else None


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def nk(Ng: int, L: float, dK: float) -> int:
    """Number of k bins (src/power.c:34-36)."""
    KF = 2 * np.pi / L
    return int(np.floor(1.73205080756887729352744634151 * (Ng // 2) * (KF / dK))) + 1


class Oracle:
    """FP64 C restatement of the reference path (liboracle.so)."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            if not os.path.exists(LIB):
                build()
            lib = C.CDLL(LIB)
            lib.og_grid_new.restype = C.c_void_p
            lib.og_grid_new.argtypes = [C.c_int, C.c_double]
            lib.og_grid_free.argtypes = [C.c_void_p]
            lib.og_grid_data.restype = _dp
            lib.og_grid_data.argtypes = [C.c_void_p]
            lib.og_grid_size.restype = C.c_long
            lib.og_grid_size.argtypes = [C.c_void_p]
            lib.og_grid_offset.argtypes = [C.c_void_p, _dp]
            lib.og_p2g.argtypes = [C.c_void_p, C.c_long, C.c_double, _dp, _dp, _dp,
                                   C.c_long, _dp, _dp, _dp, _dp]
            lib.og_p2k.argtypes = [C.c_void_p, C.c_long, C.c_double, _dp, _dp, _dp,
                                   C.c_long, _dp, _dp, _dp]
            lib.og_x2k.argtypes = [C.c_void_p, C.c_int]
            lib.og_k2x.argtypes = [C.c_void_p, C.c_int]
            lib.og_offset_phase.argtypes = [C.c_void_p, C.c_int]
            lib.og_offset_phase.restype = C.c_int
            lib.og_deconv.argtypes = [C.c_void_p]
            lib.og_g2p.argtypes = [C.c_void_p, C.c_long, _dp, _dp, _dp, _dp]
            lib.og_power.argtypes = [C.c_void_p, C.c_long, C.c_double, C.c_long]
            lib.og_pl.argtypes = [C.c_void_p, _dp, C.c_double, _dp, _lp, _dp]
            lib.og_pl.restype = C.c_int
            lib.og_pmu.argtypes = [C.c_void_p, _dp, C.c_double, C.c_int, _dp, _lp, _dp]
            lib.og_pmu.restype = C.c_int
            lib.og_rsd.argtypes = [C.c_long, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                                   C.c_double, _dp, _dp, _dp]
            lib.og_wrap.argtypes = [C.c_long, _dp, _dp, _dp, C.c_double]
            lib.og_window_box.argtypes = [C.c_void_p, C.c_int]
            lib.og_dl.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, C.c_int, C.c_double, _dp]
            lib.og_window_sphere.argtypes = [C.c_void_p, C.c_int]
            cls._lib = lib
        return cls._lib

    def __init__(self, Ng: int, L: float):
        self.Ng, self.L = int(Ng), float(L)
        self.Ng_pad = 2 * (self.Ng // 2 + 1)
        self._g = self.lib().og_grid_new(self.Ng, self.L)
        if not self._g:
            raise MemoryError("og_grid_new failed")
        n = self.lib().og_grid_size(self._g)
        self.f = np.ctypeslib.as_array(self.lib().og_grid_data(self._g), shape=(n,))

    def __del__(self):
        if getattr(self, "_g", None):
            self.lib().og_grid_free(self._g)
            self._g = None

    # views -----------------------------------------------------------------
    @property
    def real(self) -> np.ndarray:
        """[Ng, Ng, Ng_pad] real view (configuration space)."""
        return self.f.reshape(self.Ng, self.Ng, self.Ng_pad)

    @property
    def cplx(self) -> np.ndarray:
        """[Ng, Ng, Ng/2+1] complex copy (Fourier space)."""
        r = self.real
        return r[..., 0::2] + 1j * r[..., 1::2]

    @property
    def offset(self) -> np.ndarray:
        out = np.zeros(3)
        self.lib().og_grid_offset(self._g, _ptr(out))
        return out

    # reference operations -------------------------------------------------
    def p2g(self, x, y, z, V, offset, rand=None):
        x, y, z = _f64(x), _f64(y), _f64(z)
        off = _f64(offset).copy()
        xr = yr = zr = None
        Nr = 0
        if rand is not None:
            xr, yr, zr = (_f64(a) for a in rand)
            Nr = len(xr)
        self.lib().og_p2g(self._g, len(x), float(V), _ptr(x), _ptr(y), _ptr(z),
                          Nr, _ptr(xr), _ptr(yr), _ptr(zr), _ptr(off))
        return off

    def p2k(self, x, y, z, V, rand=None):
        x, y, z = _f64(x), _f64(y), _f64(z)
        xr = yr = zr = None
        Nr = 0
        if rand is not None:
            xr, yr, zr = (_f64(a) for a in rand)
            Nr = len(xr)
        self.lib().og_p2k(self._g, len(x), float(V), _ptr(x), _ptr(y), _ptr(z),
                          Nr, _ptr(xr), _ptr(yr), _ptr(zr))

    def x2k(self, phase_on: int):
        self.lib().og_x2k(self._g, int(phase_on))

    def k2x(self, phase_off: int):
        self.lib().og_k2x(self._g, int(phase_off))

    def offset_phase(self, onoff: int) -> int:
        return self.lib().og_offset_phase(self._g, int(onoff))

    def deconv(self):
        self.lib().og_deconv(self._g)

    def g2p(self, x, y, z) -> np.ndarray:
        x, y, z = _f64(x), _f64(y), _f64(z)
        out = np.zeros(len(x))
        self.lib().og_g2p(self._g, len(x), _ptr(x), _ptr(y), _ptr(z), _ptr(out))
        return out

    def window_box(self, Ngsub: int):
        """src/app/Psb.c:76-83 on the real-space grid."""
        self.lib().og_window_box(self._g, int(Ngsub))

    def window_sphere(self, Ngsub: int):
        """src/app/Pss.c:72-84 on the real-space grid."""
        self.lib().og_window_sphere(self._g, int(Ngsub))

    def dl(self, sphere: int, Nsub: int, los, iL: int, bias: float = 1.0) -> np.ndarray:
        """One line-of-sight, one-multipole step of src/app/DLsb.c:56-92
        (sphere=0) / DLss.c:54-90 (sphere=1); the grid must hold the
        unfiltered k-space field and is left in configuration space."""
        out = np.zeros(Nsub ** 3)
        self.lib().og_dl(self._g, int(sphere), int(Nsub), _ptr(_f64(los).copy()), int(iL), float(bias), _ptr(out))
        return out

    def power(self, Np: int, V: float, Nr: int = 0):
        self.lib().og_power(self._g, int(Np), float(V), int(Nr))

    def pl(self, los, dK):
        """-> (K[NK], N[NK], P[NK,4], status, los_hat)"""
        los = _f64(los).copy()
        n = nk(self.Ng, self.L, dK)
        K = np.zeros(n)
        N = np.zeros(n, dtype=np.int64)
        P = np.zeros((n, 4))
        st = self.lib().og_pl(self._g, _ptr(los), float(dK), _ptr(K),
                              N.ctypes.data_as(_lp), _ptr(P))
        return K, N, P, st, los

    def pmu(self, los, dK, Nmu=3):
        """-> (K[NK,Nmu], N[NK,Nmu], P[NK,Nmu], status, los_hat)"""
        los = _f64(los).copy()
        n = nk(self.Ng, self.L, dK)
        K = np.zeros((n, Nmu))
        N = np.zeros((n, Nmu), dtype=np.int64)
        P = np.zeros((n, Nmu))
        st = self.lib().og_pmu(self._g, _ptr(los), float(dK), int(Nmu), _ptr(K),
                               N.ctypes.data_as(_lp), _ptr(P))
        return K, N, P, st, los

    @classmethod
    def rsd(cls, x, y, z, vx, vy, vz, los, aH):
        x, y, z, vx, vy, vz = (_f64(a) for a in (x, y, z, vx, vy, vz))
        los = _f64(los).copy()
        xo, yo, zo = np.zeros_like(x), np.zeros_like(y), np.zeros_like(z)
        cls.lib().og_rsd(len(x), _ptr(x), _ptr(y), _ptr(z), _ptr(vx), _ptr(vy),
                         _ptr(vz), _ptr(los), float(aH), _ptr(xo), _ptr(yo), _ptr(zo))
        return xo, yo, zo

    @classmethod
    def wrap(cls, x, y, z, L):
        x, y, z = (_f64(a).copy() for a in (x, y, z))
        cls.lib().og_wrap(len(x), _ptr(x), _ptr(y), _ptr(z), float(L))
        return x, y, z


def power_spectrum(Ng, L, x, y, z, los, dK, Nmu=3, V=None, interlace=True):
    """Convenience: the P.c sequence fft_p2k -> P -> Pl -> Pmu on one catalog
    (src/app/P.c:55-66), in FP64.  Returns a dict of arrays."""
    V = float(L) ** 3 if V is None else V
    g = Oracle(Ng, L)
    if interlace:
        g.p2k(x, y, z, V)
    else:
        g.p2g(x, y, z, V, [0.0, 0.0, 0.0])
        g.x2k(0)
        g.deconv()
    g.power(len(x), V)
    K, N, P, st1, _ = g.pl(los, dK)
    Km, Nm, Pm, st2, _ = g.pmu(los, dK, Nmu)
    return dict(K=K, N=N, P=P, Kmu=Km, Nmu=Nm, Pmu=Pm, status=(st1, st2))
