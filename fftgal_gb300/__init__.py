"""fftgal_gb300 -- GB300-native galaxy power spectra behind fftgal's C API.

The product is the C-ABI shared library ``libfftgal_gb300.so`` (headers in
``include/``: fft.h, power.h, gal.h, io/io.h are drop-in replacements for the
reference's src/fft.h, src/power.h, src/gal.h, src/io/io.h; fftgal_gb300.h holds
the extensions).  This module is its Python host-side mirror: ``Grid`` wraps
``fft_t`` and ``Catalog`` wraps ``gal_t`` with the same operation names and
argument meanings as the reference C functions, so tests and drivers read like
the reference's own code.  Every call goes through the C ABI into the CUDA
kernels; there is no CPU fallback -- if the library is missing or fails to load
this module raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libfftgal_gb300.so")

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_lp = C.POINTER(C.c_long)

VIEW_SYNC, VIEW_LAZY = 0, 1
MEM_HOST, MEM_DEVICE = 0, 1
PLAN_BUILTIN, PLAN_MEASURED, PLAN_FILE, PLAN_CACHE = 0, 1, 2, 3


class FFT_T(C.Structure):
    """``fft_t`` of include/fft.h (field order of src/fft.h:16-24)."""
    _fields_ = [("x2k", C.c_void_p), ("k2x", C.c_void_p), ("f", _dp),
                ("Ng", C.c_int), ("Ng_pad", C.c_int), ("Ng3_pad", C.c_long),
                ("L", C.c_double), ("offset", C.c_double * 3)]


class GAL_T(C.Structure):
    """``gal_t`` of include/gal.h (src/gal.h:29-39)."""


GAL_T._fields_ = [("Np", C.c_long), ("V", C.c_double),
                  ("x", _dp), ("y", _dp), ("z", _dp),
                  ("vx", _dp), ("vy", _dp), ("vz", _dp),
                  ("rand", C.POINTER(GAL_T))]

# every function the headers declare: name -> (restype, argtypes)
_P_F, _P_G = C.POINTER(FFT_T), C.POINTER(GAL_T)
SIGNATURES = {
    # include/fft.h
    "fft_init": (_P_F, [C.c_int, C.c_double, C.c_char_p]),
    "fft_free": (None, [_P_F]),
    "fft_p2g": (None, [_P_F, _P_G, _dp]),
    "fft_g2p": (_dp, [_P_F, _P_G]),
    "fft_x2k": (None, [_P_F, C.c_int]),
    "fft_k2x": (None, [_P_F, C.c_int]),
    "fft_offset_phase": (None, [_P_F, C.c_int]),
    "fft_deconv": (None, [_P_F]),
    "fft_p2k": (None, [_P_F, _P_G]),
    "fft_exportf": (_dp, [_P_F]),
    "fft_importf": (None, [_P_F, _dp]),
    # include/power.h
    "P": (None, [_P_F, _P_G]),
    "Pl": (None, [_P_F, _P_G, _dp, C.c_double, C.c_char_p]),
    "Pmu": (None, [_P_F, _P_G, _dp, C.c_double, C.c_char_p]),
    # include/gal.h
    "gal_init": (_P_G, [C.c_long, C.c_double]),
    "gal_resize": (None, [_P_G, C.c_long]),
    "gal_free": (None, [_P_G]),
    "gal_wrap": (None, [_P_G, C.c_double]),
    "gal_rsd": (_P_G, [_P_G, _dp, C.c_double]),
    "gal_subbox": (_P_G, [_P_G, _dp, C.c_double]),
    "gal_subsphere": (_P_G, [_P_G, _dp, C.c_double]),
    "pdist2": (C.c_double, [C.c_double] * 7),
    "hat": (None, [_dp]),
    # include/io/io.h
    "gal_loadqpm_cubic": (_P_G, [C.c_char_p, C.c_double]),
    # include/fftgal_gb300.h
    "fftgal_version": (C.c_int, []),
    "fftgal_last_status": (C.c_int, []),
    "fftgal_last_error": (C.c_char_p, []),
    "fftgal_grid_precision": (C.c_int, [_P_F]),
    "fftgal_set_host_view": (C.c_int, [_P_F, C.c_int]),
    "fftgal_sync_host": (C.c_int, [_P_F]),
    "fftgal_sync_device": (C.c_int, [_P_F]),
    "fftgal_set_stream": (C.c_int, [_P_F, C.c_void_p]),
    "fftgal_get_stream": (C.c_void_p, [_P_F]),
    "fftgal_set_quiet": (C.c_int, [_P_F, C.c_int]),
    "fftgal_device_grid": (C.c_void_p, [_P_F]),
    "fftgal_copy_grid": (C.c_int, [_P_F, C.c_void_p, C.c_int]),
    "fftgal_synchronize": (C.c_int, [_P_F]),
    "fftgal_nk": (C.c_int, [C.c_int, C.c_double, C.c_double]),
    "fftgal_power_f32": (C.c_int, [_P_F, C.c_void_p, C.c_void_p, C.c_void_p, C.c_long, C.c_double,
                                   C.c_int, _dp, C.c_double, C.c_int, _dp, _lp, _dp, _dp, _lp, _dp]),
    "fftgal_window_box": (C.c_int, [_P_F, C.c_int]),
    "fftgal_window_sphere": (C.c_int, [_P_F, C.c_int]),
    "fftgal_dl_sub": (C.c_int, [_P_F, C.c_int, C.c_int, C.c_int, _dp, C.c_double, _dp]),
    "fftgal_power_mixed_f32": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, _lp, _dp,
                                          C.POINTER(C.c_int), _dp, _dp, _dp, C.c_int, C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "fftgal_power_mixed_release": (C.c_int, []),
    "fftgal_power_batch_f32": (C.c_int, [_P_F, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, _lp, _dp, _dp,
                                         C.c_double, C.c_int, _dp, _lp, _dp, _dp, _lp, _dp]),
    "fftgal_mlp_nparams": (C.c_int, []),
    "fftgal_mlp_grad": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_long, C.c_void_p, C.c_void_p,
                                  C.c_void_p]),
    "fftgal_mlp_adam": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_float,
                                  C.c_void_p]),
    "fftgal_mlp_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_long, C.c_void_p, C.c_void_p]),
    "fftgal_alias_features": (C.c_int, [C.c_int, _dp, _dp, C.c_double, C.c_double, C.POINTER(C.c_float)]),
    "fftgal_alias_envelope": (C.c_double, [C.c_double]),
    "fftgal_plan_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), _dp]),
    "fftgal_plan_autotune": (C.c_int, [C.c_void_p, _dp]),
    "fftgal_launch_shapes": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), _dp]),
    "fftgal_plan_lookup": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int)]),
    "fftgal_plan_store": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), _dp,
                                    C.c_char_p]),
    "fftgal_plan_valid": (C.c_int, [C.c_int, C.c_int, C.c_int]),
    "fftgal_set_graphs": (C.c_int, [C.c_void_p, C.c_int]),
    "fftgal_fft_columns_f32": (C.c_int, [C.c_int, C.c_void_p, C.c_int, C.c_long, C.c_long, C.c_long, C.c_int,
                                         C.c_int, C.c_void_p]),
    "fftgal_power_learned_f32": (C.c_int, [_P_F, C.c_void_p, C.c_void_p, C.c_void_p, C.c_long, C.c_double,
                                           C.c_int, _dp, C.c_double, C.c_int, C.POINTER(C.c_float), _dp, _lp,
                                           _dp, _dp, _lp, _dp]),
    "fftgal_power_learned_checked_f32": (C.c_int, [_P_F, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, _lp, _dp,
                                                   C.c_int, _dp, C.c_double, C.c_int, C.POINTER(C.c_float),
                                                   C.c_int, C.c_double, _dp, _lp, _dp, _dp, _lp, _dp,
                                                   C.POINTER(C.c_int), _dp]),
    "fftgal_power_single_f32": (C.c_int, [_P_F, C.c_void_p, C.c_void_p, C.c_void_p, C.c_long, C.c_double,
                                          C.c_int, _dp, C.c_double, C.c_int, _dp, _lp, _dp, _dp, _lp, _dp]),
    "fftgal_power_rsd_f32": (C.c_int, [_P_F, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_long, C.c_double, C.c_int, _dp, C.c_double, C.c_double,
                                       C.c_int, _dp, _lp, _dp, _dp, _lp, _dp]),
    "fftgal_set_timing": (C.c_int, [_P_F, C.c_int]),
    "fftgal_stage_times": (C.c_int, [_P_F, _dp]),
    "fftgal_g2p_sum": (C.c_int, [_P_F, _P_G, _dp]),
    "fftgal_device_bytes": (C.c_long, [_P_F]),
    "fftgal_launch_count": (C.c_long, []),
    "fftgal_power_bins_noalloc": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_long, _dp,
                                            C.c_double, C.c_int, _dp, _lp, _dp, _dp, _lp, _dp, C.c_void_p]),
}

NSTAGES = 11
STAGES = ["upload", "paint_key", "paint_scan", "paint_scatter", "paint_tile", "fft_k", "fft_j",
          "fft_i", "finish", "finish_bin", "total"]

_lib = None


def lib() -> C.CDLL:
    """Load libfftgal_gb300.so (build it first with fftgal_gb300.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIBPATH):
            raise ImportError(f"{LIBPATH} is missing: run `python -m fftgal_gb300.build`")
        L = C.CDLL(LIBPATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        L.free = C.CDLL(None).free
        L.free.argtypes = [C.c_void_p]
        _lib = L
    return _lib


class FftgalError(RuntimeError):
    pass


def _check(status: int):
    if status != 0:
        msg = lib().fftgal_last_error()
        raise FftgalError(f"status {status}: {msg.decode() if msg else ''}")


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


class Catalog:
    """``gal_t`` owned through gal_init/gal_free (src/gal.c:11-48)."""

    def __init__(self, x, y, z, V: float, vel=None, rand: "Catalog | None" = None):
        L = lib()
        n = len(x)
        self.p = L.gal_init(n, float(V))
        g = self.p.contents
        for name, a in (("x", x), ("y", y), ("z", z)):
            np.ctypeslib.as_array(getattr(g, name), shape=(max(n, 1),))[:n] = _f64(a)
        self._vel = None
        if vel is not None:
            self._vel = [_f64(v) for v in vel]
            g.vx, g.vy, g.vz = (v.ctypes.data_as(_dp) for v in self._vel)
        self._rand = rand
        if rand is not None:
            g.rand = rand.p

    @property
    def Np(self) -> int:
        return self.p.contents.Np

    def __del__(self):
        p = getattr(self, "p", None)
        if p:
            g = p.contents
            g.rand = None           # owned by its own Catalog
            g.vx = g.vy = g.vz = None
            lib().gal_free(p)
            self.p = None


class Grid:
    """``fft_t`` through the C ABI.  ``precision`` ("f32"/"f64") and
    ``host_view`` ("sync"/"lazy") are read by fft_init from the environment."""

    def __init__(self, Ng: int, L: float, wisdom: str = "FFTW_ESTIMATE",
                 precision: str | None = None, host_view: str | None = None, quiet: bool = True):
        env = {}
        if precision is not None:
            env["FFTGAL_PRECISION"] = precision
        if host_view is not None:
            env["FFTGAL_HOST_VIEW"] = host_view
        if quiet:
            env["FFTGAL_QUIET"] = "1"
        old = {k: os.environ.get(k) for k in env}
        os.environ.update(env)
        try:
            self.p = lib().fft_init(int(Ng), float(L), wisdom.encode())
        finally:
            for k, v in old.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v
        self.Ng, self.L = int(Ng), float(L)
        self.Ng_pad = self.p.contents.Ng_pad

    def __del__(self):
        p = getattr(self, "p", None)
        if p:
            lib().fft_free(p)
            self.p = None

    # -- views ---------------------------------------------------------------
    @property
    def f(self) -> np.ndarray:
        """The host view ``fft_t.f`` (Ng3_pad doubles), zero-copy."""
        n = self.p.contents.Ng3_pad
        return np.ctypeslib.as_array(self.p.contents.f, shape=(n,))

    @property
    def real(self) -> np.ndarray:
        return self.f.reshape(self.Ng, self.Ng, self.Ng_pad)

    @property
    def cplx(self) -> np.ndarray:
        r = self.real
        return r[..., 0::2] + 1j * r[..., 1::2]

    @property
    def offset(self) -> np.ndarray:
        return np.array(self.p.contents.offset[:])

    @property
    def precision(self) -> int:
        return lib().fftgal_grid_precision(self.p)

    # -- reference operations (src/fft.h, src/power.h) ------------------------
    def p2g(self, cat: Catalog, offset) -> np.ndarray:
        off = _f64(offset).copy()
        lib().fft_p2g(self.p, cat.p, off.ctypes.data_as(_dp))
        return off

    def x2k(self, phase_on: int):
        lib().fft_x2k(self.p, int(phase_on))

    def k2x(self, phase_off: int):
        lib().fft_k2x(self.p, int(phase_off))

    def offset_phase(self, onoff: int):
        lib().fft_offset_phase(self.p, int(onoff))

    def deconv(self):
        lib().fft_deconv(self.p)

    def p2k(self, cat: Catalog):
        lib().fft_p2k(self.p, cat.p)

    def g2p(self, cat: Catalog) -> np.ndarray:
        ptr = lib().fft_g2p(self.p, cat.p)
        out = np.ctypeslib.as_array(ptr, shape=(max(cat.Np, 1),))[:cat.Np].copy()
        lib().free(C.cast(ptr, C.c_void_p))
        return out

    def exportf(self) -> np.ndarray:
        ptr = lib().fft_exportf(self.p)
        out = np.ctypeslib.as_array(ptr, shape=(self.p.contents.Ng3_pad,)).copy()
        lib().free(C.cast(ptr, C.c_void_p))
        return out

    def importf(self, src: np.ndarray):
        src = _f64(src)
        lib().fft_importf(self.p, src.ctypes.data_as(_dp))

    def power(self, cat: Catalog):
        lib().P(self.p, cat.p)

    def pl(self, cat: Catalog, los, dK: float, file: str) -> np.ndarray:
        l = _f64(los).copy()
        lib().Pl(self.p, cat.p, l.ctypes.data_as(_dp), float(dK), file.encode())
        return l

    def pmu(self, cat: Catalog, los, dK: float, file: str) -> np.ndarray:
        l = _f64(los).copy()
        lib().Pmu(self.p, cat.p, l.ctypes.data_as(_dp), float(dK), file.encode())
        return l

    # -- extensions (include/fftgal_gb300.h) -------------------------------------
    def set_host_view(self, mode: int):
        _check(lib().fftgal_set_host_view(self.p, int(mode)))

    def sync_host(self):
        _check(lib().fftgal_sync_host(self.p))

    def sync_device(self):
        _check(lib().fftgal_sync_device(self.p))

    def set_graphs(self, on: bool):
        """Graph-captured batches on (default) or off (fftgal_set_graphs)."""
        _check(lib().fftgal_set_graphs(self.p, int(bool(on))))

    def plan_info(self) -> dict:
        """Launch shapes of the FFT passes (fftgal_plan_info): ``tune`` = [k rows
        per CTA, j and i log2 columns per CTA], ``source`` (FFTGAL_PLAN_*) and
        the measured ms of each pass."""
        t = (C.c_int * 3)()
        src = C.c_int()
        ms = np.zeros(3)
        _check(lib().fftgal_plan_info(self.p, t, C.byref(src), ms.ctypes.data_as(_dp)))
        return {"tune": list(t), "source": src.value, "ms": ms}

    def autotune(self) -> np.ndarray:
        """Measure the FFT launch shapes now (clears the grid)."""
        ms = np.zeros(3)
        _check(lib().fftgal_plan_autotune(self.p, ms.ctypes.data_as(_dp)))
        return ms

    def launch_shapes(self) -> dict:
        """fftgal_launch_shapes: paint CTAs per SM, binning CTAs per SM and fold
        period (0: built-in), where they came from, measured times."""
        sh = (C.c_int * 3)()
        src = C.c_int(0)
        ms = np.zeros(2)
        _check(lib().fftgal_launch_shapes(self.p, sh, C.byref(src), ms.ctypes.data_as(_dp)))
        return dict(paint_cta=sh[0], bin_cta=sh[1], bin_fold=sh[2], source=src.value, ms=ms)

    def set_stream(self, stream_ptr: int | None):
        """Run the grid's work on a CUDA stream: None for the library's own
        stream, else a cudaStream_t.  0, torch's handle of the legacy default
        stream, is passed as cudaStreamLegacy (the C API reads NULL as the
        library's own stream)."""
        if stream_ptr == 0:
            stream_ptr = 1  # cudaStreamLegacy
        _check(lib().fftgal_set_stream(self.p, stream_ptr))

    def set_timing(self, on: bool):
        _check(lib().fftgal_set_timing(self.p, int(on)))

    def stage_times(self) -> dict:
        out = np.zeros(NSTAGES)
        _check(lib().fftgal_stage_times(self.p, out.ctypes.data_as(_dp)))
        return dict(zip(STAGES, out.tolist()))

    def window_box(self, Ngsub: int):
        """Sub-box window deconvolution of the real-space grid (src/app/Psb.c:76-83)."""
        _check(lib().fftgal_window_box(self.p, int(Ngsub)))

    def window_sphere(self, Ngsub: int):
        """Sub-sphere window deconvolution of the real-space grid (src/app/Pss.c:72-84)."""
        _check(lib().fftgal_window_sphere(self.p, int(Ngsub)))

    def dl_sub(self, sphere: int, Nsub: int, los_list, bias: float = 1.0) -> np.ndarray:
        """Super-sample modes [nlos, 3, Nsub^3] of the k-space field held by the
        grid (src/app/DLsb.c / DLss.c per line of sight)."""
        l = np.ascontiguousarray(np.asarray(los_list, dtype=np.float64).reshape(-1, 3))
        out = np.zeros((len(l), 3, Nsub ** 3))
        _check(lib().fftgal_dl_sub(self.p, int(sphere), int(Nsub), len(l), l.ctypes.data_as(_dp), float(bias),
                                   out.ctypes.data_as(_dp)))
        return out

    def copy_from(self, ptr: int):
        """Fill the canonical grid from a CUDA-visible buffer (raw pointer)."""
        _check(lib().fftgal_copy_grid(self.p, ptr, 1))

    def copy_to(self, ptr: int):
        """Copy the canonical grid into a CUDA-visible buffer (raw pointer)."""
        _check(lib().fftgal_copy_grid(self.p, ptr, 0))

    def synchronize(self):
        _check(lib().fftgal_synchronize(self.p))

    def device_bytes(self) -> int:
        return lib().fftgal_device_bytes(self.p)

    def g2p_sum(self, cat: Catalog) -> np.ndarray:
        out = np.zeros(cat.Np)
        _check(lib().fftgal_g2p_sum(self.p, cat.p, out.ctypes.data_as(_dp)))
        return out

    def power_f32(self, x, y, z, V: float, los, dK: float, Nmu: int = 3, where: int = MEM_HOST,
                  Np: int | None = None, interlace: bool = True) -> dict:
        """Fused interlaced P_l and wedges of one FP32 catalog (``interlace=False``:
        a single paint, fftgal_power_single_f32).  For ``where=MEM_DEVICE`` pass
        integer device pointers and ``Np``."""
        if where == MEM_HOST:
            xs = [np.ascontiguousarray(a, dtype=np.float32) for a in (x, y, z)]
            ptrs = [a.ctypes.data for a in xs]
            Np = len(xs[0])
        else:
            ptrs = [int(x), int(y), int(z)]
        NK = lib().fftgal_nk(self.Ng, self.L, float(dK))
        K = np.zeros(NK)
        N = np.zeros(NK, dtype=np.int64)
        P = np.zeros((NK, 4))
        Km = np.zeros((NK, Nmu))
        Nm = np.zeros((NK, Nmu), dtype=np.int64)
        Pm = np.zeros((NK, Nmu))
        l = _f64(los)
        fn = lib().fftgal_power_f32 if interlace else lib().fftgal_power_single_f32
        _check(fn(self.p, ptrs[0], ptrs[1], ptrs[2], int(Np), float(V), int(where),
                                      l.ctypes.data_as(_dp), float(dK), int(Nmu),
                                      K.ctypes.data_as(_dp), N.ctypes.data_as(_lp), P.ctypes.data_as(_dp),
                                      Km.ctypes.data_as(_dp), Nm.ctypes.data_as(_lp), Pm.ctypes.data_as(_dp)))
        return dict(K=K, N=N, P=P, Kmu=Km, Nmu=Nm, Pmu=Pm)

    def power_batch_f32(self, cats, V, los, dK: float, Nmu: int = 3) -> list:
        """fftgal_power_f32 of every (x, y, z) host catalog in ``cats`` (V: one
        volume per catalog), uploads overlapped with the computation.  Arrays
        that are FP32 and C-contiguous (ideally page-locked) are used in place."""
        arrs = [[np.ascontiguousarray(a, dtype=np.float32) for a in c] for c in cats]
        n = len(arrs)
        ptr = [(C.c_void_p * n)(*[c[a].ctypes.data for c in arrs]) for a in range(3)]
        Np = np.array([len(c[0]) for c in arrs], dtype=np.int64)
        Vs = np.ascontiguousarray(np.broadcast_to(np.asarray(V, dtype=np.float64), (n,)))
        NK = lib().fftgal_nk(self.Ng, self.L, float(dK))
        K = np.zeros((n, NK))
        N = np.zeros((n, NK), dtype=np.int64)
        P = np.zeros((n, NK, 4))
        Km = np.zeros((n, NK, Nmu))
        Nm = np.zeros((n, NK, Nmu), dtype=np.int64)
        Pm = np.zeros((n, NK, Nmu))
        l = _f64(los)
        _check(lib().fftgal_power_batch_f32(self.p, n, ptr[0], ptr[1], ptr[2], Np.ctypes.data_as(_lp),
                                            Vs.ctypes.data_as(_dp), l.ctypes.data_as(_dp), float(dK), int(Nmu),
                                            K.ctypes.data_as(_dp), N.ctypes.data_as(_lp), P.ctypes.data_as(_dp),
                                            Km.ctypes.data_as(_dp), Nm.ctypes.data_as(_lp), Pm.ctypes.data_as(_dp)))
        return [dict(K=K[c], N=N[c], P=P[c], Kmu=Km[c], Nmu=Nm[c], Pmu=Pm[c]) for c in range(n)]

    def power_learned_f32(self, x, y, z, V: float, los, dK: float, params, Nmu: int = 3,
                          where: int = MEM_HOST, Np: int | None = None) -> dict:
        """fftgal_power_learned_f32: one paint, multipoles corrected by the
        perceptron with parameters ``params`` (fftgal_mlp_nparams() floats)."""
        if where == MEM_HOST:
            arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in (x, y, z)]
            ptrs = [a.ctypes.data for a in arrs]
            Np = len(arrs[0])
        else:
            ptrs = [int(x), int(y), int(z)]
        p = np.ascontiguousarray(params, dtype=np.float32)
        NK = lib().fftgal_nk(self.Ng, self.L, float(dK))
        K, N, P = np.zeros(NK), np.zeros(NK, dtype=np.int64), np.zeros((NK, 4))
        Km, Nm, Pm = np.zeros((NK, Nmu)), np.zeros((NK, Nmu), dtype=np.int64), np.zeros((NK, Nmu))
        l = _f64(los)
        _check(lib().fftgal_power_learned_f32(self.p, ptrs[0], ptrs[1], ptrs[2], int(Np), float(V), int(where),
                                              l.ctypes.data_as(_dp), float(dK), int(Nmu),
                                              p.ctypes.data_as(C.POINTER(C.c_float)), K.ctypes.data_as(_dp),
                                              N.ctypes.data_as(_lp), P.ctypes.data_as(_dp), Km.ctypes.data_as(_dp),
                                              Nm.ctypes.data_as(_lp), Pm.ctypes.data_as(_dp)))
        return dict(K=K, N=N, P=P, Kmu=Km, Nmu=Nm, Pmu=Pm)

    def power_learned_checked_f32(self, cats, V, los, dK: float, params, holdout_every: int, tol: float,
                                  Nmu: int = 3):
        """fftgal_power_learned_checked_f32 over host catalogs ``cats``:
        (results, used, disagreement), used[c] 0 learned, 1 checked
        (interlaced reported), 2 interlaced fallback."""
        arrs = [[np.ascontiguousarray(a, dtype=np.float32) for a in c] for c in cats]
        n = len(arrs)
        ptr = [(C.c_void_p * n)(*[c[a].ctypes.data for c in arrs]) for a in range(3)]
        Np = np.array([len(c[0]) for c in arrs], dtype=np.int64)
        Vs = np.ascontiguousarray(np.broadcast_to(np.asarray(V, dtype=np.float64), (n,)))
        p = np.ascontiguousarray(params, dtype=np.float32)
        NK = lib().fftgal_nk(self.Ng, self.L, float(dK))
        K, N, P = np.zeros((n, NK)), np.zeros((n, NK), dtype=np.int64), np.zeros((n, NK, 4))
        Km, Nm, Pm = np.zeros((n, NK, Nmu)), np.zeros((n, NK, Nmu), dtype=np.int64), np.zeros((n, NK, Nmu))
        used = np.zeros(n, dtype=np.int32)
        dis = np.zeros(n)
        l = _f64(los)
        _check(lib().fftgal_power_learned_checked_f32(
            self.p, n, ptr[0], ptr[1], ptr[2], Np.ctypes.data_as(_lp), Vs.ctypes.data_as(_dp), MEM_HOST,
            l.ctypes.data_as(_dp), float(dK), int(Nmu), p.ctypes.data_as(C.POINTER(C.c_float)), int(holdout_every),
            float(tol), K.ctypes.data_as(_dp), N.ctypes.data_as(_lp), P.ctypes.data_as(_dp), Km.ctypes.data_as(_dp),
            Nm.ctypes.data_as(_lp), Pm.ctypes.data_as(_dp), used.ctypes.data_as(C.POINTER(C.c_int)),
            dis.ctypes.data_as(_dp)))
        res = [dict(K=K[c], N=N[c], P=P[c], Kmu=Km[c], Nmu=Nm[c], Pmu=Pm[c]) for c in range(n)]
        return res, used, dis

    def power_rsd_f32(self, x, y, z, vx, vy, vz, V: float, los, aH: float, dK: float, Nmu: int = 3,
                      where: int = MEM_HOST, Np: int | None = None) -> dict:
        """power_f32 of the catalog displaced along ``los`` by (v . los)/aH
        (gal_rsd fused into the paint)."""
        if where == MEM_HOST:
            arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in (x, y, z, vx, vy, vz)]
            ptrs = [a.ctypes.data for a in arrs]
            Np = len(arrs[0])
        else:
            ptrs = [int(a) for a in (x, y, z, vx, vy, vz)]
        NK = lib().fftgal_nk(self.Ng, self.L, float(dK))
        K = np.zeros(NK)
        N = np.zeros(NK, dtype=np.int64)
        P = np.zeros((NK, 4))
        Km = np.zeros((NK, Nmu))
        Nm = np.zeros((NK, Nmu), dtype=np.int64)
        Pm = np.zeros((NK, Nmu))
        l = _f64(los)
        _check(lib().fftgal_power_rsd_f32(self.p, *ptrs, int(Np), float(V), int(where), l.ctypes.data_as(_dp),
                                          float(aH), float(dK), int(Nmu), K.ctypes.data_as(_dp),
                                          N.ctypes.data_as(_lp), P.ctypes.data_as(_dp), Km.ctypes.data_as(_dp),
                                          Nm.ctypes.data_as(_lp), Pm.ctypes.data_as(_dp)))
        return dict(K=K, N=N, P=P, Kmu=Km, Nmu=Nm, Pmu=Pm)


def power_bins_noalloc(fk: int, Ng: int, L: float, V: float, Np: int, los, dK: float, Nmu: int = 3,
                       stream: int | None = None) -> dict:
    """Multipoles and wedges of the deconvolved FP32 k-space grid at device
    pointer ``fk`` without any GPU allocation (fftgal_power_bins_noalloc)."""
    NK = lib().fftgal_nk(int(Ng), float(L), float(dK))
    K = np.zeros(NK)
    N = np.zeros(NK, dtype=np.int64)
    P = np.zeros((NK, 4))
    Km = np.zeros((NK, Nmu))
    Nm = np.zeros((NK, Nmu), dtype=np.int64)
    Pm = np.zeros((NK, Nmu))
    l = _f64(los)
    _check(lib().fftgal_power_bins_noalloc(int(fk), int(Ng), float(L), float(V), int(Np), l.ctypes.data_as(_dp),
                                           float(dK), int(Nmu), K.ctypes.data_as(_dp), N.ctypes.data_as(_lp),
                                           P.ctypes.data_as(_dp), Km.ctypes.data_as(_dp), Nm.ctypes.data_as(_lp),
                                           Pm.ctypes.data_as(_dp), stream))
    return dict(K=K, N=N, P=P, Kmu=Km, Nmu=Nm, Pmu=Pm)


def power_mixed_f32(cats, V, Ng, L, los, dK, Nmu: int = 3) -> list:
    """fftgal_power_mixed_f32: interlaced P_l and wedges of every (x, y, z)
    catalog of ``cats`` with its own volume V[c], grid Ng[c], box L[c] and bin
    width dK[c] (scalars broadcast), in one call; a list of result dicts."""
    n = len(cats)
    arrs = [[np.ascontiguousarray(a, dtype=np.float32) for a in c] for c in cats]
    ptr = [(C.c_void_p * n)(*[c[a].ctypes.data for c in arrs]) for a in range(3)]
    Np = np.array([len(c[0]) for c in arrs], dtype=np.int64)

    def vec(v, dt):
        return np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=dt), (n,)))

    Vs, Ls, dKs, Ngs = vec(V, np.float64), vec(L, np.float64), vec(dK, np.float64), vec(Ng, np.int32)
    out = []
    for c in range(n):
        NK = lib().fftgal_nk(int(Ngs[c]), float(Ls[c]), float(dKs[c]))
        out.append(dict(K=np.zeros(NK), N=np.zeros(NK, dtype=np.int64), P=np.zeros((NK, 4)),
                        Kmu=np.zeros((NK, Nmu)), Nmu=np.zeros((NK, Nmu), dtype=np.int64),
                        Pmu=np.zeros((NK, Nmu))))
    tabs = [(C.c_void_p * n)(*[r[k].ctypes.data for r in out]) for k in ("K", "N", "P", "Kmu", "Nmu", "Pmu")]
    l = _f64(los)
    _check(lib().fftgal_power_mixed_f32(n, ptr[0], ptr[1], ptr[2], Np.ctypes.data_as(_lp), Vs.ctypes.data_as(_dp),
                                        Ngs.ctypes.data_as(C.POINTER(C.c_int)), Ls.ctypes.data_as(_dp),
                                        l.ctypes.data_as(_dp), dKs.ctypes.data_as(_dp), int(Nmu), *tabs))
    return out


def power_mixed_release():
    _check(lib().fftgal_power_mixed_release())


def nk(Ng: int, L: float, dK: float) -> int:
    return lib().fftgal_nk(int(Ng), float(L), float(dK))


def read_table(path: str) -> np.ndarray:
    """Rows of a Pl/Pmu text file (src/power.c:80-98,157-175)."""
    rows = []
    with open(path) as fh:
        for line in fh:
            if not line.startswith("#"):
                rows.append([float(t) for t in line.split()])
    return np.array(rows)
