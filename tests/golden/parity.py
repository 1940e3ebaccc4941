"""The parity criterion of the power-spectrum path, shared by the tests and
bench.py: mode counts bit-exact, and every P_l (l = 0, 2, 4) within a relative
tolerance of the FP64 answer for k < 0.8 k_Nyq, the error taken in units of
|P_0^FP64(k)| + Pshot (shot-noise-subtracted multipoles of a uniform catalog
are ~0, so the shot noise sets the scale).  Results are dicts with K, N, P
[NK, 4] (l = 0, 2, 4, 6), Kmu, Nmu, Pmu [NK, Nmu] as returned by
fftgal_gb300.Grid.power_f32 and oracle.power_spectrum."""
from __future__ import annotations

import numpy as np

TOL_P024 = 1e-4  # k < 0.8 k_Nyq, l = 0, 2, 4 and every wedge
TOL_ALL = 1e-3   # every bin and l = 6 (FP32 rounding is amplified up to
                 # ~200x by the window deconvolution in the corner of the cube)


def errors(res: dict, ref: dict, Pshot: float, Ng: int, L: float, kfrac: float = 0.8) -> dict:
    """Largest errors of `res` against the FP64 answer `ref` (see module doc)."""
    K, P = ref["K"], ref["P"]
    den = np.abs(P[:, 0]) + Pshot
    sel = np.isfinite(P[:, 0]) & (K < kfrac * np.pi * Ng / L)
    e024 = np.abs(res["P"][sel, :3] - P[sel, :3]) / den[sel, None]
    fin = np.isfinite(P)
    e_all = (np.abs(res["P"] - P) / den[:, None])[fin]
    Pm = ref["Pmu"]
    finm = np.isfinite(Pm) & sel[:, None]
    emu = (np.abs(res["Pmu"] - Pm) / den[:, None])[finm]
    nan_same = bool(np.array_equal(np.isnan(res["P"]), np.isnan(P)))
    return {
        "max_rel_err_P024": float(e024.max()) if e024.size else 0.0,
        "max_rel_err_all_bins": float(e_all.max()) if e_all.size else 0.0,
        "max_rel_err_wedges": float(emu.max()) if emu.size else 0.0,
        "counts_exact": bool(np.array_equal(res["N"], ref["N"]) and np.array_equal(res["Nmu"], ref["Nmu"])),
        "empty_bins_match": nan_same,
        "K_max_rel": float(np.nanmax(np.abs(res["K"] - K) / np.where(K > 0, K, 1.0))),
        "bins_compared": int(sel.sum()),
    }


def passes(e: dict, tol: float = TOL_P024, tol_all: float = TOL_ALL) -> bool:
    return (e["counts_exact"] and e["empty_bins_match"] and e["max_rel_err_P024"] <= tol
            and e["max_rel_err_wedges"] <= tol and e["max_rel_err_all_bins"] <= tol_all)


def golden_result(npz, name: str, il: int, nmu: int = 3) -> dict:
    """The FP64 reference answer for catalog `name`, line of sight `il` of
    tests/golden/headline_ng1024.npz."""
    k = f"{name}_los{il}"
    return dict(K=npz[k + "_K"], N=npz[k + "_N"], P=npz[k + "_P"], Kmu=npz[f"{k}_mu{nmu}_K"],
                Nmu=npz[f"{k}_mu{nmu}_N"], Pmu=npz[f"{k}_mu{nmu}_P"])
