"""The C-ABI boundary without a GPU: the shared library loads, exports every
function that include/*.h declares, and the reference's own drivers compile
and link unchanged against these headers and this library."""
import os
import re
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
sys.path.insert(0, ROOT)
import oracle  # noqa: E402  (locates the reference checkout; test infrastructure)

REF = oracle.reference_dir() or ""


@pytest.fixture(scope="module")
def built():
    from fftgal_gb300 import build
    build.build()
    import fftgal_gb300
    return fftgal_gb300


def declared_functions():
    names = set()
    for dirpath, _, files in os.walk(INCLUDE):
        for f in files:
            if not f.endswith(".h"):
                continue
            text = open(os.path.join(dirpath, f)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            text = re.sub(r"#define[^\n]*", "", text)
            for m in re.finditer(r"^[A-Za-z_][\w \t\*]*?\b([A-Za-z_]\w*)\s*\(([^;{}]*)\)\s*[;{]", text, re.M):
                name = m.group(1)
                if m.group(0).lstrip().startswith("static"):
                    continue  # header-only helpers are not library symbols
                if name not in ("if", "for", "while", "return", "sizeof"):
                    names.add(name)
    return names


def test_headers_declare_reference_api():
    names = declared_functions()
    ref = {"fft_init", "fft_free", "fft_p2g", "fft_g2p", "fft_x2k", "fft_k2x", "fft_offset_phase",
           "fft_deconv", "fft_p2k", "fft_exportf", "fft_importf", "P", "Pl", "Pmu", "gal_init",
           "gal_resize", "gal_free", "gal_wrap", "gal_rsd", "gal_subbox", "gal_subsphere", "pdist2",
           "hat", "gal_loadqpm_cubic"}
    assert ref <= names, ref - names


def test_library_exports_every_declared_symbol(built):
    lib = built.lib()
    names = declared_functions()
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    # the ctypes signature table covers the whole header surface
    assert names <= set(built.SIGNATURES), names - set(built.SIGNATURES)


def test_nk_matches_reference_formula(built, oracle_lib):
    import numpy as np
    for Ng, L, dK in [(128, 1000.0, 2 * np.pi / 1000), (1024, 1000.0, 2 * np.pi / 1000),
                      (512, 2560.0, 0.005), (6, 10.0, 0.3)]:
        assert built.nk(Ng, L, dK) == oracle_lib.nk(Ng, L, dK)


def _have_ref_app(name):
    return os.path.exists(os.path.join(REF, "src", name)) and shutil.which("gcc")


@pytest.mark.parametrize("app", ["app/P.c", "app/Psb.c", "app/Pss.c", "app/DLsb.c", "app/DLss.c",
                                 "tests/octet.c"])
def test_reference_drivers_link_unchanged(built, tmp_path, app):
    """src/app/*.c and src/tests/octet.c compile against include/ and link
    against libfftgal_gb300.so.  `-I-` stops gcc from resolving the drivers'
    "../fft.h" next to the reference source, so "../fft.h" is found through
    include/io/ (include/io/../fft.h = include/fft.h)."""
    if not _have_ref_app(app):
        pytest.skip("reference sources not present")
    src = os.path.join(REF, "src", app)
    out = tmp_path / "a.out"
    cmd = ["gcc", "-O2", "-Wno-deprecated", "-iquote", os.path.join(INCLUDE, "io"), "-I-",
           f"-I{INCLUDE}", src, f"-L{os.path.dirname(built.LIBPATH)}", "-lfftgal_gb300",
           f"-Wl,-rpath,{os.path.dirname(built.LIBPATH)}", "-lm", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert out.exists()


def test_alias_features_definition():
    """fftgal_alias_features (host code) against its definition: k/k_Nyq,
    Pshot/den, P2/den, P4/den, d ln den / d ln k over the neighbouring bins
    with modes (one-sided at the ends, clamped to [-5, 5]); empty bins give
    zeros."""
    import numpy as np
    from fftgal_gb300 import alias_mlp as a
    rng = np.random.default_rng(1)
    NK = 12
    K = np.sort(rng.uniform(0.01, 0.5, NK))
    P = rng.normal(0, 50, (NK, 4))
    P[:, 0] = rng.uniform(10, 1000, NK)
    P[4] = np.nan  # an empty bin
    Pshot, kN = 20.0, 0.4
    X = a.features(K, P, Pshot, kN)
    ok = np.isfinite(P[:, 0])
    den = np.abs(P[:, 0]) + Pshot
    for b in range(NK):
        if not ok[b]:
            assert np.all(X[b] == 0)
            continue
        lo = b - 1
        while lo >= 0 and not ok[lo]:
            lo -= 1
        hi = b + 1
        while hi < NK and not ok[hi]:
            hi += 1
        lo = b if lo < 0 else lo
        hi = b if hi >= NK else hi
        slope = 0.0 if hi == lo else (np.log(den[hi]) - np.log(den[lo])) / (np.log(K[hi]) - np.log(K[lo]))
        want = [K[b] / kN, Pshot / den[b], P[b, 1] / den[b], P[b, 2] / den[b], np.clip(slope, -5, 5)]
        np.testing.assert_allclose(X[b], want, rtol=1e-6, atol=1e-7)


def test_alias_envelope_and_scaled_targets():
    """fftgal_alias_envelope is u^6 / (1 + u^6), and the trainer's targets are
    the raw ones over it, clipped to +-5."""
    import numpy as np
    from fftgal_gb300 import alias_mlp as a, lib
    for u in (0.0, 0.1, 0.5, 1.0, 1.7):
        assert abs(lib().fftgal_alias_envelope(u) - u ** 6 / (1 + u ** 6)) <= 1e-15
    X = np.zeros((3, a.IN), dtype=np.float32)
    X[:, 0] = [0.5, 1.0, 1.5]
    T = np.array([[1e-3, -1e-3, 0], [0.1, 0.2, -20], [100, 0, 0]], dtype=np.float32)
    S = a.scaled_targets(X, T)
    e = a.envelope(X[:, 0].astype(np.float64))
    np.testing.assert_allclose(S, np.clip(T / e[:, None], -5, 5), rtol=1e-6)
    assert S[1, 2] == -5 and S[2, 0] == 5


def declared_arities():
    out = {}
    for dirpath, _, files in os.walk(INCLUDE):
        for f in files:
            if not f.endswith(".h"):
                continue
            text = open(os.path.join(dirpath, f)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            text = re.sub(r"#define[^\n]*", "", text)
            for m in re.finditer(r"^[A-Za-z_][\w \t\*]*?\b([A-Za-z_]\w*)\s*\(([^;{}]*)\)\s*;", text, re.M):
                if m.group(0).lstrip().startswith("static"):
                    continue
                params = " ".join(m.group(2).split())
                out[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_ctypes_signatures_match_header_arities(built):
    """Every function the headers declare has as many arguments in the ctypes
    table (fftgal_gb300.SIGNATURES) as in its C prototype."""
    wrong = {n: (k, len(built.SIGNATURES[n][1])) for n, k in declared_arities().items()
             if n in built.SIGNATURES and len(built.SIGNATURES[n][1]) != k}
    assert not wrong, wrong
