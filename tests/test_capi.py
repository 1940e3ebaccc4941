"""The C-ABI boundary without a GPU: the shared library loads, exports every
function that include/*.h declares, and the reference's own drivers compile
and link unchanged against these headers and this library."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
REF = os.environ.get("FFTGAL_REFERENCE_DIR", "/root/reference")


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
