"""Plan file of the autotuner (csrc/plan.cu), host side: entries keyed by
(compute capability, SM count, Ng, precision), replaced in place, other lines
kept, missing files and malformed lines ignored.  No GPU calls."""
import ctypes as C

import numpy as np


def _lookup(lib, path, key):
    t = (C.c_int * 3)()
    r = lib.fftgal_plan_lookup(str(path).encode(), *key, t)
    return r, list(t)


def _store(lib, path, key, tune, ms=(1.0, 2.0, 3.0), dev=b"test device"):
    t = (C.c_int * 3)(*tune)
    m = np.array(ms, dtype=np.float64)
    return lib.fftgal_plan_store(str(path).encode(), *key, t, m.ctypes.data_as(C.POINTER(C.c_double)), dev)


def test_plan_file_round_trip(tmp_path):
    from fftgal_gb300 import lib
    L = lib()
    path = tmp_path / "plan.txt"
    assert _lookup(L, path, (103, 152, 1024, 4))[0] == 0  # no file: not found
    assert _store(L, path, (103, 152, 1024, 4), (4, 3, 4)) == 0
    assert _store(L, path, (103, 152, 512, 4), (8, 3, 3)) == 0
    assert _lookup(L, path, (103, 152, 1024, 4)) == (1, [4, 3, 4])
    assert _lookup(L, path, (103, 152, 512, 4)) == (1, [8, 3, 3])
    for other in ((100, 152, 1024, 4), (103, 148, 1024, 4), (103, 152, 256, 4), (103, 152, 1024, 8)):
        assert _lookup(L, path, other)[0] == 0, other
    # replacing an entry keeps one line per key and the other entries
    assert _store(L, path, (103, 152, 1024, 4), (2, 2, 5)) == 0
    lines = path.read_text().splitlines()
    assert sum("Ng=1024" in l for l in lines) == 1 and sum("Ng=512" in l for l in lines) == 1
    assert _lookup(L, path, (103, 152, 1024, 4)) == (1, [2, 2, 5])
    assert "dev=test device" in lines[-1] and "ms=1.000,2.000,3.000" in lines[-1]


def test_plan_file_keeps_foreign_lines(tmp_path):
    from fftgal_gb300 import lib
    L = lib()
    path = tmp_path / "wisdom"
    path.write_text("# comment\n(fftw-3.3.10 fftw_wisdom)\nfftgal_gb300-plan 1 cc=103 sms=152 Ng=64 garbage\n")
    assert _lookup(L, path, (103, 152, 64, 4))[0] == 0  # malformed entry ignored
    assert _store(L, path, (103, 152, 64, 4), (4, 2, 2)) == 0
    text = path.read_text()
    assert text.startswith("# comment\n(fftw-3.3.10 fftw_wisdom)\n")
    assert _lookup(L, path, (103, 152, 64, 4)) == (1, [4, 2, 2])
    assert not list(tmp_path.glob("wisdom.tmp*"))


def test_plan_store_unwritable_reports_io_error(tmp_path):
    from fftgal_gb300 import lib
    L = lib()
    path = tmp_path / "no_such_dir" / "plan.txt"
    assert _store(L, path, (103, 152, 64, 4), (4, 2, 2)) == -7
    assert b"plan file" in L.fftgal_last_error()
