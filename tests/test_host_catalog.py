"""The library's own host catalog functions (fftgal_gb300/csrc/gal.c, qpm.c),
called through libfftgal_gb300.so without a GPU:

* gal_rsd and gal_wrap against the reference's outputs stored in
  tests/golden/gal_rsd_wrap.npz (src/gal.c:51-77), bit for bit;
* gal_subbox and gal_subsphere (src/gal.c:80-159): the selected particles,
  their order and the volume bit for bit against the reference build
  (oracle/_ref, where the reference sources were available), and the number
  of randoms, lround(Npsub / alpha); the randoms themselves come from a
  different generator (splitmix64 instead of GSL's) and are checked to lie
  inside the sub-volume;
* gal_loadqpm_cubic (src/io/qpm.c:9-34) on a synthetic file in the QPM text
  format, against numpy's parse of the same text and the reference build.
"""
import ctypes as C
import os

import numpy as np
import pytest

from catalogs import uniform_box

HERE = os.path.dirname(os.path.abspath(__file__))
_dp = C.POINTER(C.c_double)


@pytest.fixture(scope="module")
def fg():
    from fftgal_gb300 import build
    build.build()
    import fftgal_gb300
    return fftgal_gb300


def _arrays(p, names=("x", "y", "z")):
    g = p.contents
    n = g.Np
    return [np.ctypeslib.as_array(getattr(g, a), shape=(max(n, 1),))[:n].copy() for a in names]


def test_gal_rsd_matches_reference(fg):
    z = np.load(os.path.join(HERE, "golden", "gal_rsd_wrap.npz"))
    x, y, zz = z["pos"]
    vx, vy, vz = z["vel"]
    L = float(z["L"])
    lib = fg.lib()
    for il, los in enumerate(z["los_set"]):
        for ia, aH in enumerate(z["aH_set"]):
            cat = fg.Catalog(x, y, zz, L ** 3, vel=(vx, vy, vz))
            l = np.array(los, dtype=np.float64)  # normalised in place, as the reference does
            d = lib.gal_rsd(cat.p, l.ctypes.data_as(_dp), float(aH))
            got = np.stack(_arrays(d))
            lib.gal_free(d)
            want = z[f"rsd_los{il}_ah{ia}"]
            assert got.tobytes() == want.tobytes(), (il, ia)
            np.testing.assert_array_equal(l, np.asarray(los) / np.sqrt(np.sum(np.square(los))))


def test_gal_wrap_matches_reference(fg):
    z = np.load(os.path.join(HERE, "golden", "gal_rsd_wrap.npz"))
    x, y, zz = z["pos"]
    L = float(z["L"])
    cat = fg.Catalog(x, y, zz, L ** 3)
    fg.lib().gal_wrap(cat.p, L)
    assert np.stack(_arrays(cat.p)).tobytes() == z["wrap"].tobytes()


def _ref():
    from oracle import reflib
    if not reflib.available():
        pytest.skip("the reference build (oracle/_ref) is not present")
    return reflib


@pytest.mark.parametrize("shape", ["box", "sphere"])
def test_gal_subvolume_selection(fg, shape):
    reflib = _ref()
    L, n, alpha = 200.0, 20_000, 0.3
    x, y, z = uniform_box(21, n, 1.5 * L, lo=-0.25 * L)  # some positions outside [0, L)
    if shape == "box":
        # wraps around the periodic edge along x and z
        region = np.array([170.0, 30.0, 20.0, 90.0, -15.0, 25.0, L])
    else:
        region = np.array([190.0, 100.0, 5.0, 40.0, L])
    ours = fg.Catalog(x, y, z, L ** 3)
    ref = reflib.RefGal(x, y, z, L ** 3)
    lib, rlib = fg.lib(), reflib.RefLib.lib()
    fn, rfn = (lib.gal_subbox, rlib.gal_subbox) if shape == "box" else (lib.gal_subsphere, rlib.gal_subsphere)
    a = fn(ours.p, region.copy().ctypes.data_as(_dp), alpha)
    b = rfn(ref.p, region.copy().ctypes.data_as(_dp), alpha)
    try:
        ga, gb = a.contents, b.contents
        assert ga.Np == gb.Np > 100
        assert ga.V == gb.V
        assert np.stack(_arrays(a)).tobytes() == np.stack(_arrays(b)).tobytes()
        ra, rb = ga.rand.contents, gb.rand.contents
        assert ra.Np == rb.Np == round(ga.Np / alpha)
        rx, ry, rz = _arrays(ga.rand)
        if shape == "box":
            x0, x1, y0, y1, z0, z1 = region[:6]
            for v, lo, hi in ((rx, x0, x1), (ry, y0, y1), (rz, z0, z1)):
                width = (hi - lo) % L
                assert np.all(v >= lo) and np.all(v < lo + width)
        else:
            c, R = region[:3], region[3]
            d = [(v - c[q] + L / 2) % L - L / 2 for q, v in enumerate((rx, ry, rz))]
            assert np.all(d[0] ** 2 + d[1] ** 2 + d[2] ** 2 < R * R)
    finally:
        lib.gal_free(a)
        rlib.gal_free(b)


def _qpm_text(n, seed=3):
    rng = np.random.default_rng(seed)
    pos = rng.random((n, 3)) * 1000.0
    vel = rng.standard_normal((n, 3)) * 300.0
    mass = rng.random(n) * 1e13
    ids = rng.integers(0, 10 ** 6, (n, 2))
    lines = [f"{p[0]:.6f} {p[1]:.6f} {p[2]:.6f} {v[0]:.4f} {v[1]:.4f} {v[2]:.4f} {m:.5e} {i[0]} {i[1]}\n"
             for p, v, m, i in zip(pos, vel, mass, ids)]
    return "".join(lines)


def test_loadqpm_cubic(fg, tmp_path):
    path = tmp_path / "mock.dat"
    path.write_text(_qpm_text(3000))
    want = np.loadtxt(path, usecols=(0, 1, 2, 3, 4, 5))
    L = 1000.0
    p = fg.lib().gal_loadqpm_cubic(str(path).encode(), L)
    try:
        g = p.contents
        assert g.Np == 3000 and g.V == L ** 3
        got = np.stack(_arrays(p, ("x", "y", "z", "vx", "vy", "vz")), axis=1)
        assert got.tobytes() == want.tobytes()
    finally:
        # the loader's velocity arrays are freed by gal_free, as in the reference
        fg.lib().gal_free(p)
    try:
        reflib = _ref()
    except pytest.skip.Exception:
        return
    q = reflib.RefLib.lib().gal_loadqpm_cubic(str(path).encode(), L)
    ref = np.stack(_arrays(q, ("x", "y", "z", "vx", "vy", "vz")), axis=1)
    assert ref.tobytes() == want.tobytes()
