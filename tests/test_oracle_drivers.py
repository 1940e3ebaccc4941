"""The oracle's restatements of the drivers' own loops -- the sub-box and
sub-sphere window deconvolutions of src/app/Psb.c:74-84 and Pss.c:71-86
(og_window_box / og_window_sphere) and the super-sample DeltaL filters of
src/app/DLsb.c:41-99 and DLss.c (og_dl) -- replayed with the oracle on the
inputs of tests/golden/drivers_small.npz and compared with the tables the
reference's own drivers wrote there (tests/golden/make_drivers_golden.py):
the first redshift-space sub-volume's Pl and Pmu tables and all six lines of
sight of DeltaL, to the 7 significant digits the drivers print.  CPU only."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def drv():
    return np.load(os.path.join(GOLD, "drivers_small.npz"))


def _params(d):
    Ng, L, Nsub, alpha, dK, a = d["params"]
    return int(Ng), float(L), int(Nsub), float(dK)


@pytest.mark.parametrize("drv_name,kind", [("Psb", "box"), ("Pss", "sphere")])
def test_subvolume_window_against_driver(oracle_lib, drv, drv_name, kind):
    d = drv
    Ng, L, Nsub, dK = _params(d)
    Vsub = float(d[f"{drv_name}_sub_V"])
    x, y, z = d[f"{drv_name}_sub_pos"]
    xr, yr, zr = d[f"{drv_name}_sub_rand"]
    g = oracle_lib.Oracle(Ng, L)
    # the driver's sequence: fft_p2k with randoms -> P -> fft_k2x(0) -> window -> fft_x2k(0) -> Pl, Pmu
    g.p2k(x, y, z, Vsub, rand=(xr, yr, zr))
    g.power(len(x), Vsub, len(xr))
    g.k2x(0)
    getattr(g, "window_" + kind)(Ng // Nsub)
    g.x2k(0)
    los = (0.0, 0.0, 1.0)
    K, N, P, st, _ = g.pl(los, dK)
    ref = d[f"{drv_name}_pl"]
    got = np.column_stack([K, N, P])
    np.testing.assert_array_equal(got[:, 1], ref[:, 1])
    np.testing.assert_allclose(got, ref, rtol=6e-7, atol=1e-300, equal_nan=True)
    Km, Nm, Pm, st2, _ = g.pmu(los, dK, 3)
    refm = d[f"{drv_name}_pmu"]
    gotm = np.stack([Km, Nm, Pm], axis=2).reshape(len(Km), -1)
    np.testing.assert_array_equal(gotm[:, 1::3], refm[:, 1::3])
    np.testing.assert_allclose(gotm, refm, rtol=6e-7, atol=1e-300, equal_nan=True)


@pytest.mark.parametrize("drv_name,sphere", [("DLsb", 0), ("DLss", 1)])
def test_super_sample_modes_against_driver(oracle_lib, drv, drv_name, sphere):
    d = drv
    Ng, L, Nsub, dK = _params(d)
    x, y, z = d["catalog"]
    g = oracle_lib.Oracle(Ng, L)
    # the driver's field: fft_p2g (offset 1/2 in DLsb.c:58, 0 in DLss.c:56),
    # fft_x2k(0), no interlacing
    off = 0.0 if sphere else 0.5
    g.p2g(x, y, z, L ** 3, [off, off, off])
    g.x2k(0)
    fk = g.f.copy()
    for il, los in enumerate(d["los6"]):
        got = np.zeros((Nsub ** 3, 3))
        for iL in range(3):
            g.f[:] = fk
            got[:, iL] = g.dl(sphere, Nsub, los, iL)
        ref = d[f"{drv_name}_los{il}"]
        scale = np.abs(ref).max()
        np.testing.assert_allclose(got, ref, rtol=6e-7, atol=6e-7 * scale)
