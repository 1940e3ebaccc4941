"""The CPU oracle pinned against the reference: the known-answer test of
src/tests/octet.c, numpy's FFT, and golden outputs of the reference's own
code (tests/golden/*.npz, written by tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

from catalogs import uniform_box

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def parse_table(text):
    rows = [[float(t) for t in ln.split()] for ln in str(text).splitlines()
            if ln and not ln.startswith("#")]
    return np.array(rows)


def header(text):
    return [ln for ln in str(text).splitlines() if ln.startswith("#")]


def test_octet_known_answer(oracle_lib):
    """src/tests/octet.c:8-62 -- Ng=2, L=2, one particle at -8 with offset 7."""
    g = oracle_lib.Oracle(2, 2.0)
    off = g.p2g([-8.0], [-8.0], [-8.0], 8.0, [7.0, 7.0, 7.0])
    assert np.all(off == -1.0)                       # remainder(7, 2) = -1
    eps = 1e-15
    r = g.real
    for i in range(2):
        for j in range(2):
            for k in range(2):
                assert abs(r[i, j, k] - 8.0 / 27 * (i + 1) * (j + 1) * (k + 1)) < eps
    g.x2k(1)
    c = g.cplx
    for i in range(2):
        for j in range(2):
            for k in range(1):   # octet.c:37 checks k < Ng/2 only
                assert abs(c[i, j, k].real - 8.0 / (1 + 2 * i) / (1 + 2 * j) / (1 + 2 * k)) < eps
                assert abs(c[i, j, k].imag) < eps
    g.k2x(0)
    r = g.real
    for i in range(2):
        for j in range(2):
            for k in range(2):
                assert abs(r[i, j, k] - 64.0 / 27 / (i + 1) / (j + 1) / (k + 1)) < eps


@pytest.mark.parametrize("Ng", [2, 3, 4, 5, 6, 7, 8, 9, 10, 12, 16, 18, 20, 24, 30, 32])
def test_fft_matches_numpy(oracle_lib, Ng):
    rng = np.random.default_rng(Ng)
    a = rng.standard_normal((Ng, Ng, Ng))
    g = oracle_lib.Oracle(Ng, float(Ng))          # L = Ng -> H^3 = 1
    g.real[..., :Ng] = a
    g.x2k(0)
    ref = np.fft.rfftn(a)
    assert np.abs(g.cplx - ref).max() <= 1e-13 * np.abs(ref).max()
    g.k2x(0)                                       # c2r / L^3 = identity
    assert np.abs(g.real[..., :Ng] - a).max() <= 1e-13 * np.abs(a).max()


def test_c2r_ignores_imag_of_self_conjugate_modes(oracle_lib):
    """FFTW's c2r discards Im X[0] and Im X[N/2] along the last axis."""
    Ng = 8
    rng = np.random.default_rng(3)
    a = rng.standard_normal((Ng, Ng, Ng))
    g = oracle_lib.Oracle(Ng, float(Ng))
    g.real[..., :Ng] = a
    g.x2k(0)
    g.real[..., 1] += 5.0                      # Im of k=0 plane
    g.real[..., Ng + 1] -= 3.0                 # Im of k=Ng/2 plane
    g.k2x(0)
    ref = np.fft.irfftn(np.fft.rfftn(a), s=(Ng, Ng, Ng), axes=(0, 1, 2))
    assert np.abs(g.real[..., :Ng] - ref).max() < 1e-12


@pytest.fixture(scope="module")
def small():
    return np.load(os.path.join(GOLD, "small_cases.npz"))


@pytest.mark.parametrize("Ng", [2, 3, 4, 5, 6, 8, 12, 16])
def test_oracle_matches_reference_small(oracle_lib, small, Ng):
    key = f"ng{Ng}"
    L = float(small[key + "_L"])
    x, y, z = small[key + "_pos"]
    xr, yr, zr = small[key + "_rand"]
    V = L ** 3
    g = oracle_lib.Oracle(Ng, L)
    off = g.p2g(x, y, z, V, small[key + "_p2g_offset_in"])
    np.testing.assert_array_equal(off, small[key + "_p2g_offset_out"])
    np.testing.assert_array_equal(g.f, small[key + "_p2g"])
    g.x2k(1)
    np.testing.assert_array_equal(g.f, small[key + "_x2k_phase"])
    g.k2x(1)
    np.testing.assert_array_equal(g.f, small[key + "_k2x_phase"])
    g.p2g(x, y, z, V, [0, 0, 0], rand=(xr, yr, zr))
    np.testing.assert_array_equal(g.f, small[key + "_p2g_rand"])
    g.p2k(x, y, z, V)
    np.testing.assert_array_equal(g.f, small[key + "_p2k"])
    g.power(len(x), V)
    np.testing.assert_array_equal(g.f, small[key + "_P"])
    KF = 2 * np.pi / L
    for il, los in enumerate(small["los_set"]):
        for idk, dK in enumerate((KF, 0.7 * KF, 2.5 * KF)):
            K, N, P, st, losh = g.pl(los, dK)
            ref = parse_table(small[f"{key}_los{il}_dk{idk}_pl"])
            got = np.column_stack([K, N, P])
            # the reference prints 7 significant digits; counts are exact
            np.testing.assert_array_equal(got[:, 1], ref[:, 1])
            np.testing.assert_allclose(got, ref, rtol=6e-7, atol=1e-300, equal_nan=True)
            Km, Nm, Pm, st2, _ = g.pmu(los, dK, 3)
            refm = parse_table(small[f"{key}_los{il}_dk{idk}_pmu"])
            gotm = np.stack([Km, Nm, Pm], axis=2).reshape(len(Km), -1)
            np.testing.assert_array_equal(gotm[:, 1::3], refm[:, 1::3])
            np.testing.assert_allclose(gotm, refm, rtol=6e-7, atol=1e-300, equal_nan=True)


def test_oracle_matches_reference_uniform_ng128(oracle_lib):
    gold = np.load(os.path.join(GOLD, "uniform_ng128.npz"))
    L, Ng, n = float(gold["L"]), int(gold["Ng"]), int(gold["Np"])
    x, y, z = uniform_box(int(gold["seed"]), n, L)
    g = oracle_lib.Oracle(Ng, L)
    g.p2k(x, y, z, L ** 3)
    fk = g.f.copy()
    np.testing.assert_allclose([fk.sum(), np.abs(fk).sum(), (fk * fk).sum()],
                               gold["fk_checksum"], rtol=1e-13)
    for il in range(4):
        g.f[:] = fk
        g.power(n, L ** 3)
        K, N, P, st, _ = g.pl(gold[f"los{il}"], 2 * np.pi / L)
        assert st == 0
        ref = parse_table(gold[f"los{il}_pl"])
        np.testing.assert_array_equal(N, ref[:, 1])
        np.testing.assert_allclose(np.column_stack([K, N, P]), ref, rtol=6e-7,
                                   atol=1e-300, equal_nan=True)
        Km, Nm, Pm, st2, _ = g.pmu(gold[f"los{il}"], 2 * np.pi / L)
        refm = parse_table(gold[f"los{il}_pmu"])
        np.testing.assert_array_equal(Nm, refm[:, 1::3])
        np.testing.assert_allclose(np.stack([Km, Nm, Pm], 2).reshape(len(Km), -1), refm,
                                   rtol=6e-7, atol=1e-300, equal_nan=True)


def test_rsd_and_wrap_against_reference_fixture(oracle_lib):
    """The oracle's gal_rsd and gal_wrap (oracle/fftgal_oracle.c) against the
    reference's own src/gal.c:51-77 outputs (tests/golden/gal_rsd_wrap.npz,
    written by tests/golden/make_golden.py from the compiled reference): bit
    for bit, including a line of sight that is not a unit vector and
    particles spread over three box lengths."""
    d = np.load(os.path.join(GOLD, "gal_rsd_wrap.npz"))
    x, y, z = d["pos"]
    vx, vy, vz = d["vel"]
    for il, los in enumerate(d["los_set"]):
        for ia, aH in enumerate(d["aH_set"]):
            got = np.stack(oracle_lib.Oracle.rsd(x, y, z, vx, vy, vz, los, float(aH)))
            np.testing.assert_array_equal(got, d[f"rsd_los{il}_ah{ia}"])
    got = np.stack(oracle_lib.Oracle.wrap(x, y, z, float(d["L"])))
    np.testing.assert_array_equal(got, d["wrap"])


def test_headline_tables_consistent():
    """tests/golden/headline_ng1024.npz: the reference's printed Pl/Pmu tables
    (src/power.c:80-98,157-175) and the oracle's full-precision binning of the
    same reference k-space grid agree -- counts exactly, values to the 7
    printed digits -- for both catalogs and every stored line of sight; every
    mode is counted once (sum N = Ng^3 - 1, src/power.c:76)."""
    import os
    from oracle.reflib import read_table
    import tempfile
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "headline_ng1024.npz"))
    Ng = int(z["Ng"])
    for name in ("uniform", "clustered"):
        for il in range(len(z["los_set"])):
            k = f"{name}_los{il}"
            with tempfile.TemporaryDirectory() as d:
                pa, pb = os.path.join(d, "pl"), os.path.join(d, "pmu")
                open(pa, "w").write(str(z[k + "_pl_text"]))
                open(pb, "w").write(str(z[k + "_pmu_text"]))
                a, b = read_table(pa), read_table(pb)
            assert np.array_equal(a[:, 1].astype(np.int64), z[k + "_N"])
            assert int(z[k + "_N"].sum()) == Ng ** 3 - 1
            np.testing.assert_allclose(a[:, 0], z[k + "_K"], rtol=1e-6)
            ok = np.isfinite(a[:, 2:])
            np.testing.assert_allclose(a[:, 2:][ok], z[k + "_P"][ok], rtol=1e-6, atol=1e-12)
            for m in range(3):
                assert np.array_equal(b[:, 3 * m + 1].astype(np.int64), z[k + "_mu3_N"][:, m])
            assert np.array_equal(z[k + "_mu10_N"].sum(axis=1), z[k + "_N"])
