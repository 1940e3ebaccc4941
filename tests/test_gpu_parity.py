"""Parity of the CUDA path (through the C ABI) with the FP64 oracle and the
reference's golden outputs.

Tolerances (stated per test):
  * FP64 grids   : grids and power sums to 1e-12 of the grid's scale; the
                   octet known answers to the reference's own eps = 1e-15.
  * FP32 grids   : grids to 2e-5 of their scale; P_l within 1e-4 of
                   (|P_0^oracle(k)| + Pshot) for k < 0.8 k_Nyq.
  * mode counts N: bit-exact in every mode; mean K per bin: 1e-12 relative.
"""
import os

import numpy as np
import pytest

from catalogs import uniform_box

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def fg():
    from fftgal_gb300 import build
    build.build()
    import fftgal_gb300
    return fftgal_gb300


@pytest.fixture(scope="module")
def small():
    return np.load(os.path.join(GOLD, "small_cases.npz"))


def parse_table(text):
    rows = [[float(t) for t in ln.split()] for ln in str(text).splitlines()
            if ln and not ln.startswith("#")]
    return np.array(rows)


def grid_close(got, want, rel):
    scale = max(np.abs(want).max(), 1e-300)
    err = np.abs(got - want).max() / scale
    assert err <= rel, f"max error {err:.3e} of scale {scale:.3e} > {rel}"


# ---------------------------------------------------------------------------
# src/tests/octet.c:8-62 through the C ABI
@pytest.mark.parametrize("prec,eps", [("f64", 1e-15), ("f32", 1e-5)])
def test_octet_known_answer(fg, prec, eps):
    """The reference's eps = 1e-15 holds for FP64 grids.  FP32 grids paint in
    fixed point with 2^-23 of a particle's weight per stencil cell and store
    FP32, hence 1e-5 at this test's normalisation (x8)."""
    g = fg.Grid(2, 2.0, precision=prec)
    cat = fg.Catalog([-8.0], [-8.0], [-8.0], 8.0)
    off = g.p2g(cat, [7.0, 7.0, 7.0])
    assert np.all(off == -1.0) and np.all(g.offset == -1.0)
    r = g.real
    for i in range(2):
        for j in range(2):
            for k in range(2):
                assert abs(r[i, j, k] - 8.0 / 27 * (i + 1) * (j + 1) * (k + 1)) < eps
    g.x2k(1)
    c = g.cplx
    for i in range(2):
        for j in range(2):
            assert abs(c[i, j, 0].real - 8.0 / (1 + 2 * i) / (1 + 2 * j)) < eps
            assert abs(c[i, j, 0].imag) < eps
    g.k2x(0)
    r = g.real
    for i in range(2):
        for j in range(2):
            for k in range(2):
                assert abs(r[i, j, k] - 64.0 / 27 / (i + 1) / (j + 1) / (k + 1)) < eps


# ---------------------------------------------------------------------------
@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("Ng", [2, 3, 4, 5, 6, 7, 8, 12, 16, 30, 32, 64, 96, 128])
def test_fft_matches_numpy(fg, prec, Ng):
    rng = np.random.default_rng(Ng)
    a = rng.standard_normal((Ng, Ng, Ng))
    g = fg.Grid(Ng, float(Ng), precision=prec)          # L = Ng -> H^3 = 1
    g.real[..., :Ng] = a
    g.x2k(0)
    ref = np.fft.rfftn(a)
    rel = 1e-13 if prec == "f64" else 2e-6
    grid_close(g.cplx, ref, rel)
    g.k2x(0)                                            # c2r / L^3 = identity
    grid_close(g.real[..., :Ng], a, rel)


# ---------------------------------------------------------------------------
@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("Ng", [2, 3, 4, 5, 6, 8, 12, 16])
def test_small_cases_match_reference(fg, oracle_lib, small, prec, Ng, tmp_path):
    key = f"ng{Ng}"
    L = float(small[key + "_L"])
    x, y, z = small[key + "_pos"]
    xr, yr, zr = small[key + "_rand"]
    V = L ** 3
    rel = 1e-12 if prec == "f64" else 2e-5
    g = fg.Grid(Ng, L, precision=prec)
    cat = fg.Catalog(x, y, z, V)
    off = g.p2g(cat, small[key + "_p2g_offset_in"])
    np.testing.assert_array_equal(off, small[key + "_p2g_offset_out"])
    grid_close(g.f, small[key + "_p2g"], rel)
    g.x2k(1)
    grid_close(g.f, small[key + "_x2k_phase"], rel)
    g.k2x(1)
    want = small[key + "_k2x_phase"].reshape(Ng, Ng, -1)[..., :Ng]
    grid_close(g.real[..., :Ng], want, rel)
    rcat = fg.Catalog(xr, yr, zr, V)
    catr = fg.Catalog(x, y, z, V, rand=rcat)
    g.p2g(catr, [0.0, 0.0, 0.0])
    grid_close(g.f, small[key + "_p2g_rand"], rel)
    g.p2k(cat)
    grid_close(g.f, small[key + "_p2k"], rel)
    g.power(cat)
    grid_close(g.f, small[key + "_P"], rel)
    # Pl/Pmu tables: counts exact, values against the oracle at full precision
    o = oracle_lib.Oracle(Ng, L)
    o.p2k(x, y, z, V)
    o.power(len(x), V)
    KF = 2 * np.pi / L
    Pshot = V / len(x)
    for il, los in enumerate(small["los_set"]):
        for idk, dK in enumerate((KF, 0.7 * KF, 2.5 * KF)):
            fpl, fmu = str(tmp_path / "pl.txt"), str(tmp_path / "pmu.txt")
            losh = g.pl(cat, los, dK, fpl)
            g.pmu(cat, los, dK, fmu)
            got = fg.read_table(fpl)
            gotm = fg.read_table(fmu)
            ref = parse_table(small[f"{key}_los{il}_dk{idk}_pl"])
            refm = parse_table(small[f"{key}_los{il}_dk{idk}_pmu"])
            # counts: bit-exact against the reference's own output
            np.testing.assert_array_equal(got[:, 1], ref[:, 1])
            np.testing.assert_array_equal(gotm[:, 1::3], refm[:, 1::3])
            # the text itself carries 7 significant digits
            K, N, P, st, losh_o = o.pl(los, dK)
            np.testing.assert_allclose(losh, losh_o, rtol=0, atol=0)
            np.testing.assert_allclose(got[:, 0], K, rtol=1e-6, equal_nan=True)
            den = np.abs(P[:, :1]) + Pshot
            ok = np.isfinite(P)
            assert np.all(np.isfinite(got[:, 2:]) == ok)
            Km, Nm, Pm, st2, _ = o.pmu(los, dK, 3)
            np.testing.assert_array_equal(gotm[:, 1::3], Nm)
            # FP64: every bin to 1e-6.  FP32: 1e-4 for k < 0.8 k_Nyq (the
            # stated parity range), 1e-3 everywhere (the window deconvolution
            # amplifies FP32 rounding ~200x in the corner of the cube)
            sel = np.broadcast_to((K < 0.8 * np.pi * Ng / L)[:, None], P.shape)
            for tol, mask in ([(1e-6, ok)] if prec == "f64" else [(1e-4, ok & sel), (1e-3, ok)]):
                assert np.all(np.abs(got[:, 2:] - P)[mask] <= (tol * np.broadcast_to(den, P.shape))[mask] + 1e-300)
                m2 = mask[:, :1].repeat(3, 1)
                assert np.all((np.abs(gotm[:, 2::3] - Pm) <= tol * (np.abs(Pm) + Pshot))[m2])


# ---------------------------------------------------------------------------
def _uniform_ng128():
    gold = np.load(os.path.join(GOLD, "uniform_ng128.npz"))
    L, Ng, n = float(gold["L"]), int(gold["Ng"]), int(gold["Np"])
    x, y, z = uniform_box(int(gold["seed"]), n, L)
    return gold, L, Ng, n, x, y, z


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_uniform_ng128_capi_matches_reference(fg, prec, tmp_path):
    """The uniform-box configuration (1e6 particles, Ng=128, interlaced)
    through the drop-in sequence fft_p2k -> P -> Pl -> Pmu, against the
    reference's own tables (tests/golden/uniform_ng128.npz)."""
    gold, L, Ng, n, x, y, z = _uniform_ng128()
    V = L ** 3
    Pshot = V / n
    g = fg.Grid(Ng, L, precision=prec, host_view="lazy")
    cat = fg.Catalog(x, y, z, V)
    g.p2k(cat)
    fk = g.exportf()
    kny = np.pi * Ng / L
    for il in range(4):
        g.importf(fk)
        g.power(cat)
        fpl, fmu = str(tmp_path / "pl.txt"), str(tmp_path / "pmu.txt")
        g.pl(cat, gold[f"los{il}"], 2 * np.pi / L, fpl)
        g.pmu(cat, gold[f"los{il}"], 2 * np.pi / L, fmu)
        got, gotm = fg.read_table(fpl), fg.read_table(fmu)
        ref, refm = parse_table(gold[f"los{il}_pl"]), parse_table(gold[f"los{il}_pmu"])
        np.testing.assert_array_equal(got[:, 1], ref[:, 1])
        np.testing.assert_array_equal(gotm[:, 1::3], refm[:, 1::3])
        np.testing.assert_allclose(got[:, 0], ref[:, 0], rtol=1e-6, equal_nan=True)
        sel = ref[:, 0] < 0.8 * kny
        den = np.abs(ref[sel, 2:3]) + Pshot
        err = np.abs(got[sel, 2:5] - ref[sel, 2:5]) / den
        assert err.max() <= 1e-4, err.max()
        errm = np.abs(gotm[sel][:, 2::3] - refm[sel][:, 2::3]) / (np.abs(refm[sel][:, 2::3]) + Pshot)
        assert errm.max() <= 1e-4, errm.max()


def test_uniform_ng128_fused_matches_reference(fg):
    """The fused single-call path (fftgal_power_f32) on the same catalog."""
    gold, L, Ng, n, x, y, z = _uniform_ng128()
    V = L ** 3
    Pshot = V / n
    g = fg.Grid(Ng, L, precision="f32", host_view="lazy")
    kny = np.pi * Ng / L
    for il in range(4):
        r = g.power_f32(x, y, z, V, gold[f"los{il}"], 2 * np.pi / L, Nmu=3)
        ref, refm = parse_table(gold[f"los{il}_pl"]), parse_table(gold[f"los{il}_pmu"])
        np.testing.assert_array_equal(r["N"], ref[:, 1])
        np.testing.assert_array_equal(r["Nmu"], refm[:, 1::3])
        sel = ref[:, 0] < 0.8 * kny
        den = np.abs(ref[sel, 2:3]) + Pshot
        # FP32 positions: the reference saw FP64 positions of the same points
        err = np.abs(r["P"][sel, :3] - ref[sel, 2:5]) / den
        assert err.max() <= 1e-4, err.max()


# ---------------------------------------------------------------------------
@pytest.mark.parametrize("Ng,Nmu", [(16, 3), (30, 10), (64, 10), (33, 4)])
def test_mode_counts_exact(fg, oracle_lib, small, Ng, Nmu):
    """N per k bin and per (k, mu) wedge are integers: they must equal the
    oracle's exactly for every line of sight and bin width."""
    L = 100.0
    x, y, z = uniform_box(7, 2000, L)
    V = L ** 3
    g = fg.Grid(Ng, L, precision="f32", host_view="lazy")
    o = oracle_lib.Oracle(Ng, L)
    o.p2k(x, y, z, V)
    o.power(len(x), V)
    KF = 2 * np.pi / L
    for los in small["los_set"]:
        for dK in (KF, 0.7 * KF, 2.5 * KF):
            r = g.power_f32(x, y, z, V, los, dK, Nmu=Nmu)
            K, N, P, st, _ = o.pl(los, dK)
            Km, Nm, Pm, st2, _ = o.pmu(los, dK, Nmu)
            np.testing.assert_array_equal(r["N"], N)
            np.testing.assert_array_equal(r["Nmu"], Nm)
            np.testing.assert_allclose(r["K"], K, rtol=1e-12, equal_nan=True)
            np.testing.assert_allclose(r["Kmu"], Km, rtol=1e-12)


@pytest.mark.parametrize("Ng", [64, 65, 66, 48])
def test_last_k_columns(fg, oracle_lib, Ng):
    """The finish + binning kernel bins the last one or two k columns mode by
    mode after its 16 x 16 x 32 blocks when they would fill a block of their
    own (Ng = 64: the Nyquist column; 65: the last column of an odd grid; 66:
    two columns) and not otherwise (48).  The fused call under the lazy view
    (finished field binned, not stored) and under the sync view (stored)
    against the FP64 oracle: the tables under the parity criterion, and the
    stored k-space grid within 1e-5 of its largest value."""
    import parity
    L, n = 200.0, 100_000
    x, y, z = (np.asarray(a, dtype=np.float32).astype(np.float64) for a in uniform_box(17, n, L))
    V, los, dK = L ** 3, (0.3, 0.5, 1.0), 2 * np.pi / L
    want = oracle_lib.power_spectrum(Ng, L, x, y, z, los, dK, Nmu=4)
    for view in ("lazy", "sync"):
        g = fg.Grid(Ng, L, precision="f32", host_view=view)
        got = g.power_f32(x, y, z, V, los, dK, Nmu=4)
        e = parity.errors(got, want, V / n, Ng, L)
        assert parity.passes(e), (view, e)
    o = oracle_lib.Oracle(Ng, L)
    o.p2k(x, y, z, V)
    grid_close(np.array(g.cplx), np.array(o.cplx), 1e-5)


def test_fp32_paint_is_bit_reproducible(fg):
    x, y, z = uniform_box(11, 200_000, 500.0)
    g = fg.Grid(64, 500.0, precision="f32", host_view="lazy")
    cat = fg.Catalog(x, y, z, 500.0 ** 3)
    g.p2g(cat, [0.5, 0.5, 0.5])
    a = g.exportf()
    g.p2g(cat, [0.5, 0.5, 0.5])
    b = g.exportf()
    assert a.tobytes() == b.tobytes()


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_g2p_reference_semantics(fg, oracle_lib, prec):
    """fft_g2p reproduces the reference (its last stencil term only,
    src/fft.c:165); fftgal_g2p_sum gives the full PCS interpolation."""
    Ng, L = 16, 80.0
    x, y, z = uniform_box(5, 300, L)
    V = L ** 3
    g = fg.Grid(Ng, L, precision=prec)
    cat = fg.Catalog(x, y, z, V)
    g.p2g(cat, [0.25, -0.5, 0.75])
    o = oracle_lib.Oracle(Ng, L)
    o.p2g(x, y, z, V, [0.25, -0.5, 0.75])
    got = g.g2p(cat)
    want = o.g2p(x, y, z)
    rel = 1e-12 if prec == "f64" else 2e-5
    grid_close(got, want, rel)
    full = g.g2p_sum(cat)
    assert np.all(np.isfinite(full)) and np.abs(full).max() > np.abs(got).max()


def test_sync_view_sees_host_writes(fg, oracle_lib):
    """Under the default host view, host writes to F() between calls are seen
    by the next call (the Psb.c / DLsb.c pattern, src/app/Psb.c:74-84)."""
    Ng, L = 8, 10.0
    rng = np.random.default_rng(2)
    a = rng.standard_normal((Ng, Ng, Ng))
    g = fg.Grid(Ng, L, precision="f64")
    g.real[..., :Ng] = a
    g.x2k(0)
    g.real[0, 0, 2] *= 3.0        # host edit in k space
    g.k2x(0)
    o = oracle_lib.Oracle(Ng, L)
    o.real[..., :Ng] = a
    o.x2k(0)
    o.real[0, 0, 2] *= 3.0
    o.k2x(0)
    grid_close(g.real[..., :Ng], o.real[..., :Ng], 1e-12)


# ---------------------------------------------------------------------------
@pytest.mark.parametrize("Ng", [256, 512, 1024])
def test_fft_large_matches_cufft(fg, Ng):
    """Large FP32 transforms against cuFFT in FP64 (torch.fft, a cross-check
    only): relative L2 error <= 1e-6 and largest error <= 1e-5 of the largest
    mode (FP32 rounding grows like log2 N)."""
    torch = pytest.importorskip("torch")
    Ngp = 2 * (Ng // 2 + 1)
    g = fg.Grid(Ng, float(Ng), precision="f32", host_view="lazy")   # H^3 = 1
    gen = torch.Generator(device="cuda").manual_seed(Ng)
    x = torch.randn((Ng, Ng, Ngp), generator=gen, device="cuda", dtype=torch.float32)
    g.copy_from(x.data_ptr())
    g.x2k(0)
    out = torch.empty_like(x)
    g.copy_to(out.data_ptr())
    got = torch.view_as_complex(out.view(Ng, Ng, Ngp // 2, 2))
    ref = torch.fft.rfftn(x[..., :Ng].double())
    diff = got.to(torch.complex128) - ref
    err_max = (diff.abs().max() / ref.abs().max()).item()
    err_l2 = (torch.linalg.vector_norm(diff) / torch.linalg.vector_norm(ref)).item()
    del ref, diff
    assert err_l2 <= 1e-6 and err_max <= 1e-5, (err_l2, err_max)
    g.k2x(0)                         # back: c2r / L^3 = identity
    g.copy_to(out.data_ptr())
    d = (out[..., :Ng] - x[..., :Ng]).double()
    back_l2 = (torch.linalg.vector_norm(d) / torch.linalg.vector_norm(x[..., :Ng].double())).item()
    back_max = (d.abs().max() / x.abs().max()).item()
    assert back_l2 <= 1e-6 and back_max <= 1e-5, (back_l2, back_max)


def _check_batch(fg, g, got, cats, V, los, dK, Nmu):
    for c, cat in enumerate(cats):
        want = g.power_f32(*cat, V[c], los, dK, Nmu=Nmu)
        np.testing.assert_array_equal(got[c]["N"], want["N"])
        np.testing.assert_array_equal(got[c]["Nmu"], want["Nmu"])
        den = np.abs(np.nan_to_num(want["P"][:, :1])) + V[c] / len(cat[0])
        ok = np.isfinite(want["P"])
        err = (np.abs(got[c]["P"] - want["P"]) / den)[ok]
        assert err.max() <= 1e-6, f"catalog {c}: {err.max():.2e}"
        errw = np.abs(got[c]["Pmu"] - want["Pmu"]) / den
        assert errw.max() <= 1e-6, f"catalog {c} wedges: {errw.max():.2e}"


@pytest.mark.parametrize("graphs", [True, False])
def test_batch_matches_single_calls(fg, graphs):
    """fftgal_power_batch_f32 (uploads on a second stream, two buffers; with
    graphs, one CUDA graph launch per catalog) gives each catalog's
    fftgal_power_f32 result: counts exact, P to 1e-6 of (|P_0| + Pshot)
    (binning sums FP32 run totals in FP64 in a varying order)."""
    Ng, L, Nmu = 64, 500.0, 4
    los, dK = (0.0, 0.6, 0.8), 2 * np.pi / L
    cats = [uniform_box(20 + c, n, L) for c, n in enumerate((40_000, 90_000, 25_000, 60_000, 5_000))]
    V = [L ** 3 * f for f in (1.0, 0.5, 2.0, 1.0, 3.0)]
    g = fg.Grid(Ng, L, precision="f32", host_view="lazy")
    g.set_graphs(graphs)
    got = g.power_batch_f32(cats, V, los, dK, Nmu=Nmu)
    _check_batch(fg, g, got, cats, V, los, dK, Nmu)


@pytest.mark.parametrize("Ng", [48, 96])
def test_graph_batch_with_the_general_fft(fg, Ng):
    """Grid sizes that are not powers of two take the mixed-radix FFT inside
    the captured graph: each catalog still matches its fftgal_power_f32."""
    L, Nmu = 400.0, 3
    los, dK = (0.0, 0.0, 1.0), 2 * np.pi / L
    cats = [uniform_box(300 + c, n, L) for c, n in enumerate((30_000, 12_000, 45_000))]
    V = [L ** 3] * len(cats)
    g = fg.Grid(Ng, L, precision="f32", host_view="lazy")
    got = g.power_batch_f32(cats, V, los, dK, Nmu=Nmu)
    _check_batch(fg, g, got, cats, V, los, dK, Nmu)


def test_batch_needs_fp32_grid(fg):
    g = fg.Grid(16, 100.0, precision="f64", host_view="lazy")
    with pytest.raises(RuntimeError):
        g.power_batch_f32([uniform_box(1, 1000, 100.0)], 100.0 ** 3, (0, 0, 1), 2 * np.pi / 100.0)


def test_graph_batches_recapture_and_reuse(fg):
    """Graph batches on one grid across calls: the same captured graphs for
    smaller catalogs, recapture for a larger catalog, other bins or another
    line of sight; a batch of one catalog; the sync host view refreshed with
    the last catalog's finished field as fftgal_power_f32 leaves it."""
    Ng, L = 32, 300.0
    dK = 2 * np.pi / L
    g = fg.Grid(Ng, L, precision="f32", host_view="lazy")
    calls = [((0, 0, 1), 3, (30_000, 20_000, 10_000)), ((0, 0, 1), 3, (5_000, 25_000)),
             ((0, 0, 1), 3, (70_000, 1_000, 50_000)), ((1, 1, 0), 10, (20_000,)), ((0, 0, 1), 4, (8_000, 9_000))]
    for q, (los, Nmu, sizes) in enumerate(calls):
        cats = [uniform_box(100 * q + c, n, L) for c, n in enumerate(sizes)]
        V = [L ** 3] * len(cats)
        got = g.power_batch_f32(cats, V, los, dK, Nmu=Nmu)
        _check_batch(fg, g, got, cats, V, los, dK, Nmu)
    gs = fg.Grid(Ng, L, precision="f32", host_view="sync")
    cats = [uniform_box(7, 12_000, L), uniform_box(8, 15_000, L)]
    gs.power_batch_f32(cats, L ** 3, (0, 0, 1), dK)
    f_batch = np.array(gs.f)
    gs.power_f32(*cats[1], L ** 3, (0, 0, 1), dK)
    np.testing.assert_allclose(f_batch, np.array(gs.f), rtol=0, atol=0)


@pytest.mark.parametrize("prec,Ng,Nsub", [("f64", 16, 2), ("f64", 24, 3), ("f64", 32, 4), ("f32", 16, 2),
                                          ("f32", 32, 2)])
@pytest.mark.parametrize("kind", ["box", "sphere"])
def test_window_deconvolution(fg, oracle_lib, prec, Ng, Nsub, kind):
    """fftgal_window_box / _sphere against the host loops of src/app/Psb.c:76-83
    and Pss.c:72-84 restated in the oracle, on a random real-space grid
    (including the sphere's twice-multiplied wrapped cells): FP64 grids bit
    for bit, FP32 grids to 1e-6 relative."""
    L, Ngsub = 100.0, Ng // Nsub
    r = np.random.default_rng(Ng * 10 + Nsub).standard_normal((Ng, Ng, 2 * (Ng // 2 + 1)))
    g = fg.Grid(Ng, L, precision=prec)
    g.real[:] = r
    getattr(g, "window_" + kind)(Ngsub)
    o = oracle_lib.Oracle(Ng, L)
    o.real[:] = r
    getattr(o, "window_" + kind)(Ngsub)
    got, want = np.array(g.real), np.array(o.real)
    assert not np.array_equal(want, r)
    if prec == "f64":
        np.testing.assert_array_equal(got, want)
    else:
        np.testing.assert_allclose(got, want, rtol=1e-6, atol=0)


@pytest.mark.parametrize("prec,Ng,Nsub", [("f64", 16, 2), ("f64", 24, 3), ("f32", 32, 4)])
@pytest.mark.parametrize("sphere", [0, 1])
def test_super_sample_modes(fg, oracle_lib, prec, Ng, Nsub, sphere):
    """fftgal_dl_sub against the loops of src/app/DLsb.c / DLss.c restated in
    the oracle (og_dl), on a painted uniform catalog, for two lines of sight:
    FP64 grids to 1e-10 and FP32 grids to 2e-5 of the largest |Delta|."""
    L = 200.0
    x, y, z = uniform_box(40 + Ng, 3000, L)
    V = L ** 3
    offset = [0.0, 0.0, 0.0] if sphere else [0.5, 0.5, 0.5]
    los_list = [(0.0, 0.0, 1.0), (1.0, 1.0, 0.0)]
    g = fg.Grid(Ng, L, precision=prec, host_view="lazy")
    cat = fg.Catalog(x, y, z, V)
    g.p2g(cat, offset)
    g.x2k(0)
    got = g.dl_sub(sphere, Nsub, los_list)
    want = np.zeros_like(got)
    o = oracle_lib.Oracle(Ng, L)
    for l, los in enumerate(los_list):
        for iL in range(3):
            o.p2g(x, y, z, V, offset)
            o.x2k(0)
            want[l, iL] = o.dl(sphere, Nsub, los, iL)
    tol = 1e-10 if prec == "f64" else 2e-5
    scale = np.abs(want).max()
    assert scale > 0
    err = np.abs(got - want).max() / scale
    assert err <= tol, f"max error {err:.2e} of {scale:.3e}"


@pytest.mark.parametrize("prec,rel", [("f64", 1e-12), ("f32", 2e-5)])
def test_empty_and_wrapped_catalogs(fg, oracle_lib, prec, rel):
    """Edge catalogs through fft_p2g (src/fft.c:57-131) against the oracle:
    no particles (NaN everywhere, as the reference's final scaling by
    1/nbar = inf gives), one particle at the origin, one on the upper
    box edge, and particles several boxes away on either side (the cell index
    wraps mod Ng), with and without a grid offset."""
    Ng, L = 16, 100.0
    V = L ** 3
    cases = [
        (np.zeros(0), np.zeros(0), np.zeros(0)),
        (np.array([0.0]), np.array([0.0]), np.array([0.0])),
        (np.array([L - 1e-9]), np.array([L * 0.5]), np.array([L - 1e-9])),
        (np.array([-0.3 * L, 2.7 * L, 0.01]), np.array([1.7 * L, -1.2 * L, 99.99]), np.array([2.5 * L, 0.5, -3.1 * L])),
    ]
    for x, y, z in cases:
        for offset in ([0.0, 0.0, 0.0], [0.5, 0.5, 0.5]):
            g = fg.Grid(Ng, L, precision=prec)
            off = g.p2g(fg.Catalog(x, y, z, V), offset)
            o = oracle_lib.Oracle(Ng, L)
            want_off = o.p2g(x, y, z, V, offset)
            np.testing.assert_array_equal(off, want_off)
            if len(x) == 0:  # the reference scales by 1/nbar = inf: NaN everywhere
                assert np.isnan(np.array(o.f)).all()
                assert np.isnan(np.array(g.f)).all()
            else:
                grid_close(np.array(g.f), np.array(o.f), rel)


@pytest.mark.parametrize("n_clump,edge,mass", [(8_000, 2e-3, 2e-6), (50_000, 1e-2, 1e-5), (400_000, 1e-3, 1e-6),
                                               (3_000_000, 1e-3, 1e-6)])
@pytest.mark.parametrize("Ng,centre", [(32, (41.3, 57.9, 12.2)), (64, (25.1, 57.9, 12.2))])
def test_dense_clump_fixed_point_scale(fg, oracle_lib, n_clump, edge, mass, Ng, centre):
    """A clump of n_clump particles inside one cell on top of 1e5 uniform ones.
    8000 and 5e4: the tile's 32-bit fixed-point sums keep 20 and 18 fraction
    bits (from the per-block count), where rounding the tiny products at the
    stencil's edge to the nearest step biases the edge cells by up to 0.06 %
    and 0.3 % of their own value (a restatement of the rounding in numpy gives
    those bounds); 4e5 and 3e6 would leave 15 and 12 bits, where the bias
    reaches several percent (10 % at 3e6), so the tile paints each grid into
    64-bit sums with 22 fraction bits.  At Ng = 64 a single-grid paint uses
    tiles of 32 i rows, whose 64-bit sums are painted one half at a time; the
    clump's stencil there straddles the two halves.  Against the FP64 oracle:
    the painted grid within 5e-6 of its largest cell, every cell above 1e-4
    of it within `edge` of its own value, the total within `mass`; the grid
    bit-reproducible; P_0,2,4 within the parity bound."""
    L = 100.0
    rng = np.random.default_rng(n_clump)
    xu, yu, zu = uniform_box(9, 100_000, L)
    c = np.array(centre)
    clump = [c[a] + rng.uniform(-0.5, 0.5, n_clump) * (L / Ng) for a in range(3)]
    x, y, z = (np.concatenate([u, v]).astype(np.float32).astype(np.float64) for u, v in zip((xu, yu, zu), clump))
    V = L ** 3
    g = fg.Grid(Ng, L, precision="f32", host_view="sync")
    cat = fg.Catalog(x, y, z, V)
    for offset in ([0.0, 0.0, 0.0], [0.5, 0.5, 0.5]):
        g.p2g(cat, offset)
        a = np.array(g.real[..., :Ng], dtype=np.float64)
        o = oracle_lib.Oracle(Ng, L)
        o.p2g(x, y, z, V, offset)
        b = np.array(o.real[..., :Ng])
        grid_close(a, b, 5e-6)
        big = np.abs(b) > 1e-4 * np.abs(b).max()
        rel = np.abs(a - b)[big] / np.abs(b)[big]
        assert rel.max() <= edge, f"offset {offset}: cell error {rel.max():.2e}"
        assert abs(a.sum() - b.sum()) <= mass * b.sum()
        g.p2g(cat, offset)
        assert a.tobytes() == np.array(g.real[..., :Ng], dtype=np.float64).tobytes()
    los, dK = (0.0, 0.0, 1.0), 2 * np.pi / L
    got = g.power_f32(x, y, z, V, los, dK, Nmu=3)
    want = oracle_lib.power_spectrum(Ng, L, x, y, z, los, dK, Nmu=3)
    import parity
    e = parity.errors(got, want, V / len(x), Ng, L)
    assert parity.passes(e), e
