"""Autotuner and plan cache (csrc/plan.cu, fft2_autotune): fft_init with a
plan file measures once, imports afterwards, reuses in-process measurements,
re-measures an entry that does not fit, and every launch shape gives a
k-space grid bit-identical to the built-in plans' (the counterpart of
FFTW_MEASURE vs FFTW_ESTIMATE, src/fft.c:26-45)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

L_BOX = 1000.0


@pytest.fixture(scope="module")
def fg():
    from fftgal_gb300 import build
    build.build()
    import fftgal_gb300
    return fftgal_gb300


def _kgrid(fg, Ng, wisdom, seed=3, Np=200000):
    rng = np.random.default_rng(seed)
    x, y, z = (rng.uniform(0, L_BOX, Np) for _ in range(3))
    g = fg.Grid(Ng, L_BOX, wisdom=str(wisdom), precision="f32", host_view="sync")
    cat = fg.Catalog(x, y, z, V=L_BOX ** 3)
    g.p2k(cat)
    return g, g.f.copy()


def _entries(path):
    return [l for l in path.read_text().splitlines() if l.startswith("fftgal_gb300-plan 1 ")]


def test_measure_then_import(fg, tmp_path):
    path = tmp_path / "plan"
    g, f_tuned = _kgrid(fg, 64, path)
    info = g.plan_info()
    assert info["source"] == fg.PLAN_MEASURED
    assert np.all(info["ms"] > 0)
    lib = fg.lib()
    for w in range(3):
        assert lib.fftgal_plan_valid(64, w, info["tune"][w]) == 1
    (line,) = _entries(path)
    assert "Ng=64 prec=4" in line
    g2, f_imported = _kgrid(fg, 64, path)
    assert g2.plan_info()["source"] == fg.PLAN_FILE and g2.plan_info()["tune"] == info["tune"]
    _, f_est = _kgrid(fg, 64, "FFTW_ESTIMATE")
    np.testing.assert_array_equal(f_tuned, f_est)
    np.testing.assert_array_equal(f_imported, f_est)
    # a new file in the same process: the measurement is reused, then exported
    path2 = tmp_path / "plan2"
    g3, _ = _kgrid(fg, 64, path2)
    assert g3.plan_info()["source"] == fg.PLAN_CACHE and g3.plan_info()["tune"] == info["tune"]
    assert len(_entries(path2)) == 1


@pytest.mark.parametrize("Ng", [128, 256])
def test_every_valid_shape_is_bit_identical(fg, tmp_path, Ng):
    """Entries with the smallest and the largest valid shape of every pass."""
    lib = fg.lib()
    _, f_est = _kgrid(fg, Ng, "FFTW_ESTIMATE")
    ks = [r for r in (1, 2, 4, 8, 16, 32, 64) if lib.fftgal_plan_valid(Ng, 0, r)]
    cs = {w: [c for c in range(6) if lib.fftgal_plan_valid(Ng, w, c)] for w in (1, 2)}
    assert len(ks) >= 2 and len(cs[1]) >= 2 and len(cs[2]) >= 2
    import torch
    cc = "%d%d" % torch.cuda.get_device_capability()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    for pick in (0, -1):
        tune = [ks[pick], cs[1][pick], cs[2][pick]]
        path = tmp_path / f"plan{pick}"
        path.write_text(f"fftgal_gb300-plan 1 cc={cc} sms={sms} Ng={Ng} prec=4 kR={tune[0]} "
                        f"jlogC={tune[1]} ilogC={tune[2]} ms=0,0,0 dev=hand written\n")
        g, f = _kgrid(fg, Ng, path)
        assert g.plan_info()["source"] == fg.PLAN_FILE and g.plan_info()["tune"] == tune
        np.testing.assert_array_equal(f, f_est)


def test_entry_that_does_not_fit_is_measured_again(fg, tmp_path):
    import torch
    cc = "%d%d" % torch.cuda.get_device_capability()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    path = tmp_path / "plan"
    path.write_text(f"fftgal_gb300-plan 1 cc={cc} sms={sms} Ng=32 prec=4 kR=3 jlogC=9 ilogC=2 ms=0,0,0 dev=x\n")
    g, f = _kgrid(fg, 32, path)
    info = g.plan_info()
    assert info["source"] in (fg.PLAN_MEASURED, fg.PLAN_CACHE)
    lib = fg.lib()
    for w in range(3):
        assert lib.fftgal_plan_valid(32, w, info["tune"][w]) == 1
    (line,) = _entries(path)
    assert "kR=3 " not in line
    _, f_est = _kgrid(fg, 32, "FFTW_ESTIMATE")
    np.testing.assert_array_equal(f, f_est)


def test_fp64_and_untunable_sizes_use_builtin_plans(fg, tmp_path):
    path = tmp_path / "plan"
    g = fg.Grid(48, L_BOX, wisdom=str(path), precision="f32")
    assert g.plan_info()["source"] == fg.PLAN_BUILTIN
    g = fg.Grid(64, L_BOX, wisdom=str(path), precision="f64")
    assert g.plan_info()["source"] == fg.PLAN_BUILTIN
    assert not path.exists()


def test_unwritable_plan_file_is_not_fatal(fg, tmp_path):
    """A plan file in a directory that does not exist cannot be written: the
    grid is still made, with the measured shapes, and nothing is created."""
    path = tmp_path / "no_such_dir" / "plan"
    _, f = _kgrid(fg, 32, path)
    _, f_est = _kgrid(fg, 32, "FFTW_ESTIMATE")
    np.testing.assert_array_equal(f, f_est)
    assert not path.exists()


_TMA_CHILD = r"""
import sys, torch
sys.path.insert(0, sys.argv[1])
import fftgal_gb300 as fg
Ng = int(sys.argv[2])
Ngp = 2 * (Ng // 2 + 1)
g = fg.Grid(Ng, float(Ng), precision="f32", host_view="lazy")
gen = torch.Generator(device="cuda").manual_seed(Ng)
x0 = torch.randn((Ng, Ng, Ngp), generator=gen, device="cuda", dtype=torch.float32)
x = x0.clone()
w = (torch.arange(x.numel(), device="cuda", dtype=torch.int64) % 1000003) + 1
def digest(t):
    b = t.view(torch.int32).reshape(-1).to(torch.int64)
    return [int(b.sum()), int((b * w).sum()), int((b ^ (w * 2654435761)).sum())]
g.copy_from(x.data_ptr())
g.x2k(0)
g.copy_to(x.data_ptr())
k = digest(x)
got = torch.view_as_complex(x.view(Ng, Ng, Ngp // 2, 2)).to(torch.complex128)
ref = torch.fft.rfftn(x0[..., :Ng].double())
fwd = float(torch.linalg.vector_norm(got - ref) / torch.linalg.vector_norm(ref))
del got, ref
g.k2x(0)
g.copy_to(x.data_ptr())
back = float(torch.linalg.vector_norm((x - x0)[..., :Ng].double()) / torch.linalg.vector_norm(x0[..., :Ng].double()))
print(k + digest(x), fwd, back)
"""


@pytest.mark.parametrize("Ng", [512, 1024])
def test_tma_i_pass(fg, tmp_path, Ng):
    """The TMA-staged i pass (FFTGAL_TMA=1): forward and backward transforms
    within the FP32 bounds of the cuFFT cross-check (relative L2 error <= 1e-6
    against torch.fft in FP64, and of the round trip); at Ng = 512 (columns
    split 32 x 16 like the register-staged kernel) the grids are bit-identical
    to a run without it, at Ng = 1024 (even and odd rows, two 512-point
    transforms) the decomposition differs, so only the bounds apply."""
    import ast
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    outs = {}
    for tma in ("1", "0"):
        env = dict(os.environ, FFTGAL_TMA=tma, FFTGAL_QUIET="1")
        r = subprocess.run([sys.executable, "-c", _TMA_CHILD, root, str(Ng)], env=env,
                           capture_output=True, text=True, timeout=900)
        assert r.returncode == 0, r.stderr[-2000:]
        line = r.stdout.strip().splitlines()[-1]
        head, fwd, back = line.rsplit(" ", 2)
        outs[tma] = (ast.literal_eval(head), float(fwd), float(back))
    for tma in ("1", "0"):
        assert outs[tma][1] <= 1e-6 and outs[tma][2] <= 1e-6, (tma, outs[tma])
    if Ng == 512:
        assert outs["1"][0] == outs["0"][0]


def test_launch_shapes_measured_and_imported(fg, tmp_path):
    """fft_init with a plan file also settles the tile paint's and the
    binning's launch shapes: measured (or taken from this process's earlier
    measurement) and written on a launch line of the file, imported from it by
    the next grid; the spectra equal the built-in shapes' up to the grouping
    of the binning's FP32 per-CTA sums, which follows the CTA count: 1e-6 of
    |P_0| + Pshot."""
    path = tmp_path / "plan"
    Ng = 128
    g = fg.Grid(Ng, L_BOX, wisdom=str(path), precision="f32", host_view="lazy")
    a = g.launch_shapes()
    assert a["source"] in (fg.PLAN_MEASURED, fg.PLAN_CACHE)
    assert a["paint_cta"] in (1, 2) and a["bin_cta"] in (1, 2, 3) and a["bin_fold"] in (0, 8, 32)
    lines = [l for l in path.read_text().splitlines() if l.startswith("fftgal_gb300-launch 1 ")]
    assert len(lines) == 1 and f" Ng={Ng} " in lines[0]
    assert len(_entries(path)) == 1  # the FFT plan line is still there
    h = fg.Grid(Ng, L_BOX, wisdom=str(path), precision="f32", host_view="lazy")
    b = h.launch_shapes()
    assert b["source"] == fg.PLAN_FILE
    assert (b["paint_cta"], b["bin_cta"], b["bin_fold"]) == (a["paint_cta"], a["bin_cta"], a["bin_fold"])
    rng = np.random.default_rng(8)
    x, y, z = (rng.uniform(0, L_BOX, 300_000) for _ in range(3))
    want = fg.Grid(Ng, L_BOX, precision="f32", host_view="lazy").power_f32(x, y, z, L_BOX ** 3, (0, 0, 1),
                                                                          2 * np.pi / L_BOX)
    got = h.power_f32(x, y, z, L_BOX ** 3, (0, 0, 1), 2 * np.pi / L_BOX)
    np.testing.assert_array_equal(got["N"], want["N"])
    ok = np.isfinite(want["P"])
    den = np.abs(want["P"][:, :1]) + L_BOX ** 3 / len(x)
    assert (np.abs(got["P"] - want["P"]) / den)[ok].max() <= 1e-6
