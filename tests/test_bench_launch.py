"""bench.py's N-rank launch without a GPU: `--gpus 2` with no WORLD_SIZE in
the environment starts two ranks under torch.distributed.run, which reduce
over gloo and print one JSON line with n_gpus = 2."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _run(args):
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, capture_output=True, text=True,
                       timeout=300, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    return [json.loads(ln) for ln in r.stdout.splitlines() if ln.startswith("{")]


def test_two_ranks_one_line():
    lines = _run(["--gpus", "2", "--launch-check"])
    assert len(lines) == 1
    out = lines[0]
    assert out["n_gpus"] == 2
    assert out["max_over_ranks"] == 2.0  # rank r reports 1 + r
    assert [r["rank"] for r in out["ranks"]] == [0, 1]


def test_one_rank_runs_in_process():
    lines = _run(["--launch-check"])
    assert len(lines) == 1 and lines[0]["n_gpus"] == 1


def test_relaunch_command():
    import bench
    a = bench.parse(["--gpus", "4", "--steps", "7"])
    saved = os.environ.pop("WORLD_SIZE", None)
    try:
        cmd = bench.relaunch_command(a, ["--gpus", "4", "--steps", "7"])
        assert cmd[1:4] == ["-m", "torch.distributed.run", "--nnodes=1"]
        assert "--nproc-per-node=4" in cmd and "127.0.0.1" in cmd
        assert cmd[-4:] == ["--gpus", "4", "--steps", "7"]
        # the CPU reference arm and single-GPU runs stay in this process
        assert bench.relaunch_command(bench.parse(["--gpus", "4", "--impl", "reference"]), []) is None
        assert bench.relaunch_command(bench.parse(["--gpus", "1"]), []) is None
        os.environ["WORLD_SIZE"] = "4"
        assert bench.relaunch_command(a, []) is None
    finally:
        if saved is None:
            os.environ.pop("WORLD_SIZE", None)
        else:
            os.environ["WORLD_SIZE"] = saved


def test_algorithmic_bytes_of_the_stages():
    """The per-stage algorithmic bytes behind the bench line's GB/s and HBM
    fractions (Ng = 1024, Np = 1e8): the lazy fused call's finish + binning
    reads both grids and stores nothing; the FFT passes read and write both."""
    import bench
    a = bench.algorithmic_bytes(1024, 100_000_000)
    G4 = 1024 * 1024 * 1026 * 4
    assert a["paint_key"] == 12 * 100_000_000
    assert a["paint_scatter"] == 28 * 100_000_000
    assert a["paint_tile"] == 16 * 100_000_000 + 2 * G4
    assert a["fft_j"] == a["fft_i"] == 4 * G4
    assert a["finish_bin"] == 2 * G4
