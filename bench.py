"""Benchmark: interlaced galaxy power spectra per second on GB300.

Workload (one step = one catalog): Np = 1e8 FP32 particles in a 1000 Mpc/h
periodic box, Ng = 1024 grid, PCS paint of both interlacing grids, r2c FFT of
both, offset phase + average + PCS deconvolution, multipoles l = 0,2,4(,6)
and 3 mu wedges with dK = 2 pi / L.  Positions are seeded synthetic catalogs
generated on the GPU (uniform, or the lognormal RSD mock with --mock lognormal).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints ONE JSON line (rank 0).  `value` = catalogs/s with positions already in
HBM (CUDA events on the launching stream, max over ranks); `e2e` = the same
call with positions in pinned host memory (host->device copy inside the timed
region, bins read back every step).  `--impl reference` times the FP64 CPU
oracle (the reference algorithm restated in C, oracle/) on the host cores.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NG, L_BOX, NP = 1024, 1000.0, 100_000_000
LOS = (0.0, 0.0, 1.0)
NMU = 3
METRIC = "catalogs/s at Ng=1024,1e8 gal (P0/2/4 err<=1e-4 vs FP64); % HBM roofline"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--ng", type=int, default=NG)
    ap.add_argument("--np", type=float, default=NP)
    ap.add_argument("--mock", default="uniform", choices=["uniform", "lognormal"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--plan", default=None,
                    help="plan file of the FFT autotuner (default: one in the temporary directory)")
    ap.add_argument("--profile-steps", type=int, default=0,
                    help="run only warmup+this many steps, no e2e/cpu legs (for ncu)")
    return ap.parse_args()


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# clocks during the timed region
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev: int):
        self.dev = dev
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-i", str(self.dev), "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for ln in open(self.path):
                t = [x.strip() for x in ln.split(",")]
                if len(t) >= 9 and t[1].replace(".", "").isdigit():
                    rows.append(t)
        except Exception:
            pass
        finally:
            try:
                os.unlink(self.path)
            except Exception:
                pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows]
        smax = max(float(r[2]) for r in rows)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": reasons,
                "samples": len(rows), "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit())}


# ---------------------------------------------------------------------------
# CPU oracle baseline (bounded sample, extrapolated to the full workload)
def cpu_sample(seed: int = 1, Ng: int = 256, scale: int = 64):
    """Time the FP64 oracle (p2k + P + Pl + Pmu, src/fft.c:257-276,
    src/power.c:12-178 restated in C) on an Ng grid with Np/scale particles
    (scale = (1024/Ng)^3 keeps the full workload's particle density) and
    extrapolate to Ng=1024, 1e8: particle, grid and binning work x scale, FFT
    work x scale x log(1024^3)/log(Ng^3) (N log N).
    Returns (seconds per full catalog, sample seconds)."""
    import numpy as np
    import oracle
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from catalogs import uniform_box
    n = int(NP) // scale
    x, y, z = uniform_box(seed, n, L_BOX)
    V = L_BOX ** 3
    t0 = time.perf_counter()
    g = oracle.Oracle(Ng, L_BOX)
    g.p2k(x, y, z, V)
    g.power(n, V)
    g.pl(LOS, 2 * math.pi / L_BOX)
    g.pmu(LOS, 2 * math.pi / L_BOX, NMU)
    t_all = time.perf_counter() - t0
    # one FFT alone, to split the N log N part from the linear part
    rnd = np.random.default_rng(seed).standard_normal(g.f.shape)
    g.f[:] = rnd
    t1 = time.perf_counter()
    g.x2k(0)
    t_fft = time.perf_counter() - t1
    lin = max(t_all - 2 * t_fft, 0.0)
    full = lin * scale + 2 * t_fft * scale * (math.log2(NG ** 3) / math.log2(Ng ** 3))
    return full, t_all + t_fft


def _cpu_worker(args):
    seed, Ng = args
    return cpu_sample(seed, Ng, (NG // Ng) ** 3)


def run_reference(args):
    """--impl reference: the CPU path on all host cores (one single-threaded
    oracle process per core, the reference's one-process-per-mock model)."""
    import multiprocessing as mp
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    # keep every process's memory (~0.35 GB at Ng=256) well inside the host
    try:
        import psutil
        mem_gb = psutil.virtual_memory().available / 2 ** 30
        cores = max(1, min(cores, int(mem_gb // 1.0)))
    except Exception:
        pass
    ctx = mp.get_context("spawn")
    times = []
    with ctx.Pool(cores) as pool:
        for w in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            res = pool.map(_cpu_worker, [(100 + w * cores + c, 256) for c in range(cores)])
            wall = time.perf_counter() - t0
            if w >= args.warmup:
                # catalogs per second across the concurrent processes
                times.append(sum(1.0 / r[0] for r in res))
    value = statistics.median(times)
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "catalogs/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 / value, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (uniform, seeded)",
        "config": {"workload": f"interlaced P_l + 3 wedges, Ng={NG}, Np=1e8, L={L_BOX:g}",
                   "sample": "Ng=256, Np=1.5625e6 per process, extrapolated x64 (FFT x64x30/24)"},
        "cpu_baseline": {"value": value, "unit": "catalogs/s", "cores": cores, "kind": "port",
                         "sample": "FP64 oracle restating src/fft.c + src/power.c, Ng=256 with Np/64 per "
                                   "process, one process per core, extrapolated to Ng=1024/1e8"},
        "e2e": {"value": value, "unit": "catalogs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


# ---------------------------------------------------------------------------
def make_catalog(torch, Np: int, seed: int, mock: str, dev):
    """(3, N) FP32 positions on the device: a uniform box, or a lognormal
    mock (256^3 field, Zel'dovich velocities, redshift space along z) with
    about Np particles."""
    if mock == "uniform":
        g = torch.Generator(device=dev)
        g.manual_seed(seed)
        return torch.rand((3, Np), generator=g, device=dev, dtype=torch.float32) * L_BOX
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from lognormal import lognormal_catalog
    x, y, z, vx, vy, vz = lognormal_catalog(seed, 256, L_BOX, Np)
    pos = np.stack([x, y, z + vz]).astype(np.float32)  # gal_rsd along z with aH = 1
    return torch.from_numpy(pos).to(dev)


def algorithmic_bytes(Ng: int, Np: int):
    """Minimal HBM bytes per launch of each stage (FP32 grids, 2 grids)."""
    G4 = Ng * Ng * 2 * (Ng // 2 + 1) * 4      # one padded FP32 grid
    R4 = Ng ** 3 * 4                           # one unpadded real grid
    return {
        "upload": 12 * Np,
        "paint_key": 12 * Np + 8 * Np,         # read x,y,z; write key + rank
        "paint_scan": 0,
        "paint_scatter": 12 * Np + 8 * Np + 16 * Np,
        "paint_tile": 16 * Np + 2 * G4,        # sorted records in, both grids out
        "fft_k": 2 * (R4 + G4),                # both grids, read real rows, write half spectra
        "fft_j": 2 * 2 * G4,
        "fft_i": 2 * 2 * G4,
        "finish": 0,                           # fused into finish_bin
        "finish_bin": 3 * G4,                  # read both grids, write one, bin its power
    }


def run_ours(args):
    import numpy as np
    import torch
    import torch.distributed as dist
    import fftgal_gb300 as fg
    from fftgal_gb300 import worklist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    Ng, Np = args.ng, int(args.np)
    dK = 2 * math.pi / L_BOX
    V = L_BOX ** 3

    pos = make_catalog(torch, Np, 1234 + rank, args.mock, dev)
    Np = int(pos.shape[1])
    # the FFT launch shapes come from the autotuner's plan file (measured on
    # the first run on a device, like FFTW_MEASURE wisdom)
    plan = args.plan or os.path.join(tempfile.gettempdir(), f"fftgal_gb300_plan_rank{local}.txt")
    grid = fg.Grid(Ng, L_BOX, wisdom=plan, precision="f32", host_view="lazy")
    grid.set_stream(stream.cuda_stream)
    xp, yp, zp = (pos[a].data_ptr() for a in range(3))

    def step():
        return grid.power_f32(xp, yp, zp, V, LOS, dK, Nmu=NMU, where=fg.MEM_DEVICE, Np=Np)

    def barrier():
        torch.cuda.synchronize(dev)
        if world > 1:
            dist.barrier()

    for _ in range(args.warmup):
        res = step()
    barrier()
    if args.profile_steps:
        for _ in range(args.profile_steps):
            step()
        barrier()
        if rank == 0:
            print(json.dumps({"profile_steps": args.profile_steps}), flush=True)
        return

    grid.set_timing(True)
    stages = {k: [] for k in fg.STAGES}
    launches0 = fg.lib().fftgal_launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        e0.record(stream)
        for _ in range(args.steps):
            res = step()
            for k, v in grid.stage_times().items():
                stages[k].append(v)
        e1.record(stream)
        barrier()
    launches = fg.lib().fftgal_launch_count() - launches0
    ms = worklist.max_over_ranks(e0.elapsed_time(e1))  # whole job: the slowest rank
    value = world * args.steps / (ms / 1000.0)
    clocks = clk.summary()
    grid.set_timing(False)

    # e2e: positions in pinned host memory, copied every step
    host = torch.empty((3, Np), dtype=torch.float32, pin_memory=True)
    host.copy_(pos)
    hp = [host[a].numpy() for a in range(3)]
    # fftgal_power_batch_f32: one catalog per step, each copied host -> device
    # inside the timed region (overlapping the previous catalog's computation)
    grid.power_batch_f32([hp] * 2, V, LOS, dK, Nmu=NMU)
    barrier()
    k2 = max(3, args.steps)  # one catalog per timed step, as the device-resident leg
    e0.record(stream)
    grid.power_batch_f32([hp] * k2, V, LOS, dK, Nmu=NMU)
    e1.record(stream)
    barrier()
    ms2 = worklist.max_over_ranks(e0.elapsed_time(e1))
    e2e = world * k2 / (ms2 / 1000.0)
    NK = fg.nk(Ng, L_BOX, dK)
    d2h = NK * (4 + NMU + 1) * 8

    # roofline of the dominant kernel
    hbm, peak_kind = peaks()
    avg = {k: statistics.mean(v) for k, v in stages.items()}
    algo = algorithmic_bytes(Ng, Np)
    kern = {k: avg[k] for k in algo if k != "upload"}
    dom = max(kern, key=kern.get)
    achieved = algo[dom] / (avg[dom] / 1000.0) / 1e9
    # DRAM bytes per launch of each kernel at this workload, from an ncu capture
    # (profiles/traffic_ng1024_np1e8.txt, "stage bytes" lines)
    traffic = None
    tr_path = os.path.join(ROOT, "profiles", "traffic_ng1024_np1e8.txt")
    if Ng == NG and Np == int(NP) and os.path.exists(tr_path):
        for line in open(tr_path):
            f = line.split("#")[0].split()
            if len(f) == 2 and f[0] == dom:
                traffic = int(f[1])
    # whole-step algorithmic bytes of the unfused pipeline: paint 12 Np + 2 G,
    # FFT 2 HBM passes (R+W) per grid, phase/average/deconv 3 G, binning G
    G4 = Ng * Ng * 2 * (Ng // 2 + 1) * 4
    step_algo = 12 * Np + 2 * G4 + 2 * 4 * G4 + 3 * G4 + G4
    stage_table = {k: {"ms": round(avg[k], 4),
                       "GBs": (round(algo[k] / (avg[k] / 1000.0) / 1e9, 1) if algo.get(k) and avg[k] > 0 else None)}
                   for k in algo}

    out = None
    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            full, wall = cpu_sample(1, 512, 8)
            cpu = {"value": 1.0 / full, "unit": "catalogs/s", "cores": 1, "kind": "port",
                   "sample": f"FP64 oracle (src/fft.c + src/power.c restated), Ng=512, Np=1.25e7 uniform, "
                             f"{wall:.1f}s, extrapolated to Ng=1024/1e8 (x8, FFT x8x30/27)"}
        out = {
            "metric": METRIC, "value": value, "unit": "catalogs/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": ("synthetic (uniform, seeded, generated on the GPU)" if args.mock == "uniform" else
                     "synthetic (lognormal mock with z-RSD, seeded, numpy)"),
            "config": {"workload": f"interlaced PCS P_l (l=0,2,4,6) + {NMU} mu-wedges, Ng={Ng}, Np={Np:.0e}, "
                                   f"L={L_BOX:g}, dK=2pi/L, FP32 positions+grids, FP64 bin sums",
                       "Ng": Ng, "Np": Np, "los": LOS, "mock": args.mock,
                       "l2": "inputs larger than L2 (two 4.3 GB grids per step)",
                       "parallelism": f"replicas x{world}",
                       "fft_plan": {"source": ["built-in", "measured", "plan file", "process cache"][
                           grid.plan_info()["source"]], "tune": grid.plan_info()["tune"]},
                       "particles_per_s": round(value * Np, 1),
                       "particles_per_s_e2e": round(e2e * Np, 1),
                       "stages_ms": stage_table,
                       "step_roofline": {"algorithmic_bytes": step_algo,
                                         "achieved_GBs": round(step_algo / (ms / args.steps / 1000) / 1e9, 1),
                                         "frac": round(step_algo / (ms / args.steps / 1000) / 1e9 / hbm, 4)}},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": hbm,
                         "unit": "GB/s", "frac": round(achieved / hbm, 4), "traffic": traffic,
                         "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                         else "fallback 6.8 TB/s"},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e, "unit": "catalogs/s", "h2d_bytes_per_step": 12 * Np,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": int(launches),
            "clocks": clocks,
            "check": {"P0_k5": float(res["P"][5, 0]), "Pshot": V / Np, "N_k5": int(res["N"][5])},
        }
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
