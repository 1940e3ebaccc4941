"""Benchmark: interlaced galaxy power spectra per second on GB300.

Workload (one step = one catalog): Np = 1e8 FP32 particles in a 1000 Mpc/h
periodic box, Ng = 1024 grid, PCS paint of both interlacing grids, r2c FFT of
both, offset phase + average + PCS deconvolution, multipoles l = 0,2,4(,6)
and 3 mu wedges with dK = 2 pi / L.  The catalog is the seeded uniform box of
tests/golden/catalogs.py (splitmix64, seed 20240: the same FP32 positions on
every machine), whose FP64 reference answer is tests/golden/headline_ng1024.npz;
``--mock lognormal`` times a clustered redshift-space mock instead.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints ONE JSON line (rank 0).  `value` = catalogs/s with positions already in
HBM (CUDA events on the launching stream, max over ranks); `e2e` = the same
call with positions in pinned host memory (host->device copy inside the timed
region, bins read back every step); `parity` = the timed call's P_l and wedges
against the FP64 answer (the committed reference tables, and the FP64 oracle
run live on this host's CPU on the same catalog); `cpu_baseline` = that live
FP64 run, one full catalog on one core.  ``--impl reference`` times the FP64
CPU path (the reference algorithm restated in C, oracle/) on full catalogs,
one single-threaded process per host core that memory allows.
With ``--gpus N`` (N > 1) and no WORLD_SIZE in the environment the script
starts itself under torch.distributed.run with N ranks, one GPU each.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import socket
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

NG, L_BOX, NP = 1024, 1000.0, 100_000_000
SEED = 20240  # the uniform catalog of tests/golden/headline_ng1024.npz
LOS = (0.0, 0.0, 1.0)
NMU = 3
METRIC = "catalogs/s at Ng=1024,1e8 gal (P0/2/4 err<=1e-4 vs FP64); % HBM roofline"
GOLDEN = os.path.join(ROOT, "tests", "golden", "headline_ng1024.npz")


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--ng", type=int, default=NG)
    ap.add_argument("--np", type=float, default=NP)
    ap.add_argument("--mock", default="uniform", choices=["uniform", "lognormal"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-correction leg")
    ap.add_argument("--plan", default=None,
                    help="plan file of the FFT autotuner (default: one in the temporary directory)")
    ap.add_argument("--profile-steps", type=int, default=0,
                    help="run only warmup+this many steps, no e2e/cpu legs (for ncu)")
    ap.add_argument("--workload", default="headline", choices=["headline", "mixed64"],
                    help="mixed64: 64 lognormal redshift-space mocks with Np log-uniform in [2e6, 2e7], "
                         "Ng from {256, 384, 512} and fold factors from {1, 2, 4}, through one "
                         "fftgal_power_mixed_f32 call per step")
    ap.add_argument("--launch-check", action="store_true",
                    help="exercise the N-rank launch and the max-over-ranks reduction without a GPU "
                         "(gloo) and print the JSON line")
    return ap.parse_args(argv)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# N ranks from one command line
def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def relaunch_command(args, argv) -> list | None:
    """The torch.distributed.run command that runs this script on args.gpus
    ranks, or None when this process is already a rank (WORLD_SIZE set), runs
    one GPU, or runs the CPU reference arm (rank 0 only, no relaunch)."""
    if "WORLD_SIZE" in os.environ or args.gpus <= 1 or args.impl == "reference":
        return None
    return [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
            "--master-addr", "127.0.0.1", f"--master-port={_free_port()}", os.path.abspath(__file__)] + list(argv)


def launch_check(args):
    """One line from N gloo ranks: the launch path and max_over_ranks without a GPU."""
    import torch.distributed as dist
    from fftgal_gb300 import worklist
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        dist.init_process_group("gloo")
    t = worklist.max_over_ranks(1.0 + rank)
    ranks = worklist.gather_tables({rank: {"rank": rank, "local_rank": int(os.environ.get("LOCAL_RANK", "0"))}},
                                   world)
    if rank == 0:
        print(json.dumps({"launch_check": True, "n_gpus": world, "max_over_ranks": t, "ranks": ranks}), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


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
# catalogs
def host_catalog(Ng: int, Np: int, seed: int, mock: str):
    """FP32 x, y, z (numpy) of the benchmark catalog: the seeded uniform box,
    or a lognormal redshift-space mock (256^3 field, z-RSD with aH = 1)."""
    import numpy as np
    if mock == "uniform":
        from catalogs import uniform_box_f32
        return uniform_box_f32(seed, Np, L_BOX)
    from lognormal import lognormal_catalog
    x, y, z, vx, vy, vz = lognormal_catalog(seed, 256, L_BOX, Np)
    return tuple(np.ascontiguousarray(a, dtype=np.float32) for a in (x, y, z + vz))


# ---------------------------------------------------------------------------
# FP64 CPU path (test infrastructure: the oracle restates src/fft.c and
# src/power.c; it is the checker and the CPU baseline, never the product)
def oracle_catalog_run(Ng: int, Np: int, seed: int, mock: str, los, dK: float, nmu: int, warm: bool = True):
    """The P.c sequence fft_p2k -> P -> Pl -> Pmu (src/app/P.c:55-66) of the
    FP64 oracle on the benchmark catalog (FP32 positions widened to FP64),
    single-threaded.  Returns (result dict, seconds of the path, timestamps)."""
    import oracle
    x, y, z = host_catalog(Ng, Np, seed, mock)
    V = L_BOX ** 3
    if warm:  # page in the library and its code paths on a tiny grid
        oracle.power_spectrum(16, L_BOX, x[:1000], y[:1000], z[:1000], los, dK, Nmu=nmu, V=V)
    x, y, z = (a.astype("float64") for a in (x, y, z))
    t0 = time.monotonic()
    g = oracle.Oracle(Ng, L_BOX)
    g.p2k(x, y, z, V)
    g.power(len(x), V)
    K, N, P, _, _ = g.pl(los, dK)
    Km, Nm, Pm, _, _ = g.pmu(los, dK, nmu)
    t1 = time.monotonic()
    return dict(K=K, N=N, P=P, Kmu=Km, Nmu=Nm, Pmu=Pm), t1 - t0, (t0, t1)


def _oracle_proc(args_tuple, barrier, queue):
    """--impl reference worker: build the catalog, wait for the others, time one catalog."""
    Ng, Np, seed, mock, los, dK, nmu = args_tuple
    import oracle
    from catalogs import uniform_box_f32  # noqa: F401  (imported before the barrier)
    x, y, z = host_catalog(Ng, Np, seed, mock)
    V = L_BOX ** 3
    oracle.power_spectrum(16, L_BOX, x[:1000], y[:1000], z[:1000], los, dK, Nmu=nmu, V=V)
    x, y, z = (a.astype("float64") for a in (x, y, z))
    barrier.wait()
    t0 = time.monotonic()
    g = oracle.Oracle(Ng, L_BOX)
    g.p2k(x, y, z, V)
    g.power(len(x), V)
    g.pl(los, dK)
    g.pmu(los, dK, nmu)
    queue.put((t0, time.monotonic()))


def _host_memory_gb() -> float:
    try:
        for ln in open("/proc/meminfo"):
            if ln.startswith("MemAvailable:"):
                return int(ln.split()[1]) / 2 ** 20
    except Exception:
        pass
    return 16.0


def oracle_bytes(Ng: int, Np: int) -> float:
    """Host memory of one FP64 oracle catalog run: the grid and its
    interlacing copy, FP64 and FP32 positions, and numpy temporaries."""
    G8 = Ng * Ng * 2 * (Ng // 2 + 1) * 8
    return 2 * G8 + Np * (24 + 12) + 2 * 2 ** 30


def run_reference(args):
    """--impl reference: the FP64 CPU path on full catalogs of the workload,
    one single-threaded oracle process per host core that memory allows (the
    reference's one-process-per-mock model, src/app/job_P.sh:22-26), started
    together after each has built its catalog.  value = catalogs finished / wall."""
    import multiprocessing as mp
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    Ng, Np = args.ng, int(args.np)
    dK = 2 * math.pi / L_BOX
    cores = os.cpu_count() or 1
    mem = _host_memory_gb()
    nproc = max(1, min(cores, int(0.8 * mem * 2 ** 30 // oracle_bytes(Ng, Np))))
    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(nproc + 1)
    queue = ctx.Queue()
    procs = [ctx.Process(target=_oracle_proc, args=((Ng, Np, SEED, args.mock, LOS, dK, NMU), barrier, queue))
             for _ in range(nproc)]
    for p in procs:
        p.start()
    barrier.wait()
    t0 = time.monotonic()
    spans = [queue.get() for _ in range(nproc)]
    wall = max(s[1] for s in spans) - t0
    for p in procs:
        p.join()
    per = [s[1] - s[0] for s in spans]
    value = nproc / wall
    sample = (f"{nproc} full catalogs run concurrently (Ng={Ng}, Np={Np:.0e} {args.mock}, seed {SEED}), "
              f"FP64 oracle fft_p2k+P+Pl+Pmu, one process per core, {wall:.1f} s wall; "
              f"per catalog {min(per):.1f}-{max(per):.1f} s")
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "catalogs/s",
        "n_gpus": 0, "n_gpus_requested": args.gpus, "cores": nproc,
        "steps": nproc, "steps_requested": args.steps, "warmup": 1,
        "warmup_note": "one Ng=16 pass per process before the timed catalog",
        "ms_per_step": 1000.0 * wall / nproc, "timed_region_s": wall,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (uniform, seeded splitmix64: the catalog of the GPU arm)",
        "config": {"workload": workload_name(Ng, Np), "Ng": Ng, "Np": Np, "mock": args.mock,
                   "host_memory_gb": round(mem, 1), "host_cores": cores},
        "cpu_baseline": {"value": value, "unit": "catalogs/s", "cores": nproc, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "catalogs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


# ---------------------------------------------------------------------------
def workload_name(Ng: int, Np: int) -> str:
    return (f"interlaced PCS P_l (l=0,2,4,6) + {NMU} mu-wedges, Ng={Ng}, Np={Np:.0e}, L={L_BOX:g}, dK=2pi/L, "
            f"FP32 positions+grids, FP64 bin sums")


def algorithmic_bytes(Ng: int, Np: int):
    """Minimal HBM bytes per launch of each stage (FP32 grids, 2 grids)."""
    G4 = Ng * Ng * 2 * (Ng // 2 + 1) * 4      # one padded FP32 grid
    R4 = Ng ** 3 * 4                           # one unpadded real grid
    return {
        "upload": 12 * Np,
        "paint_key": 12 * Np,                  # read x,y,z (key histogram in L2)
        "paint_scan": 0,
        "paint_scatter": 12 * Np + 16 * Np,    # read x,y,z; write the 16-byte records
        "paint_tile": 16 * Np + 2 * G4,        # sorted records in, both grids out
        "fft_k": 2 * (R4 + G4),                # both grids, read real rows, write half spectra
        "fft_j": 2 * 2 * G4,
        "fft_i": 2 * 2 * G4,
        "finish": 0,                           # fused into finish_bin
        "finish_bin": 2 * G4,                  # read both grids, bin the finished power (lazy view: not stored)
    }


def parity_block(res, Ng: int, Np: int, mock: str, live):
    """The timed call's result against the FP64 answers: the committed
    reference tables (uniform catalog at the headline size) and the live
    oracle run on this host."""
    import numpy as np
    import parity
    Pshot = L_BOX ** 3 / Np
    out = {"criterion": "mode counts exact; P0/2/4 and wedges within 1e-4 of |P0|+Pshot for k<0.8 kNyq; "
                        "every bin within 1e-3"}
    if mock == "uniform" and Ng == NG and Np == NP and os.path.exists(GOLDEN):
        z = np.load(GOLDEN)
        e = parity.errors(res, parity.golden_result(z, "uniform", 0, NMU), Pshot, Ng, L_BOX)
        e["pass"] = parity.passes(e)
        e["source"] = "tests/golden/headline_ng1024.npz (reference fft_p2k/P/Pl/Pmu, FP64)"
        out["vs_reference_tables"] = e
    if live is not None:
        e = parity.errors(res, live, Pshot, Ng, L_BOX)
        e["pass"] = parity.passes(e)
        e["source"] = "FP64 oracle on this host, same catalog"
        out["vs_live_oracle"] = e
    return out


def run_mixed(args):
    """--workload mixed64: the covariance-set configuration.  64 lognormal mocks
    (512^3 Gaussian field, P(k) = 1e4 (k/0.1)^-1.5 exp(-(k/0.5)^2), Poisson
    sampled, displaced by the Zel'dovich displacement and shifted along z by
    f Psi_z with f = 0.8, independent seeds) generated on the GPU and kept
    there; one step = one fftgal_power_mixed_f32 call over all 64."""
    import ctypes as C
    import numpy as np
    import torch
    import fftgal_gb300 as fg
    from fftgal_gb300 import mocks
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    rng = np.random.default_rng(64)
    ncat, f = 64, 0.8
    Nps = 10 ** rng.uniform(np.log10(2e6), np.log10(2e7), ncat)
    Ngs = rng.choice([256, 384, 512], ncat)
    folds = rng.choice([1, 2, 4], ncat)
    cats = []
    for c in range(ncat):
        x, y, z, vx, vy, vz = mocks.lognormal_catalog(512, L_BOX, float(Nps[c]), seed=1000 + c, f=f, device=dev)
        cats.append(torch.stack([x + vx / f, y + vy / f, z + vz / f + vz]).contiguous())
        del x, y, z, vx, vy, vz
    torch.cuda.empty_cache()
    n_part = sum(int(t.shape[1]) for t in cats)
    lib = fg.lib()
    ptr = [(C.c_void_p * ncat)(*[t[a].data_ptr() for t in cats]) for a in range(3)]
    Np = np.array([t.shape[1] for t in cats], dtype=np.int64)
    V = np.full(ncat, L_BOX ** 3)
    L = np.ascontiguousarray(L_BOX / folds, dtype=np.float64)
    dK = np.ascontiguousarray(2 * np.pi / L, dtype=np.float64)
    Ngc = np.ascontiguousarray(Ngs, dtype=np.int32)
    los = np.array(LOS)
    tabs = []
    for c in range(ncat):
        NK = fg.nk(int(Ngc[c]), float(L[c]), float(dK[c]))
        tabs.append([np.zeros(NK), np.zeros(NK, dtype=np.int64), np.zeros(NK * 4), np.zeros(NK * NMU),
                     np.zeros(NK * NMU, dtype=np.int64), np.zeros(NK * NMU)])
    outs = [(C.c_void_p * ncat)(*[tabs[c][q].ctypes.data for c in range(ncat)]) for q in range(6)]
    dp = C.POINTER(C.c_double)

    def step():
        rc = lib.fftgal_power_mixed_f32(ncat, ptr[0], ptr[1], ptr[2], Np.ctypes.data_as(C.POINTER(C.c_long)),
                                        V.ctypes.data_as(dp), Ngc.ctypes.data_as(C.POINTER(C.c_int)),
                                        L.ctypes.data_as(dp), los.ctypes.data_as(dp), dK.ctypes.data_as(dp), NMU,
                                        *outs)
        if rc != 0:
            raise RuntimeError(lib.fftgal_last_error().decode())

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()  # returns after the last catalog's tables are on the host
    torch.cuda.synchronize(dev)
    wall = time.perf_counter() - t0
    groups = sorted({(int(a), int(b)) for a, b in zip(Ngs, folds)})
    print(json.dumps({
        "metric": "catalogs/s, 64 mixed lognormal RSD mocks (Ng 256/384/512, folds 1/2/4, Np 2e6-2e7)",
        "value": ncat * args.steps / wall, "unit": "catalogs/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * wall / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (lognormal mocks generated on the GPU, seeds 1000-1063)",
        "config": {"workload": "mixed64", "catalogs": ncat, "particles": n_part, "groups_Ng_fold": groups,
                   "Nmu": NMU, "positions": "device-resident", "timing": "host wall clock around the calls"},
    }), flush=True)


def learned_leg(args, fg, grid, stream, barrier, ptrs, Np, dK, ms_interlaced, res_interlaced):
    """Learned aliasing correction on the same catalog: one paint + FFT, the
    multipoles corrected by the committed perceptron (fftgal_power_learned_f32),
    timed like the interlaced leg; its P_l error against the FP64 reference
    tables beside the plain single paint's and the interlaced estimator's, on
    the benchmark catalog and (at the headline size) on the clustered catalog
    of the same tables."""
    import numpy as np
    import torch
    import parity
    from fftgal_gb300 import alias_mlp
    params = alias_mlp.load()
    V = L_BOX ** 3
    xp, yp, zp = ptrs

    def learned():
        return grid.power_learned_f32(xp, yp, zp, V, LOS, dK, params, Nmu=NMU, where=fg.MEM_DEVICE, Np=Np)

    def single():
        return grid.power_f32(xp, yp, zp, V, LOS, dK, Nmu=NMU, where=fg.MEM_DEVICE, Np=Np, interlace=False)

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = {}
    for name, fn in (("learned", learned), ("single_paint", single)):
        for _ in range(max(2, args.warmup)):
            r = fn()
        barrier()
        e0.record(stream)
        for _ in range(args.steps):
            r = fn()
        e1.record(stream)
        barrier()
        ms = e0.elapsed_time(e1) / args.steps
        out[name] = {"catalogs_per_s": 1000.0 / ms, "ms_per_step": ms, "result": r}
        # stage times of three more calls, outside the timed region
        grid.set_timing(True)
        st = {k: [] for k in fg.STAGES}
        for _ in range(3):
            fn()
            for k, v in grid.stage_times().items():
                st[k].append(v)
        grid.set_timing(False)
        out[name]["stages_ms"] = {k: round(float(np.median(v)), 4) for k, v in st.items()
                                  if float(np.median(v)) > 0.005}
    Ng = grid.Ng
    summary = {
        "catalogs_per_s": out["learned"]["catalogs_per_s"],
        "speedup_vs_interlaced": ms_interlaced / out["learned"]["ms_per_step"],
        "single_paint_catalogs_per_s": out["single_paint"]["catalogs_per_s"],
        "stages_ms": {"learned": out["learned"]["stages_ms"], "single_paint": out["single_paint"]["stages_ms"]},
        "params": "fftgal_gb300/alias_mlp_params.npy",
    }
    if not (args.mock == "uniform" and Ng == NG and Np == NP and os.path.exists(GOLDEN)):
        return summary
    z = np.load(GOLDEN)
    Pshot = V / Np

    def errs(r, name):
        e = parity.errors(r, parity.golden_result(z, name, 0, NMU), Pshot, Ng, L_BOX)
        return {"max_rel_err_P024": e["max_rel_err_P024"], "max_rel_err_wedges": e["max_rel_err_wedges"]}

    summary["vs_fp64_uniform"] = {"interlaced": errs(res_interlaced, "uniform"),
                                  "learned": errs(out["learned"]["result"], "uniform"),
                                  "single_paint": errs(out["single_paint"]["result"], "uniform")}
    from catalogs import clustered_box
    c = [np.ascontiguousarray(a, dtype=np.float32) for a in
         clustered_box(int(z["clustered_seed"]), NP, L_BOX, int(z["clustered_nclusters"]),
                       float(z["clustered_sigma"]))]
    dev = torch.device("cuda", torch.cuda.current_device())
    pos = torch.from_numpy(np.stack(c)).to(dev)
    del c
    cp = [pos[a].data_ptr() for a in range(3)]
    r_int = grid.power_f32(*cp, V, LOS, dK, Nmu=NMU, where=fg.MEM_DEVICE, Np=NP)
    r_learn = grid.power_learned_f32(*cp, V, LOS, dK, params, Nmu=NMU, where=fg.MEM_DEVICE, Np=NP)
    r_single = grid.power_f32(*cp, V, LOS, dK, Nmu=NMU, where=fg.MEM_DEVICE, Np=NP, interlace=False)
    del pos
    summary["vs_fp64_clustered"] = {"interlaced": errs(r_int, "clustered"), "learned": errs(r_learn, "clustered"),
                                    "single_paint": errs(r_single, "clustered")}
    summary["error_unit"] = "|P0_FP64|+Pshot, k<0.8 kNyq, los (0,0,1)"
    return summary


def run_ours(args):
    import numpy as np
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    Ng, Np = args.ng, int(args.np)
    dK = 2 * math.pi / L_BOX
    V = L_BOX ** 3

    # the FP64 CPU run (cpu_baseline and live parity) starts before any CUDA
    # call, in a spawned process, and runs while the GPU legs are timed
    pool = live_job = None
    if rank == 0 and not args.no_cpu_baseline and not args.profile_steps:
        if oracle_bytes(Ng, Np) < 0.8 * _host_memory_gb() * 2 ** 30:
            import multiprocessing as mp
            pool = mp.get_context("spawn").Pool(1)
            live_job = pool.apply_async(oracle_catalog_run, (Ng, Np, SEED, args.mock, LOS, dK, NMU))

    import torch
    import torch.distributed as dist
    import fftgal_gb300 as fg
    from fftgal_gb300 import worklist

    if world > 1:
        dist.init_process_group("nccl")
    if torch.cuda.device_count() <= local:
        raise SystemExit(f"bench: rank {rank} needs GPU {local}, {torch.cuda.device_count()} visible")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)

    hx = host_catalog(Ng, Np, SEED, args.mock)
    Np = len(hx[0])
    host = torch.empty((3, Np), dtype=torch.float32, pin_memory=True)
    for a in range(3):
        host[a].numpy()[:] = hx[a]
    del hx
    pos = host.to(dev)
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
    hp = [host[a].numpy() for a in range(3)]
    # fftgal_power_batch_f32: one catalog per step, each copied host -> device
    # inside the timed region (overlapping the previous catalog's computation)
    grid.power_batch_f32([hp] * 2, V, LOS, dK, Nmu=NMU)
    barrier()
    k2 = max(3, args.steps)  # one catalog per timed step, as the device-resident leg
    e0.record(stream)
    res_e2e = grid.power_batch_f32([hp] * k2, V, LOS, dK, Nmu=NMU)
    e1.record(stream)
    barrier()
    ms2 = worklist.max_over_ranks(e0.elapsed_time(e1))
    e2e = world * k2 / (ms2 / 1000.0)
    NK = fg.nk(Ng, L_BOX, dK)
    d2h = NK * (4 + NMU + 1) * 8

    # rank 0 only, synchronising its own device (the other ranks wait at the final barrier)
    learned = learned_leg(args, fg, grid, stream, lambda: torch.cuda.synchronize(dev), (xp, yp, zp), Np, dK,
                          ms / args.steps, res) if rank == 0 and not args.no_learned else None

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
    # per stage: CUDA-event ms, algorithmic GB/s and its fraction of the
    # measured HBM peak (the positions are on the device: no upload stage)
    stage_table = {}
    for k in algo:
        gbs = (algo[k] / (avg[k] / 1000.0) / 1e9
               if k != "upload" and algo.get(k) and avg[k] > 0.005 else None)
        stage_table[k] = {"ms": round(avg[k], 4), "GBs": None if gbs is None else round(gbs, 1),
                          "frac_of_hbm": None if gbs is None else round(gbs / hbm, 4)}

    if rank == 0:
        cpu = live = None
        if live_job is not None:
            live, secs, _ = live_job.get()
            pool.close()
            pool.join()
            cpu = {"value": 1.0 / secs, "unit": "catalogs/s", "cores": 1, "kind": "port",
                   "sample": f"one full catalog of this workload (Ng={Ng}, Np={Np:.0e} {args.mock}, seed {SEED}, "
                             f"positions widened to FP64): FP64 oracle restating src/fft.c + src/power.c, "
                             f"fft_p2k+P+Pl+Pmu, {secs:.1f} s on 1 core"}
        par = parity_block(res, Ng, Np, args.mock, live)
        # the same catalog through the e2e call: equal up to the order of the
        # FP64 atomic additions of the bin sums
        den = np.abs(res["P"][:, :1]) + L_BOX ** 3 / Np
        fin = np.isfinite(res["P"])
        par["e2e_vs_device_resident_max_rel"] = float(
            (np.abs(res_e2e[-1]["P"] - res["P"]) / den)[fin].max())
        out = {
            "metric": METRIC, "value": value, "unit": "catalogs/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": (f"synthetic (uniform box, splitmix64 seed {SEED}, FP32, generated on the host)"
                     if args.mock == "uniform" else "synthetic (lognormal mock with z-RSD, seeded, numpy)"),
            "config": {"workload": workload_name(Ng, Np),
                       "Ng": Ng, "Np": Np, "los": LOS, "mock": args.mock, "seed": SEED,
                       "l2": "inputs larger than L2 (two 4.3 GB grids per step)",
                       "parallelism": f"replicas x{world}",
                       "fft_plan": {"source": ["built-in", "measured", "plan file", "process cache"][
                           grid.plan_info()["source"]], "tune": grid.plan_info()["tune"]},
                       "launch_shapes": {k: v for k, v in grid.launch_shapes().items() if k != "ms"},
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
            "parity": par,
            "learned": learned,
        }
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    args = parse(argv)
    cmd = relaunch_command(args, argv)
    if cmd is not None:
        if not args.launch_check:
            import torch
            if torch.cuda.device_count() < args.gpus:
                raise SystemExit(f"bench: --gpus {args.gpus} but {torch.cuda.device_count()} GPUs visible")
        sys.exit(subprocess.call(cmd))
    if args.launch_check:
        launch_check(args)
    elif args.impl == "reference":
        run_reference(args)
    elif args.workload == "mixed64":
        run_mixed(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
