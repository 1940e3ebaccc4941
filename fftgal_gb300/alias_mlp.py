"""Learned aliasing correction: training and evaluation of the perceptron of
csrc/mlp.cu (5 -> 64 -> 64 -> 64 -> 3, tanh, FP32) that maps single-paint
multipoles to interlaced ones (fftgal_power_learned_f32).

Training pairs come from lognormal mocks (fftgal_gb300.mocks) with redshift-space
distortion along z: each mock is measured twice on the same catalog, with the
interlaced estimator (fftgal_power_f32, src/fft.c:257-276) and with a single
paint (fftgal_power_single_f32); the raw targets are (P_l^int - P_l^single) /
den, den = |P0^single| + Pshot, for l = 0, 2, 4 in every k bin with modes, and
the network learns them divided by the envelope e(k / k_Nyq) = u^6 / (1 + u^6)
and clipped to +-5 (``scaled_targets``): the raw targets span seven decades
from k << k_Nyq to the corners of the cube, and the bins past about 1.5 k_Nyq
hold few modes whose differences are noise.  The gradient and Adam kernels run
on the GPU (their FP64 restatement for the parity tests is oracle/mlp.py).

    python -m fftgal_gb300.alias_mlp train --pairs 2000 --out params.npy
    python -m fftgal_gb300.alias_mlp eval --params params.npy --ng 1024 --np 1e8
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import time

import numpy as np

IN, HID, OUT = 5, 64, 3
L_BOX = 1000.0
HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_PARAMS = os.path.join(HERE, "alias_mlp_params.npy")


def _layout():
    sizes = [("W1", IN * HID), ("b1", HID), ("W2", HID * HID), ("b2", HID), ("W3", HID * HID), ("b3", HID),
             ("W4", HID * OUT), ("b4", OUT)]
    off, out = 0, {}
    for name, n in sizes:
        out[name] = (off, n)
        off += n
    return out, off


LAYOUT, NPARAMS = _layout()
SHAPES = {"W1": (IN, HID), "b1": (HID,), "W2": (HID, HID), "b2": (HID,), "W3": (HID, HID), "b3": (HID,),
          "W4": (HID, OUT), "b4": (OUT,)}


def unpack(p):
    return {k: np.asarray(p[o:o + n]).reshape(SHAPES[k]) for k, (o, n) in LAYOUT.items()}


def init_params(seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAMS, dtype=np.float32)
    for k, (o, n) in LAYOUT.items():
        if k.startswith("W"):
            fan_in, fan_out = SHAPES[k]
            p[o:o + n] = rng.normal(0.0, math.sqrt(1.0 / fan_in), n) * (0.1 if k == "W4" else 1.0)
    return p


class Trainer:
    """Adam on the GPU kernels; data as (n, 5) / (n, 3) FP32 torch tensors."""

    def __init__(self, params, device="cuda"):
        import torch
        from . import lib
        self.torch, self.lib = torch, lib()
        self.dev = torch.device(device)
        self.p = torch.tensor(np.asarray(params, dtype=np.float32), device=self.dev)
        self.g = torch.zeros_like(self.p)
        self.m = torch.zeros_like(self.p)
        self.v = torch.zeros_like(self.p)
        self.loss = torch.zeros(1, dtype=torch.float32, device=self.dev)
        self.step_no = 0
        self.stream = torch.cuda.current_stream(self.dev).cuda_stream

    def _check(self, rc):
        from . import _check
        _check(rc)

    def grad(self, X, T):
        self.g.zero_()
        self.loss.zero_()
        self._check(self.lib.fftgal_mlp_grad(self.p.data_ptr(), X.data_ptr(), T.data_ptr(), int(X.shape[0]),
                                             self.g.data_ptr(), self.loss.data_ptr(), self.stream))
        return self.g, float(self.loss.item())

    def step(self, X, T, lr):
        _, loss = self.grad(X, T)
        self.step_no += 1
        self._check(self.lib.fftgal_mlp_adam(self.p.data_ptr(), self.g.data_ptr(), self.m.data_ptr(),
                                             self.v.data_ptr(), self.step_no, float(lr), self.stream))
        return loss

    def params(self) -> np.ndarray:
        return self.p.detach().cpu().numpy().astype(np.float32)


def forward_gpu(params, X):
    import torch
    from . import lib, _check
    dev = torch.device("cuda")
    p = torch.tensor(np.asarray(params, dtype=np.float32), device=dev)
    x = torch.tensor(np.asarray(X, dtype=np.float32), device=dev)
    y = torch.zeros((len(x), OUT), dtype=torch.float32, device=dev)
    _check(lib().fftgal_mlp_forward(p.data_ptr(), x.data_ptr(), int(len(x)), y.data_ptr(),
                                    torch.cuda.current_stream(dev).cuda_stream))
    return y.cpu().numpy()


TARGET_CLIP = 5.0


def envelope(u):
    """fftgal_alias_envelope: u^6 / (1 + u^6)."""
    u6 = np.asarray(u, dtype=np.float64) ** 6
    return u6 / (1.0 + u6)


def scaled_targets(X, T, clip: float = TARGET_CLIP):
    """The network's targets: raw targets over the envelope of each bin's
    k / k_Nyq (feature 0), clipped to +-clip."""
    e = envelope(X[:, 0])[:, None]
    return np.clip(np.asarray(T, dtype=np.float64) / e, -clip, clip).astype(np.float32)


def features(K, P, Pshot, kNyq):
    """fftgal_alias_features: X[NK][5] for single-paint multipoles P[NK][4]."""
    from . import lib, _check, _dp
    K = np.ascontiguousarray(K, dtype=np.float64)
    P = np.ascontiguousarray(P, dtype=np.float64)
    X = np.zeros((len(K), IN), dtype=np.float32)
    _check(lib().fftgal_alias_features(len(K), K.ctypes.data_as(_dp), P.ctypes.data_as(_dp), float(Pshot),
                                       float(kNyq), X.ctypes.data_as(C.POINTER(C.c_float))))
    return X


def pair(grid, Ng, L, cat, los=(0.0, 0.0, 1.0)):
    """Single-paint and interlaced multipoles of one catalog (device tensors
    x, y, z), the features and the targets of its bins with modes."""
    from . import MEM_DEVICE
    x, y, z = cat
    Np = int(x.numel())
    V, dK = L ** 3, 2 * math.pi / L
    args = (x.data_ptr(), y.data_ptr(), z.data_ptr(), V, los, dK)
    s = grid.power_f32(*args, Nmu=3, where=MEM_DEVICE, Np=Np, interlace=False)
    i = grid.power_f32(*args, Nmu=3, where=MEM_DEVICE, Np=Np, interlace=True)
    Pshot = V / Np
    X = features(s["K"], s["P"], Pshot, math.pi * Ng / L)
    den = np.abs(s["P"][:, 0]) + Pshot
    T = (i["P"][:, :3] - s["P"][:, :3]) / den[:, None]
    ok = (s["N"] > 0) & np.all(np.isfinite(T), axis=1)
    return s, i, X[ok], T[ok].astype(np.float32), ok


def make_pairs(n_pairs: int, seed: int, sizes=(256, 512), np_range=(1e6, 3e7), slopes=(-2.5, -1.0), log=None):
    """Features and raw targets of ``n_pairs`` fresh mocks (mesh of the mock =
    the grid, Ng drawn from ``sizes``, Np log-uniform, spectral slope
    uniform)."""
    import torch
    from . import Grid
    from .mocks import lognormal_catalog
    rng = np.random.default_rng(seed)
    grids = {Ng: Grid(Ng, L_BOX, precision="f32", host_view="lazy") for Ng in sizes}
    for g in grids.values():  # the mocks are written on torch's stream: order the paint after them
        g.set_stream(torch.cuda.current_stream().cuda_stream)
    Xs, Ts = [], []
    for q in range(n_pairs):
        Ng = int(rng.choice(sizes))
        Np = float(np.exp(rng.uniform(math.log(np_range[0]), math.log(np_range[1]))))
        slope = float(rng.uniform(*slopes))
        x, y, z, vx, vy, vz = lognormal_catalog(Ng, L_BOX, Np, seed=int(rng.integers(1 << 30)), slope=slope,
                                                axes=(2,))
        zr = (z + vz).contiguous()  # gal_rsd along z, aH = 1
        torch.cuda.synchronize()
        _, _, X, T, _ = pair(grids[Ng], Ng, L_BOX, (x, y, zr))
        if log:
            log(f"pair {q}: Ng {Ng} Np {int(x.numel())} slope {slope:.2f} max|T| {np.abs(T).max():.3e} "
                f"at k/kN {X[np.abs(T).max(1).argmax(), 0]:.3f}")
        Xs.append(X)
        Ts.append(T)
        del x, y, z, vz, zr
    torch.cuda.empty_cache()
    return np.concatenate(Xs), np.concatenate(Ts)


def train(X, T, epochs: int = 60, batch: int = 4096, lr: float = 2e-3, seed: int = 0, log=None):
    import torch
    tr = Trainer(init_params(seed))
    dev = tr.dev
    Xd = torch.tensor(X, device=dev)
    Td = torch.tensor(T, device=dev)
    n = len(X)
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    hist = []
    for ep in range(epochs):
        perm = torch.randperm(n, generator=gen, device=dev)
        lr_ep = lr * (0.5 * (1 + math.cos(math.pi * ep / epochs)))
        tot = 0.0
        for b0 in range(0, n, batch):
            idx = perm[b0:b0 + batch]
            tot += tr.step(Xd[idx].contiguous(), Td[idx].contiguous(), lr_ep) * len(idx)
        hist.append(tot / n)
        if log:
            log(f"epoch {ep} loss {tot / n:.3e}")
    return tr.params(), hist


def load(path: str = DEFAULT_PARAMS) -> np.ndarray:
    p = np.load(path).astype(np.float32)
    if p.shape != (NPARAMS,):
        raise ValueError(f"{path}: {p.shape}, expected ({NPARAMS},)")
    return p


def evaluate(params, Ng: int, Np: float, n_mocks: int = 2, seed: int = 12345, mock_n: int | None = None):
    """Fresh-seed mocks: errors of single-paint and single-paint + MLP against
    the interlaced estimate (the reference measurement), in units of den, for k < 0.8 k_Nyq
    and over all bins; and the two pipelines' device times."""
    import torch
    from . import Grid, MEM_DEVICE, lib, _check, _dp, _lp
    from .mocks import lognormal_catalog
    g = Grid(Ng, L_BOX, precision="f32", host_view="lazy")
    g.set_stream(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(seed)
    p = np.ascontiguousarray(params, dtype=np.float32)
    out = []
    for q in range(n_mocks):
        slope = float(rng.uniform(-2.5, -1.0))
        x, y, z, vx, vy, vz = lognormal_catalog(mock_n or Ng, L_BOX, Np, seed=int(rng.integers(1 << 30)),
                                                slope=slope, axes=(2,))
        zr = (z + vz).contiguous()
        torch.cuda.synchronize()
        s, i, X, T, ok = pair(g, Ng, L_BOX, (x, y, zr))
        NK = len(s["K"])
        K = np.zeros(NK)
        N = np.zeros(NK, dtype=np.int64)
        Pl = np.zeros((NK, 4))
        los = np.array([0.0, 0.0, 1.0])
        Nx = int(x.numel())
        dK = 2 * math.pi / L_BOX
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        times = {}
        for name in ("interlaced", "single", "learned"):
            torch.cuda.synchronize()
            ev0.record()
            for _ in range(3):
                if name == "learned":
                    _check(lib().fftgal_power_learned_f32(
                        g.p, x.data_ptr(), y.data_ptr(), zr.data_ptr(), Nx, L_BOX ** 3, MEM_DEVICE,
                        los.ctypes.data_as(_dp), dK, 3, p.ctypes.data_as(C.POINTER(C.c_float)),
                        K.ctypes.data_as(_dp), N.ctypes.data_as(_lp), Pl.ctypes.data_as(_dp), None, None, None))
                else:
                    g.power_f32(x.data_ptr(), y.data_ptr(), zr.data_ptr(), L_BOX ** 3, los, dK, Nmu=3,
                                where=MEM_DEVICE, Np=Nx, interlace=(name == "interlaced"))
            ev1.record()
            torch.cuda.synchronize()
            times[name] = ev0.elapsed_time(ev1) / 3
        Pshot = L_BOX ** 3 / Nx
        den = np.abs(s["P"][:, 0]) + Pshot
        kN = math.pi * Ng / L_BOX
        sel = ok & (s["K"] < 0.8 * kN)

        def err(P):
            e = np.abs(P[:, :3] - i["P"][:, :3]) / den[:, None]
            return dict(max_below_0p8=float(e[sel].max()), rms_below_0p8=float(np.sqrt((e[sel] ** 2).mean())),
                        max_all=float(e[ok].max()), rms_all=float(np.sqrt((e[ok] ** 2).mean())))

        out.append(dict(slope=slope, Np=Nx, single=err(s["P"]), learned=err(Pl), ms=times))
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--pairs", type=int, default=2000)
    t.add_argument("--epochs", type=int, default=60)
    t.add_argument("--seed", type=int, default=2024)
    t.add_argument("--out", default=DEFAULT_PARAMS)
    t.add_argument("--save-pairs", default=None, help="write the features and targets to this .npz")
    t.add_argument("--load-pairs", default=None, help="train on the features and targets of this .npz")
    e = sub.add_parser("eval")
    e.add_argument("--params", default=DEFAULT_PARAMS)
    e.add_argument("--ng", type=int, default=1024)
    e.add_argument("--np", type=float, default=1e8)
    e.add_argument("--mocks", type=int, default=2)
    e.add_argument("--seed", type=int, default=12345)
    a = ap.parse_args(argv)
    if a.cmd == "train":
        t0 = time.time()
        if a.load_pairs:
            d = np.load(a.load_pairs)
            X, T = d["X"], d["T"]
        else:
            X, T = make_pairs(a.pairs, a.seed)
        if a.save_pairs:
            np.savez(a.save_pairs, X=X, T=T)
        t1 = time.time()
        params, hist = train(X, scaled_targets(X, T), epochs=a.epochs, seed=a.seed, log=print)
        np.save(a.out, params)
        print(json.dumps(dict(pairs=a.pairs, samples=len(X), gen_s=round(t1 - t0, 1), max_abs_t=float(np.abs(T).max()),
                              train_s=round(time.time() - t1, 1), loss_first=hist[0], loss_last=hist[-1])))
    else:
        res = evaluate(load(a.params), a.ng, a.np, n_mocks=a.mocks, seed=a.seed)
        print(json.dumps(res))


if __name__ == "__main__":
    main()
