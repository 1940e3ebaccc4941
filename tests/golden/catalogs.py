"""Seeded synthetic catalogs shared by the golden-fixture generator and the
tests.  The generator is splitmix64 written with numpy integer arithmetic, so
the same seed gives the same positions on every machine and numpy version."""
from __future__ import annotations

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64_uniform(seed: int, n: int, start: int = 0) -> np.ndarray:
    """Doubles start .. start+n-1 in [0, 1) of the splitmix64 stream started
    at `seed`."""
    with np.errstate(over="ignore"):
        s = (np.uint64(seed) + np.uint64(0x9E3779B97F4A7C15)
             * np.arange(start + 1, start + n + 1, dtype=np.uint64))
        z = s
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def uniform_box(seed: int, n: int, L: float, lo: float = 0.0):
    """x, y, z uniform in [lo, lo+L) (the uniform-box configuration: positions
    uniform-random in a periodic box, FP64)."""
    u = splitmix64_uniform(seed, 3 * n).reshape(3, n)
    return tuple(lo + L * u[a] for a in range(3))


def uniform_box_f32(seed: int, n: int, L: float, chunk: int = 1 << 23):
    """FP32 x, y, z equal to uniform_box(seed, n, L) rounded to FP32, generated
    in chunks so that 1e8-particle catalogs need little more memory than
    their FP32 arrays."""
    out = [np.empty(n, dtype=np.float32) for _ in range(3)]
    for a in range(3):
        for s0 in range(0, n, chunk):
            m = min(chunk, n - s0)
            out[a][s0:s0 + m] = L * splitmix64_uniform(seed, m, start=a * n + s0)
    return tuple(out)


def clustered_box(seed: int, n: int, L: float, nclusters: int, sigma: float):
    """x, y, z of a Neyman-Scott cluster process in the periodic box [0, L)^3:
    `nclusters` centres uniform in the box, each particle attached to a
    uniformly drawn centre and offset per axis by sigma times a unit-variance
    Irwin-Hall variate (sum of 4 uniforms, centred, times sqrt(3)), wrapped
    into the box.  Only splitmix64 integers and single IEEE additions,
    multiplications and divisions are used, so the same seed gives the same
    positions on every machine."""
    c = uniform_box(seed, nclusters, L)
    idx = (splitmix64_uniform(seed + 1, n) * nclusters).astype(np.int64)
    out = []
    for a in range(3):
        u = splitmix64_uniform(seed + 2 + a, 4 * n).reshape(4, n)
        off = (((u[0] + u[1]) + u[2]) + u[3] - 2.0) * (sigma * 1.7320508075688772)
        del u
        x = c[a][idx] + off
        out.append(x - L * np.floor(x / L))
    return tuple(out)


def float32_positions(x, y, z):
    """FP32 copies of FP64 positions (round to nearest) and their exact FP64
    values: the catalog as the FP32 path sees it and as the FP64 reference
    path is given it."""
    p32 = [np.ascontiguousarray(a, dtype=np.float32) for a in (x, y, z)]
    return p32, [a.astype(np.float64) for a in p32]
