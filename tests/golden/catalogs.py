"""Seeded synthetic catalogs shared by the golden-fixture generator and the
tests.  The generator is splitmix64 written with numpy integer arithmetic, so
the same seed gives the same positions on every machine and numpy version."""
from __future__ import annotations

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64_uniform(seed: int, n: int) -> np.ndarray:
    """n doubles in [0, 1) from the splitmix64 stream started at `seed`."""
    with np.errstate(over="ignore"):
        s = (np.uint64(seed) + np.uint64(0x9E3779B97F4A7C15)
             * np.arange(1, n + 1, dtype=np.uint64))
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
