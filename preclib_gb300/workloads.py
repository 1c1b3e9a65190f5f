"""Seeded synthetic operands of the benchmark configurations.

Vectorised numpy generators (no oracle involvement):
  * splitmix64(seed, n): the SplitMix64 stream, limb i = mix(seed + (i+1)*gamma)
  * operand(seed, n): n uniform limbs, top limb forced nonzero
  * batch_sizes(seed, count): log-uniform lo in [200, 65536] limbs, hi = lo * U[1, 2]
"""
from __future__ import annotations

import numpy as np

GAMMA = np.uint64(0x9E3779B97F4A7C15)
M1 = np.uint64(0xBF58476D1CE4E5B9)
M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, n: int) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + (np.arange(1, n + 1, dtype=np.uint64) * GAMMA)
        z = (z ^ (z >> np.uint64(30))) * M1
        z = (z ^ (z >> np.uint64(27))) * M2
        return z ^ (z >> np.uint64(31))


def operand(seed: int, n: int) -> np.ndarray:
    a = splitmix64(seed, n)
    if n and a[-1] == 0:
        a[-1] = 1
    return a


def batch_sizes(seed: int, count: int, lo_min: int = 200, lo_max: int = 65536):
    """(lo, hi) limb counts: lo log-uniform in [lo_min, lo_max], hi = round(lo * U[1,2])."""
    rng = np.random.default_rng(seed)
    lo = np.rint(np.exp(rng.uniform(np.log(lo_min), np.log(lo_max), count))).astype(np.int64)
    hi = np.rint(lo * rng.uniform(1.0, 2.0, count)).astype(np.int64)
    return lo, hi
