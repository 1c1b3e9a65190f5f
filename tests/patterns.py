"""Operand generators of the reference's own tests (test helpers).

  lcg32(seed, n)   test/test_prec.cpp:63-76   x = x*1664525 + 1013904223, limb = x|1
  lcg64(seed, n)   test/bench_ntt.cpp:6-17    x = x*6364136223846793005 + 1442695040888963407, limb = x|1
  torture(name, n, second)  test/fft_torture.cpp:22-49, 58-72 (patterns and shapes)
  splitmix64(seed, n)       SplitMix64 stream, top limb forced nonzero (benchmark operands)
"""
from __future__ import annotations

import numpy as np

import oracle as O

# (name, even-limb value of a, odd/second value, alternate, popcount-parity)
TORTURE_PATTERNS = [
    ("all-ones", 0xFFFFFFFFFFFFFFFF, 0xFFFFFFFFFFFFFFFF, False, False),
    ("ffff0000", 0xFFFF0000FFFF0000, 0xFFFF0000FFFF0000, False, False),
    ("0000ffff", 0x0000FFFF0000FFFF, 0x0000FFFF0000FFFF, False, False),
    ("ff00x00ff", 0xFF00FF00FF00FF00, 0x00FF00FF00FF00FF, False, False),
    ("highxlow", 0xFFFFFFFF00000000, 0x00000000FFFFFFFF, False, False),
    ("carry-run", 0xFFFFFFFFFFFFFF00, 0x00FFFFFFFFFFFFFF, False, False),
    ("alternating", 0xFFFFFFFFFFFFFFFF, 0, True, False),
    ("popcount", 0, 0, False, True),
]
TORTURE_SHAPES = [(193, 193), (255, 256), (511, 767), (1024, 1024), (1536, 2048), (2048, 2048),
                  (2049, 2049), (3072, 4096), (4096, 4096), (6144, 8192), (8192, 8192)]


def _filled(n, even, odd, alternate):
    r = np.full(n, even, dtype=np.uint64)
    if alternate:
        r[1::2] = np.uint64(odd)
    if n and r[-1] == 0:
        r[-1] = np.uint64(even if even else 0xFFFFFFFFFFFFFFFF)
    return r


def _popcount_parity(n):
    i = np.arange(n, dtype=np.uint64)
    par = np.zeros(n, dtype=np.uint64)
    x = i.copy()
    while x.any():
        par ^= x & np.uint64(1)
        x >>= np.uint64(1)
    r = np.where(par == 1, np.uint64(0xFFFF), np.uint64(0)).astype(np.uint64)
    nz = np.flatnonzero(r)
    return r[: nz[-1] + 1] if len(nz) else r[:0]


def torture(name: str, an: int, bn: int):
    """Operands (a, b) of one fft_torture case (test/fft_torture.cpp:80-107, 136-141)."""
    for (pname, va, vb, alt, pop) in TORTURE_PATTERNS:
        if pname == name:
            if pop:
                return _popcount_parity(an), _popcount_parity(bn)
            return _filled(an, va, vb, alt), _filled(bn, vb, va, alt)
    raise KeyError(name)


def lcg32(seed, n):
    return O.lcg32_pattern(seed, n)


def lcg64(seed, n):
    return O.lcg64_pattern(seed, n)


def splitmix64(seed, n):
    a = O.splitmix64(seed, n)
    if n and a[-1] == 0:
        a[-1] = 1
    return a


def make(gen: dict):
    kind = gen["kind"]
    if kind == "torture":
        a, b = torture(gen["pattern"], gen["an"], gen["bn"])
        return a, b
    fn = {"lcg32": lcg32, "lcg64": lcg64, "splitmix64": splitmix64}[kind]
    a = fn(gen["seed_a"], gen["an"])
    b = fn(gen["seed_b"], gen["bn"])
    return a, b
