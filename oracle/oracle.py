"""ctypes wrappers over the oracle restatement and the reference build.

Test infrastructure only.  Arrays are numpy uint64 limb vectors
(little-endian limbs, value = sum a[i] * 2**(64*i)).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = {}

_u64p = ctypes.POINTER(ctypes.c_uint64)


def build(quiet: bool = True) -> None:
    """Compile liboracle.so in place (gcc, a fraction of a second)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_u64p)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        for name in ("oracle_mul_basic", "oracle_mul_ntt", "oracle_mul"):
            f = getattr(L, name)
            f.restype = ctypes.c_size_t
            f.argtypes = [_u64p, ctypes.c_size_t, _u64p, ctypes.c_size_t, _u64p]
        L.oracle_mul_fft.restype = ctypes.c_size_t
        L.oracle_mul_fft.argtypes = [_u64p, ctypes.c_size_t, _u64p, ctypes.c_size_t, _u64p,
                                     ctypes.POINTER(ctypes.c_double)]
        L.oracle_mod_u64.restype = ctypes.c_uint64
        L.oracle_mod_u64.argtypes = [_u64p, ctypes.c_size_t, ctypes.c_uint64]
        L.oracle_splitmix64.restype = None
        L.oracle_splitmix64.argtypes = [ctypes.c_uint64, ctypes.c_size_t, _u64p]
        L.oracle_lcg64_pattern.restype = None
        L.oracle_lcg64_pattern.argtypes = [ctypes.c_uint64, ctypes.c_size_t, _u64p]
        L.oracle_lcg32_pattern.restype = None
        L.oracle_lcg32_pattern.argtypes = [ctypes.c_uint32, ctypes.c_size_t, _u64p]
        L.oracle_last_fft_error.restype = ctypes.c_double
        L.oracle_last_fft_zones.restype = ctypes.c_int
        _LIB = L
    return _LIB


def ref_lib(variant: str = ""):
    """The reference compiled from its own sources, or None if absent."""
    if variant not in _REF:
        name = "libprecref%s.so" % (("_" + variant) if variant else "")
        path = os.path.join(HERE, "_ref", name)
        if not os.path.exists(path):
            _REF[variant] = None
        else:
            L = ctypes.CDLL(path)
            for fname in ("ref_mul_ntt", "ref_mul_basic", "ref_mul"):
                f = getattr(L, fname)
                f.restype = ctypes.c_size_t
                f.argtypes = [_u64p, ctypes.c_size_t, _u64p, ctypes.c_size_t, _u64p]
            L.ref_mul_fft.restype = ctypes.c_size_t
            L.ref_mul_fft.argtypes = [_u64p, ctypes.c_size_t, _u64p, ctypes.c_size_t, _u64p,
                                      ctypes.POINTER(ctypes.c_double)]
            L.ref_sqr.restype = ctypes.c_size_t
            L.ref_sqr.argtypes = [_u64p, ctypes.c_size_t, _u64p]
            _REF[variant] = L
    return _REF[variant]


def _c(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint64)


def _call(fn, a, b):
    a, b = _c(a), _c(b)
    out = np.zeros(max(len(a) + len(b), 1), dtype=np.uint64)
    fn(_ptr(a), len(a), _ptr(b), len(b), _ptr(out))
    return out[: len(a) + len(b)]


def mul_basic(a, b) -> np.ndarray:
    return _call(lib().oracle_mul_basic, a, b)


def mul_ntt(a, b) -> np.ndarray:
    return _call(lib().oracle_mul_ntt, a, b)


def mul(a, b) -> np.ndarray:
    """operator* for the bands the GPU library replaces."""
    return _call(lib().oracle_mul, a, b)


def mul_fft(a, b):
    """Returns (product limbs, max rounding distance of this product)."""
    a, b = _c(a), _c(b)
    out = np.zeros(max(len(a) + len(b), 1), dtype=np.uint64)
    err = ctypes.c_double(0.0)
    lib().oracle_mul_fft(_ptr(a), len(a), _ptr(b), len(b), _ptr(out), ctypes.byref(err))
    return out[: len(a) + len(b)], err.value


def mod_u64(a, q: int) -> int:
    a = _c(a)
    return int(lib().oracle_mod_u64(_ptr(a), len(a), q))


def is_prime_u64(n: int) -> bool:
    """Miller-Rabin with the first twelve prime bases, deterministic below
    3.3 * 10^24 (so for every 64-bit n)."""
    if n < 2:
        return False
    bases = (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37)
    for p in bases:
        if n % p == 0:
            return n == p
    d, s = n - 1, 0
    while d % 2 == 0:
        d //= 2
        s += 1
    for a in bases:
        x = pow(a, d, n)
        if x in (1, n - 1):
            continue
        for _ in range(s - 1):
            x = x * x % n
            if x == n - 1:
                break
        else:
            return False
    return True


def random_primes61(seed: int, count: int) -> list:
    """`count` distinct primes in [2^60, 2^61) drawn from a seeded generator:
    the moduli of the schoolbook spot check (a*b mod q against (a mod q)(b mod q))."""
    import random
    rng = random.Random(seed)
    out = []
    while len(out) < count:
        q = rng.randrange(1 << 60, 1 << 61) | 1
        if q not in out and is_prime_u64(q):
            out.append(q)
    return out


def spot_check(p, a, b, seed: int, fixed=()) -> None:
    """Asserts p == a*b modulo the `fixed` moduli and two random 61-bit
    primes of `seed` (the primes are named in the failure message)."""
    for q in tuple(fixed) + tuple(random_primes61(seed, 2)):
        want = mod_u64(a, q) * mod_u64(b, q) % q
        got = mod_u64(p, q)
        assert got == want, "product differs modulo %d" % q


def splitmix64(seed: int, n: int) -> np.ndarray:
    out = np.zeros(max(n, 1), dtype=np.uint64)
    lib().oracle_splitmix64(seed, n, _ptr(out))
    return out[:n]


def lcg64_pattern(seed: int, n: int) -> np.ndarray:
    out = np.zeros(max(n, 1), dtype=np.uint64)
    lib().oracle_lcg64_pattern(seed, n, _ptr(out))
    return out[:n]


def lcg32_pattern(seed: int, n: int) -> np.ndarray:
    out = np.zeros(max(n, 1), dtype=np.uint64)
    lib().oracle_lcg32_pattern(seed, n, _ptr(out))
    return out[:n]


def ref_mul_ntt(a, b, variant=""):
    return _call(ref_lib(variant).ref_mul_ntt, a, b)


def ref_mul(a, b, variant=""):
    return _call(ref_lib(variant).ref_mul, a, b)


def ref_mul_basic(a, b, variant=""):
    return _call(ref_lib(variant).ref_mul_basic, a, b)


def ref_sqr(a, variant=""):
    """The reference's precn_sqr (src/mul_basic.cpp:193-204)."""
    a = _c(a)
    out = np.zeros(max(2 * len(a), 1), dtype=np.uint64)
    ref_lib(variant).ref_sqr(_ptr(a), len(a), _ptr(out))
    return out[: 2 * len(a)]


def ref_mul_fft(a, b, variant=""):
    a, b = _c(a), _c(b)
    out = np.zeros(max(len(a) + len(b), 1), dtype=np.uint64)
    err = ctypes.c_double(0.0)
    ref_lib(variant).ref_mul_fft(_ptr(a), len(a), _ptr(b), len(b), _ptr(out), ctypes.byref(err))
    return out[: len(a) + len(b)], err.value


def to_int(a) -> int:
    """Python integer of a limb vector (for small cross-checks)."""
    return int.from_bytes(_c(a).tobytes(), "little")


def from_int(x: int, n: int) -> np.ndarray:
    return np.frombuffer(x.to_bytes(8 * n, "little"), dtype=np.uint64).copy()
