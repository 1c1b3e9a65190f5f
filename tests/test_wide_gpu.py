"""GPU parity of the 64-bit-digit plan (prime set 2: whole limbs as digits,
five primes, half the points of the 32-bit-digit transform) through the C
ABI: the shapes at the edges of its range, against the oracle and against
the 32-bit-digit plan."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

B1 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _mul(gpu, a, b, wide):
    prev = gpu.set_wide_digits(wide)
    try:
        out = gpu.mul(a, b, ntt=True)
        return out, gpu.last_stats().log2_n
    finally:
        gpu.set_wide_digits(prev)


# (an, bn, transform log2 with 64-bit digits allowed)
EDGES = [
    (1 << 16, 1 << 16, 18),        # 2^17 coefficients: 2^17 points would be below 2^18, 32-bit digits
    (1 << 17, 1 << 17, 18),        # the first 64-bit-digit length, both operands exactly half
    ((1 << 17) + 1, 1 << 17, 20),  # one operand above half: 32-bit digits (2^19 + 2 coefficients)
    (1 << 17, 1, 19),              # 2^17 coefficients: 32-bit digits
    (1 << 17, 2, 18),              # 2^17 + 1 coefficients, a at exactly half: 64-bit digits
    (130000, 100000, 18),
    (200000, 50001, 19),           # unbalanced: 32-bit digits
    (65537, 65535, 18),
]


@pytest.mark.parametrize("an,bn,k", EDGES)
def test_edges_vs_oracle(gpu, an, bn, k):
    a = O.splitmix64(an + 7, an)
    b = O.splitmix64(bn + 11, bn)
    a[-1] |= np.uint64(1 << 63)
    b[-1] |= np.uint64(1 << 63)
    got, kk = _mul(gpu, a, b, True)
    assert kk == k
    assert np.array_equal(got, O.mul_ntt(a, b))


def test_random_shapes_both_widths(gpu):
    """Random shapes 70000 .. 400000 limbs, random and all-ones-heavy
    operands: the two digit widths agree, and agree with the oracle."""
    rng = np.random.default_rng(2024)
    for t in range(12):
        an = int(np.exp(rng.uniform(np.log(70000), np.log(400000))))
        bn = int(np.exp(rng.uniform(np.log(70000), np.log(400000)))) if t % 3 else an
        a = O.splitmix64(1000 + t, an)
        b = O.splitmix64(2000 + t, bn)
        if t % 4 == 0:
            a[: an // 2] = np.uint64(0xFFFFFFFFFFFFFFFF)
            b[bn // 3:] = np.uint64(0xFFFFFFFFFFFFFFFF)
        wide, _ = _mul(gpu, a, b, True)
        narrow, _ = _mul(gpu, a, b, False)
        assert np.array_equal(wide, narrow), (an, bn)
        assert np.array_equal(wide, O.mul_ntt(a, b)), (an, bn)


def test_large_both_widths(gpu):
    """2^19 .. 2^24-point products (sets 2 and 3 against sets 0 and 1):
    64-bit and 32-bit digits bit for bit."""
    for (an, bn) in ((1 << 18, 1 << 18), (3 << 18, 1 << 20), (1 << 20, 999999), (1 << 21, 1 << 21),
                     (1 << 22, 1 << 22), (3 << 21, 1 << 22)):
        a = O.splitmix64(an, an)
        b = O.splitmix64(bn + 3, bn)
        wide, kw = _mul(gpu, a, b, True)
        narrow, kn = _mul(gpu, a, b, False)
        assert kw == kn - 1, (an, bn)
        assert np.array_equal(wide, narrow), (an, bn)


def test_all_ones_square_set3_bound(gpu):
    """(2^(64n) - 1)^2 at n = 2^24 (2^25 points on set 3): the largest
    single-transform square, coefficients up to 2^24 (2^64 - 1)^2."""
    n = 1 << 24
    a = np.full(n, B1)
    got = gpu.sqr(a)
    st = gpu.last_stats()
    assert st.log2_n == 25 and st.primes == 5
    assert got[0] == 1 and not got[1:n].any()
    assert got[n] == np.uint64(0xFFFFFFFFFFFFFFFE) and (got[n + 1:] == B1).all()


def test_all_ones_unbalanced(gpu):
    """(B^n - 1)(B^m - 1) = B^(n+m) - B^n - B^m + 1 (B = 2^64), n > m:
    limbs 1, 0 .. 0 (to m), B-1 .. B-1 (to n), B-2, B-1 .. B-1."""
    B1 = np.uint64(0xFFFFFFFFFFFFFFFF)
    for (n, m) in ((1 << 20, 600000), (1 << 20, (1 << 20) - 1), (70000, 40000)):
        a = np.full(n, B1)
        b = np.full(m, B1)
        want = np.zeros(n + m, np.uint64)
        want[0] = 1
        want[m:n] = B1
        want[n] = np.uint64(0xFFFFFFFFFFFFFFFE)
        want[n + 1:] = B1
        got, k = _mul(gpu, a, b, True)
        assert np.array_equal(got, want), (n, m, k)
