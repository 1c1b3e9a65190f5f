"""GPU parity of squares (the reference's precn_sqr, src/mul_basic.cpp:193-204,
reached from operator* when both operands are the same object,
mul_basic.cpp:244-246): one operand transform per prime on the four-step
path, bit-exact against the oracle and the reference-generated vectors."""
import hashlib

import numpy as np
import pytest

import oracle as O
import patterns

pytestmark = pytest.mark.gpu


def _digest(out):
    return hashlib.sha256(np.ascontiguousarray(out, dtype="<u8").tobytes()).hexdigest()


def test_sqr_golden(gpu, golden):
    for rec in golden:
        if rec["ref_fn"] != "sqr":
            continue
        a, _ = patterns.make(rec["gen"])
        assert _digest(gpu.sqr(a)) == rec["sha256"], rec["name"]
        assert _digest(gpu.mul(a, a, ntt=True)) == rec["sha256"], rec["name"]


@pytest.mark.parametrize("n", [1, 2, 17, 192, 193, 1000, 2048, 2049, 6144, 6145, 8192, 10007,
                               32768, 65537, 131072, 300001])
def test_sqr_vs_oracle(gpu, n):
    a = O.splitmix64(7 * n + 1, n)
    want = O.mul_ntt(a, a)
    assert np.array_equal(gpu.sqr(a), want), n
    # a == b by pointer takes the square route in prec_gpu_mul too
    assert np.array_equal(gpu.mul(a, a, ntt=True), want), n
    # equal contents in separate arrays: the two-operand route, same result
    assert np.array_equal(gpu.mul(a, a.copy(), ntt=True), want), n


def test_sqr_each_length(gpu):
    """Every transform length 2^5 .. 2^21, both the single-CTA and the
    four-step kernels, squares of operands with the top bit set: 32-bit
    digits (2^k points for 2^(k-2) limbs), then 64-bit digits (2^(k-1)
    points from 2^18)."""
    for wide in (False, True):
        prev = gpu.set_wide_digits(wide)
        try:
            for k in range(5, 22):
                n = 1 << (k - 2)
                a = O.splitmix64(k + 500, n)
                a[-1] |= np.uint64(1 << 63)
                assert np.array_equal(gpu.mul(a, a, ntt=True), O.mul_ntt(a, a)), (wide, k)
                assert gpu.last_stats().log2_n == (k - 1 if wide and k >= 19 else k)
        finally:
            gpu.set_wide_digits(prev)


def test_sqr_all_ones(gpu):
    """(2^(64n) - 1)^2 = 2^(128n) - 2^(64n+1) + 1: maximal carries; at
    n = 2^21 the largest coefficient, n (2^64 - 1)^2, is within 2^0.16 of the
    five primes' product."""
    for n in (5000, 70000, 1 << 20, 1 << 21):
        a = np.full(n, np.uint64(0xFFFFFFFFFFFFFFFF))
        got = gpu.sqr(a)
        want = np.zeros(2 * n, np.uint64)
        want[0] = 1
        want[n] = np.uint64(0xFFFFFFFFFFFFFFFE)
        want[n + 1:] = np.uint64(0xFFFFFFFFFFFFFFFF)
        assert np.array_equal(got, want), n


def _spot(p, a, seed=3):
    O.spot_check(p, a, a, seed, fixed=(2305843009213693951, 4611686018427387847, 1152921504606846883))


def test_sqr_large_both_prime_sets(gpu):
    """2^22-point (prime set 0, 32-bit digits), 2^21- and 2^22-point (set 2,
    64-bit digits), 2^24 / 2^25-point (prime set 1, 32-bit digits) and
    2^23 / 2^24-point (set 3, 64-bit digits) squares."""
    for (n, s, k, wide) in ((1 << 20, 3, 22, False), (1 << 20, 3, 21, True), (1 << 21, 6, 22, True),
                            (3 << 20, 4, 24, False), (3 << 21, 5, 25, False), (3 << 20, 4, 23, True),
                            (3 << 21, 5, 24, True)):
        prev = gpu.set_wide_digits(wide)
        try:
            a = O.splitmix64(s, n)
            p = gpu.sqr(a)
            assert gpu.last_stats().log2_n == k
            _spot(p, a, s)
            assert p[-1] != 0
        finally:
            gpu.set_wide_digits(prev)


def test_sqr_device_same_pointer(gpu):
    torch = pytest.importorskip("torch")
    for n in (40000, 1 << 18, 300):
        a = O.splitmix64(n + 9, n)
        ta = torch.from_numpy(a.view(np.int64)).cuda()
        to = torch.empty(2 * n, dtype=torch.int64, device="cuda")
        gpu.mul_device(ta.data_ptr(), n, ta.data_ptr(), n, to.data_ptr())
        gpu.stream_check()
        assert np.array_equal(to.cpu().numpy().view(np.uint64), O.mul_ntt(a, a)), n


def test_sqr_in_batch(gpu):
    """Squares and products of one length class in one batch: the squares
    form their own class (one operand transform)."""
    torch = pytest.importorskip("torch")
    sizes = [(20000, True), (20000, False), (20001, True), (300, True), (70000, True)]
    ops, items, wants = [], [], []
    for i, (n, sq) in enumerate(sizes):
        a = O.splitmix64(100 + i, n)
        b = a if sq else O.splitmix64(200 + i, n)
        ta = torch.from_numpy(a.view(np.int64)).cuda()
        tb = ta if sq else torch.from_numpy(b.view(np.int64)).cuda()
        to = torch.empty(2 * n, dtype=torch.int64, device="cuda")
        ops.append((ta, tb, to))
        items.append((ta.data_ptr(), n, tb.data_ptr(), n, to.data_ptr()))
        wants.append(O.mul_ntt(a, b))
    gpu.mul_batch(items)
    for (ta, tb, to), want in zip(ops, wants):
        assert np.array_equal(to.cpu().numpy().view(np.uint64), want)
