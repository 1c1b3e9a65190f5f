"""CPU tests of the oracle: pinned to the reference's golden vectors and,
where the reference build exists, to the reference itself."""
import hashlib
import random

import numpy as np
import pytest

import oracle as O
import patterns


def _digest(out):
    return hashlib.sha256(np.ascontiguousarray(out, dtype="<u8").tobytes()).hexdigest()


def test_golden_vectors(golden):
    """Every reference-generated product is reproduced bit-exactly, and the
    FFT restatement reproduces the reference's rounding distances.  (The
    4M x 4M record, 12 s of oracle time, is pinned on the GPU path only:
    test_ntt_gpu.py.)"""
    for rec in golden:
        if rec["limbs"] > (1 << 21) + 2:
            continue
        a, b = patterns.make(rec["gen"])
        if rec["ref_fn"] == "sqr":
            out = O.mul_ntt(a, a)  # an exact square, whichever band made it
        elif rec["ref_fn"] == "ntt":
            out = O.mul_ntt(a, b)
        elif rec["ref_fn"] == "fft":
            out, err = O.mul_fft(a, b)
            assert err == rec["fft_max_err"], rec["name"]
        else:
            out = O.mul(a, b)
        assert len(out) == rec["limbs"]
        assert _digest(out) == rec["sha256"], rec["name"]


def test_torture_zone_counts(golden):
    """test/fft_torture.cpp over its 88 cases reports (run from the
    reference's sources) danger_fftmuls 8, danger_fftmuls_1_4 1,
    danger_fftmuls_3_8 0 and max_fft_rounding_error 0.25390625; the one
    product above 1/4 is all-ones 1024x1024 (16-bit digits)."""
    errs = {r["name"]: r["fft_max_err"] for r in golden
            if r["name"].startswith("torture_") and "fft_max_err" in r}
    assert len(errs) == 88
    assert sum(e > 0.125 for e in errs.values()) == 8
    assert [n for n, e in errs.items() if e > 0.25] == ["torture_all-ones_1024x1024_fft"]
    assert max(errs.values()) == 0.25390625


def test_kat_square_of_2_32_minus_1():
    """(2^32-1)^2 = 0xFFFFFFFE00000001 (test/test_prec.cpp:189-192)."""
    x = np.array([0xFFFFFFFF], dtype=np.uint64)
    for out in (O.mul_ntt(x, x), O.mul_fft(x, x)[0], O.mul_basic(x, x)):
        assert int(out[0]) == 0xFFFFFFFE00000001 and int(out[1]) == 0


def test_repunit_identity():
    """9 * R_1000 + 1 == 10^1000 (test/test_prec.cpp:417-427), products
    formed through the oracle's dispatcher by square-and-multiply."""
    def ints(v):
        n = max(1, (v.bit_length() + 63) // 64)
        return O.from_int(v, n)

    def mul(x, y):
        return O.to_int(O.mul(ints(x), ints(y)))

    def pow10(e):
        r, b = 1, 10
        while e:
            if e & 1:
                r = mul(r, b)
            b = mul(b, b)
            e >>= 1
        return r
    rep = (10 ** 1000 - 1) // 9
    assert mul(9, rep) + 1 == pow10(1000) == 10 ** 1000


@pytest.mark.parametrize("an,bn", [(1, 1), (3, 2), (24, 25), (193, 200), (1024, 1025), (1100, 2000),
                                   (6144, 6144), (6145, 6150), (9000, 4600)])
def test_oracle_bands_exact(an, bn):
    rng = np.random.default_rng(an * 7 + bn)
    a = rng.integers(0, 2 ** 64, an, dtype=np.uint64)
    b = rng.integers(0, 2 ** 64, bn, dtype=np.uint64)
    a[-1] |= np.uint64(1)
    b[-1] |= np.uint64(1)
    want = O.to_int(a) * O.to_int(b)
    assert O.to_int(O.mul_ntt(a, b)) == want
    assert O.to_int(O.mul_fft(a, b)[0]) == want
    assert O.to_int(O.mul(a, b)) == want
    if an * bn <= 1 << 22:
        assert O.to_int(O.mul_basic(a, b)) == want


def test_mod_spot_check():
    a = O.splitmix64(9, 5000)
    b = O.splitmix64(10, 4000)
    p = O.mul_ntt(a, b)
    for q in (2305843009213693951, 4611686018427387847, 1152921504606846883):
        assert O.mod_u64(p, q) == O.mod_u64(a, q) * O.mod_u64(b, q) % q


@pytest.mark.skipif(O.ref_lib() is None, reason="reference build absent (oracle/_ref)")
def test_oracle_matches_reference_random():
    """Restatement vs the reference compiled from its own sources."""
    rnd = random.Random(1234)
    for trial in range(40):
        an = rnd.choice([rnd.randint(1, 300), rnd.randint(193, 6144), rnd.randint(6145, 40000)])
        bn = max(1, int(an * rnd.uniform(0.5, 1.0)))
        a = O.splitmix64(trial * 2 + 100, an)
        b = O.splitmix64(trial * 2 + 101, bn)
        if trial % 5 == 0:
            a[-1] = 1  # short top limb
        assert np.array_equal(O.mul_ntt(a, b), O.ref_mul_ntt(a, b))
        fo, fe = O.mul_fft(a, b)
        ro, re = O.ref_mul_fft(a, b)
        assert np.array_equal(fo, ro) and fe == re
        assert np.array_equal(O.mul(a, b), O.ref_mul(a, b))


def test_random_primes61_and_spot_check():
    """The spot check's moduli are primes in [2^60, 2^61), fixed by the seed,
    and the check catches a single flipped bit of a product."""
    qs = O.random_primes61(5, 8)
    assert qs == O.random_primes61(5, 8) and len(set(qs)) == 8
    assert all((1 << 60) <= q < (1 << 61) and O.is_prime_u64(q) for q in qs)
    # composites that fool weaker tests: Carmichael numbers, strong pseudoprimes
    for n in (561, 1105, 3215031751, 2152302898747, 3474749660383, 341550071728321, 3825123056546413051):
        assert not O.is_prime_u64(n)
    assert [n for n in range(2, 60) if O.is_prime_u64(n)] == [2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43,
                                                              47, 53, 59]
    a, b = O.splitmix64(1, 300), O.splitmix64(2, 200)
    p = O.mul_basic(a, b)
    O.spot_check(p, a, b, 7, fixed=(2305843009213693951,))
    p[100] ^= np.uint64(1)
    with pytest.raises(AssertionError):
        O.spot_check(p, a, b, 7)
