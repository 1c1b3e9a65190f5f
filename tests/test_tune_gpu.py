"""GPU parity of every kernel configuration the autotuner can choose
(column/row split, columns per CTA, column radix cap, rows per CTA,
per-prime streams), and of products after tuning."""
import itertools

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _reset(gpu):
    gpu.tune_reset()
    yield
    gpu.tune_reset()


def _configs(gpu, k):
    out = []
    for k1, cg, cmr, rmr, rows, split in itertools.product(range(5, 14), (4, 8), (4, 6), (4, 6), (1, 2, 4, 8, 16, 32),
                                                           (0, 1)):
        cfg = dict(log2_n=k, log2_cols=k1, col_group=cg, col_radix_cap=cmr, row_radix_cap=rmr, rows_per_cta=rows,
                   split_primes=split)
        try:
            gpu.tune_set(**cfg)
        except gpu.PrecGpuError:
            continue
        out.append(cfg)
    gpu.tune_reset()
    return out


@pytest.mark.parametrize("wide", [False, True])
@pytest.mark.parametrize("k", [13, 16, 20, 22])
def test_every_config_bit_exact(gpu, k, wide):
    """Every kernel configuration of a length, on 32-bit digits and on 64-bit
    digits (the same kernels on five primes' residues)."""
    if wide and k < 18:
        pytest.skip("64-bit digits start at 2^18 points")
    n = 1 << (k - 2)
    if wide:  # both operands within the lower half of 2^k points of 64-bit digits
        shapes = [(2 * n, 2 * n), (2 * n, n + 1)]
    else:  # balanced, and one operand above N/2 digits
        shapes = [(n, n), (n + n // 2 - 3, n // 2 + 1)]
    cases = []
    for an, bn in shapes:
        a = O.splitmix64(k * 7 + an, an)
        b = O.splitmix64(k * 11 + bn, bn)
        cases.append((a, b, O.mul_ntt(a, b)))
    cfgs = _configs(gpu, k)
    assert len(cfgs) >= 8
    prev = gpu.set_wide_digits(wide)
    try:
        for cfg in cfgs:
            gpu.tune_set(**cfg)
            for a, b, want in cases:
                got = gpu.mul(a, b, ntt=True)
                assert gpu.last_stats().log2_n == k
                assert np.array_equal(got, want), cfg
    finally:
        gpu.set_wide_digits(prev)
        gpu.tune_reset()


def _spot(p, a, b):
    O.spot_check(p, a, b, 91, fixed=(2305843009213693951, 4611686018427387847))


@pytest.mark.parametrize("wide", [False, True])
def test_prime_set_1_configs(gpu, wide):
    """2^24 points, rows of 2^13: every valid column configuration on set 1
    (the reference's primes, 32-bit digits) and on set 3 (five primes,
    64-bit digits), residue spot checks and agreement between configs."""
    k, n = 24, (3 << 20) if not wide else (3 << 21)
    a = O.splitmix64(91, n)
    b = O.splitmix64(92, n)
    ref = None
    prev = gpu.set_wide_digits(wide)
    try:
        for cfg in _configs(gpu, k):
            gpu.tune_set(**cfg)
            p = gpu.mul(a, b, ntt=True)
            assert gpu.last_stats().log2_n == k
            assert gpu.last_stats().primes == (5 if wide else 3)
            if ref is None:
                _spot(p, a, b)
                ref = p
            else:
                assert np.array_equal(p, ref), cfg
    finally:
        gpu.set_wide_digits(prev)


def test_autotune_installs_exact_configs(gpu, tmp_path):
    res = gpu.autotune(13, 21)
    assert [r["log2_n"] for r in res] == list(range(13, 22))
    for r in res:
        assert 0 < r["ms"] <= r["default_ms"] * 1.0001
        cur = gpu.tune_get(r["log2_n"])
        assert cur["log2_cols"] == r["log2_cols"] and cur["rows_per_cta"] == r["rows_per_cta"]
    for k in (13, 17, 21):
        n = 1 << (k - 2)
        a = O.splitmix64(k, n)
        b = O.splitmix64(k + 1, n - 5)
        assert np.array_equal(gpu.mul(a, b, ntt=True), O.mul_ntt(a, b)), k
    path = str(tmp_path / "t.txt")
    gpu.tune_save(path)
    gpu.tune_reset()
    gpu.tune_load(path)
    assert gpu.tune_get(21)["ms"] == pytest.approx(res[-1]["ms"], rel=1e-5)
