"""CPU tests of the boundary: the C ABI library loads, exports every symbol
its header declares, and its host-side plan logic answers without a GPU."""
import os
import re

import numpy as np
import pytest

from preclib_gb300 import native, workloads

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(prec_gpu_\w+)\s*\(", src))
    return names


def test_header_symbols_exported():
    lib = native.lib()
    declared = _declared()
    assert declared, "no declarations found"
    for name in sorted(declared):
        assert hasattr(lib, name), name
    assert declared <= set(native.EXPORTS) | declared


def test_python_binding_covers_header():
    assert _declared() == set(native.EXPORTS)


def test_ntt_plan_sizes():
    prev = native.set_wide_digits(False)
    try:
        # 32-bit digits: 2^k >= da + db - 1 digits
        assert native.ntt_log2(8192, 8192) == 15
        assert native.ntt_log2(1 << 20, 1 << 20) == 22
        assert native.ntt_log2(3000, 3000) == 14
        assert native.ntt_log2(1, 1) == 5
        assert native.ntt_log2(1 << 24, 1 << 24) == 26
        assert native.ntt_log2(1 << 24, (1 << 24) + 1) == 0  # beyond the 2^26-point transform
        native.set_wide_digits(True)
        # 64-bit digits from 2^18 to 2^25 points, both operands in the lower half
        assert native.ntt_log2(8192, 8192) == 15
        assert native.ntt_log2(1 << 16, 1 << 16) == 18
        assert native.ntt_log2(1 << 17, 1 << 17) == 18
        assert native.ntt_log2(1 << 20, 1 << 20) == 21
        assert native.ntt_log2(1 << 21, 1 << 21) == 22
        assert native.ntt_log2(3000, 3000) == 14
        assert native.ntt_log2(1 << 20, 1000) == 21
        # one operand above half the 64-bit-digit transform: 32-bit digits
        assert native.ntt_log2(3 << 19, 1 << 19) == 22
        # 2^23 .. 2^25 points: the second five-prime set
        assert native.ntt_log2(1 << 22, 1 << 22) == 23
        assert native.ntt_log2(1 << 24, 1 << 24) == 25
        assert native.ntt_log2(3 << 22, 1 << 22) == 25  # one operand above half: 32-bit digits
        # small transforms: 32-bit digits
        assert native.ntt_log2(1500, 1500) == 13
        assert native.ntt_log2(1, 1) == 5
    finally:
        native.set_wide_digits(prev)


def test_strerror():
    assert native.strerror(0) == "ok"
    assert "0.25" in native.strerror(native.E_FFT_ROUNDING)


def test_splitmix_matches_oracle():
    import oracle as O
    for seed in (1, 2, 12345):
        assert np.array_equal(workloads.splitmix64(seed, 1000), O.splitmix64(seed, 1000))


def test_batch_sizes_shape():
    lo, hi = workloads.batch_sizes(7, 4096)
    assert lo.min() >= 200 and lo.max() <= 65536
    assert (hi >= lo).all() and (hi <= 2 * lo).all()


def test_no_device_fails_loudly():
    """Without a usable device the library reports E_NODEV (no CPU fallback)."""
    rc = native.lib().prec_gpu_init(0)
    if rc == native.OK:
        pytest.skip("a CUDA device is present")
    assert rc == native.E_NODEV
    with pytest.raises(native.PrecGpuError):
        native.mul(np.ones(3, np.uint64), np.ones(3, np.uint64))


def test_block_limbs():
    """Products with an operand above the block size run blocked (no single
    transform length); the size is clamped to [1024, 2^24]."""
    prev = native.set_block_limbs(4096)
    try:
        assert native.ntt_log2(4097, 10) == 0
        assert native.ntt_log2(4096, 4096) > 0
        assert native.set_block_limbs(10) == 4096
        assert native.set_block_limbs(0) == 1024
        assert native.set_block_limbs(1 << 30) == 1 << 24
        assert native.ntt_log2((1 << 24) + 1, 5) == 0
        assert native.ntt_log2(1 << 24, 5) > 0
    finally:
        native.set_block_limbs(prev)


def test_noalloc_rejects_oversize():
    """The no-allocation entry point refuses more than 131072 limbs from the
    sizes alone, before any CUDA call and before it looks at the pointers
    (so this runs without a device, with null pointers).  Sizes whose sum
    or doubled sum wraps 64 bits are refused the same way."""
    L = native.lib()
    for an, bn in ((65537, 65536), (1 << 63, 1), (1, 1 << 63), ((1 << 64) - 1, 2), (131072, 1), (131073, 0)):
        assert L.prec_gpu_mul_device_noalloc(None, an, None, bn, None, None) == native.E_TOO_LARGE, (an, bn)
    # within the limit, the null pointers are the error
    assert L.prec_gpu_mul_device_noalloc(None, 65536, None, 65536, None, None) == native.E_ARG
    assert L.prec_gpu_mul_device_noalloc(None, 0, None, 0, None, None) == native.E_ARG


def _fft_bound(b, k):
    """Error bound of an FP64 convolution of 2^k points on b-bit digits (the
    library's rule: |x||y| <= N 2^(2b-2), e = 2^-53, beta = 2^-52, doubled
    for the two operands packed in one complex transform)."""
    import math
    e, beta = 2.0 ** -53, 2.0 ** -52
    g = math.expm1(3 * k * math.log1p(e) + (3 * k + 1) * math.log1p(e * math.sqrt(5)) + 3 * k * math.log1p(beta))
    return 2.0 * 2.0 ** (k + 2 * b - 2) * g


def _fft_width(an, bn):
    for b in range(16, 7, -1):
        da, db = (64 * an + b - 1) // b + 1, (64 * bn + b - 1) // b + 1
        k = 6
        while (1 << k) < da + db - 1:
            k += 1
        if k <= 16 and _fft_bound(b, k) < 0.25:
            return b
    return 0


def test_fft_digit_width_rule():
    """The FP64 band takes the widest digit (16 .. 8 bits) whose error bound
    stays below 1/4 on a transform of at most 2^16 points; outside the band
    (0 or above 6144 limbs) it reports 0."""
    import random
    rng = random.Random(5)
    shapes = [(1, 1), (193, 193), (1000, 1000), (3000, 3000), (6144, 6144), (6144, 10), (200, 6144),
              (2048, 2048), (2049, 2039), (4096, 4096)]
    shapes += [(rng.randrange(1, 6145), rng.randrange(1, 6145)) for _ in range(200)]
    for an, bn in shapes:
        assert native.fft_digit_bits(an, bn) == _fft_width(an, bn), (an, bn)
    assert native.fft_digit_bits(3000, 3000) == 14  # the config-2 FFT product
    assert native.fft_digit_bits(6145, 6145) == 0
    assert native.fft_digit_bits(0, 100) == 0
