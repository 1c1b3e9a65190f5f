"""GPU parity of the FP64 FFT band (193..6144 limbs) through the C ABI:
bit-exact against the reference-generated golden vectors and the oracle,
with the per-product rounding distance reported and bounded."""
import hashlib
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle as O
import patterns

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _digest(out):
    return hashlib.sha256(np.ascontiguousarray(out, dtype="<u8").tobytes()).hexdigest()


def test_golden_vectors_fft_band(gpu, golden):
    """Every golden product whose operands fit the band, through mul_fft."""
    n = 0
    for rec in golden:
        g = rec["gen"]
        if max(g["an"], g["bn"]) > 6144:
            continue
        a, b = patterns.make(g)
        if rec["ref_fn"] == "sqr":
            b = a
        out = gpu.mul(a, b, fft=True)
        assert _digest(out) == rec["sha256"], rec["name"]
        st = gpu.last_stats()
        if len(a) and len(b) and (np.any(a) and np.any(b)):
            assert st.path == 2, rec["name"]
            assert 0.0 <= st.fft_max_distance <= 0.25, rec["name"]
        n += 1
    assert n > 150


def test_torture_fft_band(gpu):
    """fft_torture's shapes x patterns within the band; distances stay far
    below the reference's own worst case (0.2539 with 16-bit digits)."""
    worst = 0.0
    for (an, bn) in patterns.TORTURE_SHAPES:
        if max(an, bn) > 6144:
            continue
        for p in patterns.TORTURE_PATTERNS:
            a, b = patterns.torture(p[0], an, bn)
            if len(a) == 0 or len(b) == 0:
                continue
            got = gpu.mul(a, b, fft=True)
            assert np.array_equal(got, O.mul_ntt(a, b)), (p[0], an, bn)
            worst = max(worst, gpu.last_stats().fft_max_distance)
    assert worst < 0.125, worst


@pytest.mark.parametrize("an,bn", [(193, 193), (200, 150), (255, 256), (1000, 999), (1024, 1024),
                                   (1025, 1025), (2049, 2039), (3000, 3000), (4095, 4097),
                                   (6144, 6144), (6144, 3100), (6144, 10)])
def test_random_fft_band(gpu, an, bn):
    a = O.splitmix64(an * 3 + bn, an)
    b = O.splitmix64(an * 5 + bn + 7, bn)
    got = gpu.mul(a, b, fft=True)
    assert np.array_equal(got, O.mul_ntt(a, b))
    st = gpu.last_stats()
    assert st.path == 2 and 0 < st.fft_max_distance < 0.125


def test_band_routing(gpu):
    """prec_gpu_mul: <=192 limbs and >6144 limbs -> NTT, otherwise FP64."""
    for (an, bn, path) in ((100, 90, 0), (193, 10, 2), (6144, 6144, 2), (6145, 6145, 1), (20000, 15000, 1)):
        a = O.splitmix64(an, an)
        b = O.splitmix64(bn + 1, bn)
        got = gpu.mul(a, b)
        assert np.array_equal(got, O.mul(a, b))
        assert gpu.last_stats().path == path, (an, bn)


def test_square_above_band_goes_to_ntt(gpu):
    """precn_sqr sends squares above 192 limbs to mul_fft (src/mul_basic.cpp:203);
    above 6144 limbs the GPU mul_fft runs them on the NTT kernels."""
    a = O.splitmix64(77, 9000)
    got = gpu.mul(a, a, fft=True)
    assert np.array_equal(got, O.mul_ntt(a, a))
    assert gpu.last_stats().path == 1


def test_rounding_failure_leaves_output_untouched():
    """With a forced 24-bit digit width (coefficients near 2^50, far past
    what FP64 rounds exactly) the FP64 band cannot round correctly: the call
    must return PREC_GPU_E_FFT_ROUNDING, report the distance and leave the
    output buffer as it was (run in a child process so the test knob stays
    local)."""
    code = r'''
import sys, numpy as np
sys.path.insert(0, %r)
from preclib_gb300 import native
import oracle as O
native.init(0)
a = O.splitmix64(1, 1000); b = O.splitmix64(2, 1000)
out = np.full(2000, 0x5A5A5A5A5A5A5A5A, dtype=np.uint64)
rc = native.lib().prec_gpu_mul_fft(native._p(a), 1000, native._p(b), 1000, native._p(out))
st = native.last_stats()
assert rc == native.E_FFT_ROUNDING, (rc, st.fft_max_distance)
assert st.fft_max_distance > 0.25, st.fft_max_distance
assert (out == 0x5A5A5A5A5A5A5A5A).all()
print("ok")
''' % ROOT
    env = dict(os.environ, PREC_GPU_FFT_DIGIT_BITS="24")
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "ok" in r.stdout, r.stdout + r.stderr
