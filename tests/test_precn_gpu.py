"""GPU parity of the interposer (preclib_gb300/precn/prec_gpu_precn.cpp):
preclib-style precn_t calls of mul_ntt / mul_fft return the reference's
exact, normalised products, squares through one object, zero in preclib's
form, and mul_fft's COUNT_FFTS statistics from the library's distances."""
import ctypes

import numpy as np
import pytest

import oracle as O
from precn_shim import shim

pytestmark = pytest.mark.gpu
_u64p = ctypes.POINTER(ctypes.c_uint64)


@pytest.fixture(scope="module")
def S(gpu, tmp_path_factory):
    return shim.load(shim.build(str(tmp_path_factory.mktemp("precn"))))


def _call(S, which, a, b, square=False):
    a = np.ascontiguousarray(a, np.uint64)
    b = a if square else np.ascontiguousarray(b, np.uint64)
    out = np.zeros(max(len(a) + len(b), 1), np.uint64)
    ok = ctypes.c_int(0)
    n = S.shim_mul(which, int(square), a.ctypes.data_as(_u64p), len(a), b.ctypes.data_as(_u64p), len(b),
                   out.ctypes.data_as(_u64p), ctypes.byref(ok))
    assert ok.value == 1
    return out[:n]


def _trim(x):
    nz = np.flatnonzero(x)
    return x[: nz[-1] + 1] if len(nz) else x[:0]


@pytest.mark.parametrize("an,bn", [(1, 1), (100, 57), (193, 193), (1024, 1000), (3000, 2999), (6144, 4000),
                                   (6145, 6145), (20000, 12001)])
def test_interposed_products(S, an, bn):
    a = O.splitmix64(an + 3, an)
    b = O.splitmix64(bn + 4, bn)
    want = _trim(O.mul_ntt(a, b))
    assert np.array_equal(_call(S, 0, a, b), want)
    assert np.array_equal(_call(S, 1, a, b), want)


@pytest.mark.parametrize("n", [150, 2048, 6144, 9000])
def test_interposed_square_one_object(S, n):
    a = O.splitmix64(n + 8, n)
    want = _trim(O.mul_ntt(a, a))
    assert np.array_equal(_call(S, 0, a, None, square=True), want)
    assert np.array_equal(_call(S, 1, a, None, square=True), want)


def test_interposed_zero_and_unnormalised_inputs(S):
    z = np.zeros(4, np.uint64)
    a = O.splitmix64(5, 300)
    assert len(_call(S, 0, z, a)) == 0
    assert len(_call(S, 1, a, z)) == 0
    padded = np.concatenate([a, np.zeros(7, np.uint64)])
    assert np.array_equal(_call(S, 1, padded, padded), _trim(O.mul_ntt(a, a)))


def test_interposed_fft_counters(S):
    """Every FP64-band product counts in total_fftmuls; the maximum distance
    stays below 1/4 (digit widths chosen by the error bound), so the
    1/4 and 3/8 danger counters stay at zero."""
    c0 = (ctypes.c_uint64 * 4)()
    e0 = ctypes.c_double()
    S.shim_fft_counters(c0, ctypes.byref(e0))
    ones = np.full(1024, np.uint64(0xFFFFFFFFFFFFFFFF))
    _call(S, 1, ones, ones)                   # FP64 band
    _call(S, 1, O.splitmix64(1, 3000), O.splitmix64(2, 3000))
    _call(S, 0, O.splitmix64(3, 3000), O.splitmix64(4, 3000))  # NTT band: not counted
    c1 = (ctypes.c_uint64 * 4)()
    e1 = ctypes.c_double()
    S.shim_fft_counters(c1, ctypes.byref(e1))
    assert c1[0] - c0[0] == 2
    assert c1[2] == c0[2] and c1[3] == c0[3]
    assert 0.0 < e1.value < 0.25
