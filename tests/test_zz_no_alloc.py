"""GPU test of prec_gpu_mul_device_noalloc, the entry point for callers that
cannot allocate device memory (their memory belongs to their own pool
allocator, they cannot take cudaFree's device-wide synchronisation, or
their host forbids allocation after start-up).

Through the C ABI, two calls in a row of the no-allocation entry point must
give exactly the limbs of the allocating entry point prec_gpu_mul_device and
of the oracle (the tolerance of every product test here: bit-exact), on the
single-CTA path and on four-step lengths 2^13, 2^16 and 2^18 (the largest
allowed), and for a square passed as one buffer twice.  After the calls,
prec_gpu_stream_check reports the kernels' error word clear.  The file is
named to be collected last, and it sets up everything it uses, so it passes
in a fresh process and after the other tests alike.
"""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint64).view(np.int64)).cuda()


@pytest.mark.parametrize("an,bn,seed,square", [
    (65536, 65535, 41, False),   # 2^18 points, the largest product allowed
    (1000, 777, 43, False),      # single-CTA kernel (2^12 points)
    (3000, 1000, 45, False),     # 2^13 points: the shortest four-step length
    (16000, 16000, 47, False),   # 2^16 points
    (20000, 20000, 49, True),    # a square: one buffer for both operands
])
def test_noalloc_matches_allocating_entry_point(an, bn, seed, square):
    torch = pytest.importorskip("torch")
    from preclib_gb300 import native, workloads
    L = native.lib()
    stream = torch.cuda.current_stream().cuda_stream
    a = workloads.operand(seed, an)
    b = a if square else workloads.operand(seed + 1, bn)
    ta = _dev(torch, a)
    tb = ta if square else _dev(torch, b)
    want = torch.empty(an + bn, dtype=torch.int64, device="cuda")
    native.check(L.prec_gpu_mul_device(ta.data_ptr(), an, tb.data_ptr(), bn, want.data_ptr(), stream))
    native.stream_check(stream)
    ref = O.mul_ntt(a, b)
    assert np.array_equal(want.cpu().numpy().view(np.uint64), ref)
    for call in range(2):  # two calls in a row share the static scratch
        got = torch.full((an + bn,), -1, dtype=torch.int64, device="cuda")
        rc = L.prec_gpu_mul_device_noalloc(ta.data_ptr(), an, tb.data_ptr(), bn, got.data_ptr(), stream)
        assert rc == native.OK, native.strerror(rc)
        # synchronises and reads (then clears) the kernels' error word
        assert L.prec_gpu_stream_check(stream) == native.OK
        assert torch.equal(got, want), (an, bn, call)
        assert np.array_equal(got.cpu().numpy().view(np.uint64), ref), (an, bn, call)
