"""GPU test of prec_gpu_mul_device_noalloc, the entry point for callers that
cannot allocate device memory (their memory belongs to their own pool
allocator, they cannot take cudaFree's device-wide synchronisation, or
their host forbids allocation after start-up).

Through the C ABI, two calls in a row of the no-allocation entry point must
give exactly the limbs of the allocating entry point prec_gpu_mul_device
(the tolerance of every product test here: bit-exact).  The file is named
to be collected last, and it sets up everything it uses, so it passes in a
fresh process and after the other tests alike.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint64).view(np.int64)).cuda()


def test_noalloc_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    from preclib_gb300 import native, workloads
    L = native.lib()
    stream = torch.cuda.current_stream().cuda_stream
    # a four-step product (2^18 points, the largest allowed) and a single-CTA one
    for (an, bn, seed) in ((65536, 65535, 41), (1000, 777, 43)):
        a = workloads.operand(seed, an)
        b = workloads.operand(seed + 1, bn)
        ta, tb = _dev(torch, a), _dev(torch, b)
        want = torch.empty(an + bn, dtype=torch.int64, device="cuda")
        native.check(L.prec_gpu_mul_device(ta.data_ptr(), an, tb.data_ptr(), bn, want.data_ptr(), stream))
        native.stream_check(stream)
        for call in range(2):  # two calls in a row share the static scratch
            got = torch.full((an + bn,), -1, dtype=torch.int64, device="cuda")
            rc = L.prec_gpu_mul_device_noalloc(ta.data_ptr(), an, tb.data_ptr(), bn, got.data_ptr(), stream)
            assert rc == native.OK, native.strerror(rc)
            torch.cuda.synchronize()
            assert torch.equal(got, want), (an, bn, call)
