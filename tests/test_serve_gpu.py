"""GPU tests of the serving loop: requests of uneven sizes submitted while
others run are admitted by HBM footprint, overlap on the device, and each
result is bit-identical to the same product run alone."""
import threading
import time

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _setup(torch, sizes, seed):
    tot = sum(a + b for a, b in sizes)
    host = O.splitmix64(seed, tot)
    d_in = torch.from_numpy(host.view(np.int64)).cuda()
    d_out = torch.full((tot,), -1, dtype=torch.int64, device="cuda")
    offs, o = [], 0
    for a, b in sizes:
        offs.append(o)
        o += a + b
    bi, bo = d_in.data_ptr(), d_out.data_ptr()
    items = [(bi + 8 * off, a, bi + 8 * (off + a), b, bo + 8 * off) for off, (a, b) in zip(offs, sizes)]
    return host, d_in, d_out, offs, items


def _alone(gpu, torch, it):
    a_ptr, an, b_ptr, bn, _ = it
    to = torch.empty(an + bn, dtype=torch.int64, device="cuda")
    gpu.mul_device(a_ptr, an, b_ptr, bn, to.data_ptr())
    gpu.stream_check()
    return to.cpu().numpy().view(np.uint64)


def test_mixed_equals_alone(gpu):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    sizes = [(int(s), int(s * rng.uniform(0.5, 1.0)) or 1)
             for s in np.rint(np.exp(rng.uniform(np.log(256), np.log(1 << 21), 60)))]
    sizes[3] = (1 << 22, 1 << 22)  # one very large request in the mix
    host, d_in, d_out, offs, items = _setup(torch, sizes, 99)
    torch.cuda.synchronize()
    # budget: room for the largest workspace plus a little, so admission queues
    srv = gpu.Server(hbm_budget_bytes=600 << 20, slots=6)
    tickets = []

    def producer():
        for it in items:
            tickets.append(srv.submit(*it))
            time.sleep(rng.exponential(0.0005))
    th = threading.Thread(target=producer)
    th.start()
    th.join()
    srv.drain(120)
    st = srv.stats()
    assert st.completed == len(items) and st.failed == 0
    assert st.peak_bytes <= 600 << 20
    assert st.peak_in_flight >= 2  # work overlapped on the device
    assert 0 < st.p50_ms <= st.p99_ms <= st.max_ms
    for t in tickets:
        assert srv.wait(t, 1.0) >= 0.0
    srv.close()
    for i, it in enumerate(items):
        off, (a, b) = offs[i], sizes[i]
        mixed = d_out[off:off + a + b].cpu().numpy().view(np.uint64)
        assert np.array_equal(mixed, _alone(gpu, torch, it)), (i, sizes[i])
    # and against the oracle for the small ones
    for i in range(0, len(items), 9):
        off, (a, b) = offs[i], sizes[i]
        if a + b <= 200000:
            mixed = d_out[off:off + a + b].cpu().numpy().view(np.uint64)
            assert np.array_equal(mixed, O.mul_ntt(host[off:off + a], host[off + a:off + a + b]))


def test_oversize_request_refused(gpu):
    torch = pytest.importorskip("torch")
    srv = gpu.Server(hbm_budget_bytes=1 << 20, slots=2)
    # real device buffers: the refusal is the host's, but no kernel could
    # ever be handed an address that is not device memory
    da = torch.zeros(1 << 20, dtype=torch.int64, device="cuda")
    db = torch.zeros(1 << 20, dtype=torch.int64, device="cuda")
    dout = torch.zeros(2 << 20, dtype=torch.int64, device="cuda")
    with pytest.raises(gpu.PrecGpuError) as e:
        # needs ~100 MB of workspace; refused on the host
        srv.submit(da.data_ptr(), 1 << 20, db.data_ptr(), 1 << 20, dout.data_ptr())
    assert e.value.code == gpu.E_NOMEM
    srv.close()
