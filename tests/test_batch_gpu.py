"""GPU tests of the batch form: many device-resident products of uneven
sizes planned into length classes, captured into a CUDA graph and replayed;
every product bit-exact against the single-product path and, for a sample,
the oracle."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _sizes(seed, count, lo_max=70000):
    rng = np.random.default_rng(seed)
    lo = np.rint(np.exp(rng.uniform(0, np.log(lo_max), count))).astype(np.int64)
    hi = np.rint(lo * rng.uniform(1.0, 3.0, count)).astype(np.int64)
    sizes = [(int(l), int(h)) if rng.random() < 0.5 else (int(h), int(l)) for l, h in zip(lo, hi)]
    sizes[0] = (0, 17)  # a zero-length operand
    sizes[1] = (1, 1)
    return sizes


class DevBatch:
    """Operands and outputs of a batch packed into one device buffer each."""

    def __init__(self, torch, sizes, seed):
        self.torch = torch
        self.sizes = sizes
        tot_in = sum(a + b for a, b in sizes)
        self.inp = torch.empty(max(tot_in, 1), dtype=torch.int64, device="cuda")
        self.out = torch.empty(max(tot_in, 1), dtype=torch.int64, device="cuda")
        self.off = []
        o = 0
        for a, b in sizes:
            self.off.append(o)
            o += a + b
        self.fill(seed)

    def fill(self, seed):
        host = np.concatenate([O.splitmix64(seed + i, a + b) for i, (a, b) in enumerate(self.sizes)] or
                              [np.zeros(1, np.uint64)])
        self.host = host
        self.inp.copy_(self.torch.from_numpy(host.view(np.int64)))

    def items(self):
        base_i, base_o = self.inp.data_ptr(), self.out.data_ptr()
        return [(base_i + 8 * o, a, base_i + 8 * (o + a), b, base_o + 8 * o)
                for o, (a, b) in zip(self.off, self.sizes)]

    def operands(self, i):
        o, (a, b) = self.off[i], self.sizes[i]
        return self.host[o:o + a], self.host[o + a:o + a + b]

    def result(self, i):
        o, (a, b) = self.off[i], self.sizes[i]
        return self.out[o:o + a + b].cpu().numpy().view(np.uint64)


def _plain(gpu, torch, db, i):
    a, b = db.operands(i)
    if len(a) == 0 or len(b) == 0:
        return np.zeros(len(a) + len(b), np.uint64)
    ta = torch.from_numpy(a.view(np.int64)).cuda()
    tb = torch.from_numpy(b.view(np.int64)).cuda()
    to = torch.empty(len(a) + len(b), dtype=torch.int64, device="cuda")
    gpu.mul_device(ta.data_ptr(), len(a), tb.data_ptr(), len(b), to.data_ptr())
    gpu.stream_check()
    return to.cpu().numpy().view(np.uint64)


def test_batch_graph_and_replay(gpu):
    torch = pytest.importorskip("torch")
    sizes = _sizes(11, 220)
    db = DevBatch(torch, sizes, 1000)
    batch = gpu.Batch(db.items())
    ncls, nbytes = batch.info()
    assert ncls >= 8
    stream = torch.cuda.current_stream().cuda_stream
    for rnd in range(2):
        if rnd:
            db.fill(5000)  # new operand values, same buffers: the graph replays
        db.out.fill_(-1)
        batch.run(stream)
        gpu.stream_check(stream)
        for i in range(len(sizes)):
            got = db.result(i)
            assert np.array_equal(got, _plain(gpu, torch, db, i)), (rnd, i, sizes[i])
        for i in range(0, len(sizes), 11):
            a, b = db.operands(i)
            if len(a) and len(b):
                assert np.array_equal(db.result(i), O.mul_ntt(a, b)), (rnd, i, sizes[i])
    batch.close()


def test_batch_one_shot_and_chunking(gpu, monkeypatch):
    """The one-shot form, with a tiny workspace budget so that every
    four-step class runs in several chunks."""
    torch = pytest.importorskip("torch")
    monkeypatch.setenv("PREC_GPU_BATCH_CLASS_BYTES", str(40 << 20))
    sizes = _sizes(12, 120, lo_max=120000)
    db = DevBatch(torch, sizes, 77)
    db.out.fill_(-1)
    gpu.mul_batch(db.items(), torch.cuda.current_stream().cuda_stream)
    for i in range(len(sizes)):
        assert np.array_equal(db.result(i), _plain(gpu, torch, db, i)), (i, sizes[i])


def test_config3_workload_tuned_vs_oracle(gpu):
    """The batch benchmark's workload (4096 products, lo log-uniform in
    [200, 65536] limbs, hi = lo * U[1, 2], SplitMix64 seed 7) after the
    autotuner picked its length classes' kernels: a seeded sample of 64
    products equals the oracle, and every product equals the plain path."""
    torch = pytest.importorskip("torch")
    from preclib_gb300 import workloads
    lo, hi = workloads.batch_sizes(7, 4096)
    sizes = [(int(h), int(l)) for l, h in zip(lo, hi)]
    try:
        gpu.autotune(13, max(gpu.ntt_log2(a, b) for a, b in sizes))
        db = DevBatch(torch, sizes, 7)
        b = gpu.Batch(db.items())
        b.run()
        gpu.stream_check()
        b.close()
        rng = np.random.default_rng(7)
        for i in sorted(rng.choice(len(sizes), size=64, replace=False).tolist()):
            a_, b_ = db.operands(i)
            assert np.array_equal(db.result(i), O.mul_ntt(a_, b_)), sizes[i]
        out = db.out.cpu().numpy().view(np.uint64)
        for i in range(0, len(sizes), 97):
            o, (a_, b_) = db.off[i], sizes[i]
            assert np.array_equal(out[o:o + a_ + b_], _plain(gpu, torch, db, i)), sizes[i]
    finally:
        gpu.tune_reset()


def test_batch_both_digit_widths(gpu):
    """The same batch planned with 64-bit digits allowed (classes of five
    primes where the shapes fit) and with 32-bit digits only: identical
    limbs, and a sample equals the oracle."""
    torch = pytest.importorskip("torch")
    sizes = _sizes(13, 150, lo_max=200000)
    db = DevBatch(torch, sizes, 31)
    outs = []
    for wide in (False, True):
        prev = gpu.set_wide_digits(wide)
        try:
            db.out.fill_(-1)
            b = gpu.Batch(db.items())
            b.run()
            gpu.stream_check()
            b.close()
            outs.append(db.out.cpu().numpy().copy())
        finally:
            gpu.set_wide_digits(prev)
    assert np.array_equal(outs[0], outs[1])
    for i in range(0, len(sizes), 13):
        a, b = db.operands(i)
        if len(a) and len(b):
            assert np.array_equal(db.result(i), O.mul_ntt(a, b)), sizes[i]
