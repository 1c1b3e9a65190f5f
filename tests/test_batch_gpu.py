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


def _mid_class_sizes(seed, count):
    """Products whose transforms have 2^13 .. 2^16 points on 32-bit digits
    (the persistent class kernel's classes), squares among them."""
    rng = np.random.default_rng(seed)
    sizes = []
    for i in range(count):
        k = 13 + i % 4
        # an + bn in (2^(k-2), 2^(k-1)]: 2*(an+bn) - 1 digits need 2^k points
        total = int(rng.integers((1 << (k - 2)) + 2, (1 << (k - 1)) + 1))
        if i % 5 == 4:
            sizes.append((total // 2, total // 2))
        else:
            an = int(rng.integers(1, total))
            sizes.append((an, total - an))
    return sizes


def test_batch_persistent_class_kernel(gpu, monkeypatch):
    """PREC_GPU_BATCH_PERSISTENT=1: the 2^13 .. 2^16-point classes run as one
    persistent kernel each (work items from a ticket, bounded waits on
    per-product phase counters).  Every product equals the oracle, on the
    first run and on a graph replay with new operand values."""
    torch = pytest.importorskip("torch")
    monkeypatch.setenv("PREC_GPU_BATCH_PERSISTENT", "1")
    sizes = _mid_class_sizes(21, 160)
    db = DevBatch(torch, sizes, 900)
    sq = [i for i, (a, b) in enumerate(sizes) if a == b]
    items = db.items()
    for i in sq:  # a square: the same operand pointer twice
        items[i] = (items[i][0], sizes[i][0], items[i][0], sizes[i][0], items[i][4])
    batch = gpu.Batch(items)
    stream = torch.cuda.current_stream().cuda_stream
    c0 = gpu.launch_count()
    for rnd in range(2):
        if rnd:
            db.fill(7000)
        db.out.fill_(-1)
        batch.run(stream)
        gpu.stream_check(stream)
        for i, (an, bn) in enumerate(sizes):
            a, b = db.operands(i)
            if i in sq:
                b = a
            assert np.array_equal(db.result(i), O.mul_ntt(a, b)), (rnd, i, sizes[i])
    # one kernel per class per run: 4 lengths, products and squares apart
    # (8 classes), not 4 phase kernels each
    assert gpu.launch_count() - c0 == 2 * 8
    batch.close()


def test_batch_persistent_wait_runs_out(gpu, monkeypatch):
    """A dependency wait of the persistent class kernel that can never be
    satisfied (PREC_GPU_BATCH_NEVER_SIGNAL=1: the forward tiles leave their
    counters untouched) gives up after its poll limit: the run ends, the
    stream check reports PREC_GPU_E_TIMEOUT, and the context stays usable
    (a normal batch afterwards is exact)."""
    torch = pytest.importorskip("torch")
    from preclib_gb300.native import E_TIMEOUT, PrecGpuError
    sizes = _mid_class_sizes(22, 12)
    db = DevBatch(torch, sizes, 300)
    stream = torch.cuda.current_stream().cuda_stream
    monkeypatch.setenv("PREC_GPU_BATCH_PERSISTENT", "1")
    monkeypatch.setenv("PREC_GPU_BATCH_NEVER_SIGNAL", "1")
    monkeypatch.setenv("PREC_GPU_BATCH_SPIN_LIMIT", "4000")
    batch = gpu.Batch(db.items())
    batch.run(stream)
    with pytest.raises(PrecGpuError) as ei:
        gpu.stream_check(stream)
    assert ei.value.code == E_TIMEOUT
    batch.close()
    monkeypatch.delenv("PREC_GPU_BATCH_NEVER_SIGNAL")
    monkeypatch.delenv("PREC_GPU_BATCH_SPIN_LIMIT")
    batch = gpu.Batch(db.items())
    db.out.fill_(-1)
    batch.run(stream)
    gpu.stream_check(stream)
    for i in range(len(sizes)):
        a, b = db.operands(i)
        assert np.array_equal(db.result(i), O.mul_ntt(a, b)), (i, sizes[i])
    batch.close()
