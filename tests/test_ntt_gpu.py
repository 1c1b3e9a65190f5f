"""GPU parity of the NTT band through the C ABI: bit-exact against the
oracle and against the reference-generated golden vectors."""
import hashlib

import numpy as np
import pytest

import oracle as O
import patterns

pytestmark = pytest.mark.gpu


def _digest(out):
    return hashlib.sha256(np.ascontiguousarray(out, dtype="<u8").tobytes()).hexdigest()


def test_golden_vectors_ntt(gpu, golden):
    """Every golden product (NTT, FFT and dispatcher records alike: the
    product is an exact integer) through the NTT band."""
    for rec in golden:
        a, b = patterns.make(rec["gen"])
        if rec["ref_fn"] == "sqr":
            b = a  # the same vector: the square route
        out = gpu.mul(a, b, ntt=True)
        assert _digest(out) == rec["sha256"], rec["name"]


def test_kat_square(gpu):
    x = np.array([0xFFFFFFFF], dtype=np.uint64)
    out = gpu.mul(x, x, ntt=True)
    assert out.tolist() == [0xFFFFFFFE00000001, 0]


@pytest.mark.parametrize("an,bn", [(1, 1), (2, 1), (7, 5), (64, 64), (192, 193), (1000, 999),
                                   (2047, 2049), (2048, 2048), (2049, 2049), (4096, 4095),
                                   (4097, 4097), (6144, 8192), (8192, 8192), (10000, 5001),
                                   (16384, 16384), (40000, 39999), (65536, 65536), (100001, 50001)])
@pytest.mark.parametrize("wide", [False, True])
def test_random_vs_oracle(gpu, an, bn, wide):
    a = O.splitmix64(an * 31 + bn, an)
    b = O.splitmix64(an * 37 + bn + 1, bn)
    prev = gpu.set_wide_digits(wide)
    try:
        got = gpu.mul(a, b, ntt=True)
    finally:
        gpu.set_wide_digits(prev)
    assert np.array_equal(got, O.mul_ntt(a, b))


@pytest.mark.parametrize("wide", [False, True])
def test_both_paths_each_length(gpu, wide):
    """Every transform length 2^5 .. 2^19 (single-CTA and four-step), with
    32-bit digits and with 64-bit digits where the plan takes them."""
    prev = gpu.set_wide_digits(wide)
    try:
        for k in range(5, 20):
            n = 1 << (k - 2)  # 2n digits per operand -> N = 2^k
            a = O.splitmix64(k, n)
            b = O.splitmix64(k + 100, n)
            a[-1] |= np.uint64(1 << 63)
            b[-1] |= np.uint64(1 << 63)
            got = gpu.mul(a, b, ntt=True)
            assert np.array_equal(got, O.mul_ntt(a, b)), k
    finally:
        gpu.set_wide_digits(prev)


@pytest.mark.parametrize("wide,k", [(False, 20), (False, 21), (False, 23), (True, 19), (True, 20), (True, 22)])
def test_large_lengths_vs_oracle(gpu, wide, k):
    """The transform lengths above 2^19 that no golden digest covers, against the
    oracle: the default configurations of sets 0 and 2, whose column kernels
    run compiled for their row length."""
    n = 1 << (k - 1 if wide else k - 2)  # balanced operands filling a 2^k-point transform
    a = O.splitmix64(k * 7 + 1, n)
    b = O.splitmix64(k * 7 + 2, n)
    a[-1] |= np.uint64(1 << 63)
    b[-1] |= np.uint64(1 << 63)
    prev = gpu.set_wide_digits(wide)
    try:
        got = gpu.mul(a, b, ntt=True)
        st = gpu.last_stats()
    finally:
        gpu.set_wide_digits(prev)
    assert st.log2_n == k and st.path == 1 and st.digit_bits == (64 if wide else 32)
    assert np.array_equal(got, O.mul_ntt(a, b))


def test_zero_and_padding(gpu):
    z = np.zeros(5, np.uint64)
    a = O.splitmix64(3, 9000)
    assert not gpu.mul(z, a, ntt=True).any()
    assert len(gpu.mul(z, a, ntt=True)) == 9005
    # high zero limbs are trimmed by the host API and the tail zero-filled
    ap = np.concatenate([a, np.zeros(100, np.uint64)])
    b = O.splitmix64(4, 7000)
    got = gpu.mul(ap, b, ntt=True)
    assert len(got) == 9100 + 7000
    assert np.array_equal(got[:16000], O.mul_ntt(a, b)) and not got[16000:].any()


def test_all_ones_maximal_carries(gpu):
    """(2^(64n)-1)^2 has the longest carry runs the CRT output can produce."""
    for n in (1, 33, 2049, 6145, 70000, 1 << 20):
        a = np.full(n, 0xFFFFFFFFFFFFFFFF, dtype=np.uint64)
        got = gpu.mul(a, a, ntt=True)
        want = np.zeros(2 * n, np.uint64)
        want[0] = 1
        want[n:] = np.uint64(0xFFFFFFFFFFFFFFFF)
        want[n] = np.uint64(0xFFFFFFFFFFFFFFFE)
        assert np.array_equal(got, want), n


@pytest.mark.parametrize("n,k", [(3000, 1500), (5000, 1024), (9000, 4096), (70000, 30001), (1 << 20, 1 << 19)])
def test_all_ones_runs_across_carry_blocks(gpu, n, k):
    """(2^(64n)-1) * (2^(64k)+1) and (2^(64n)-1) * 2^(64k): results with
    all-ones runs spanning many 1024-limb carry blocks."""
    a = np.full(n, 0xFFFFFFFFFFFFFFFF, dtype=np.uint64)
    b = np.zeros(k + 1, np.uint64)
    b[0] = 1
    b[k] = 1
    want = O.to_int(a) * O.to_int(b)
    assert O.to_int(gpu.mul(a, b, ntt=True)) == want
    b[0] = 0
    assert O.to_int(gpu.mul(a, b, ntt=True)) == O.to_int(a) << (64 * k)


def test_torture_ntt(gpu):
    for (an, bn) in patterns.TORTURE_SHAPES:
        for p in patterns.TORTURE_PATTERNS:
            a, b = patterns.torture(p[0], an, bn)
            if len(a) == 0 or len(b) == 0:
                continue
            assert np.array_equal(gpu.mul(a, b, ntt=True), O.mul_ntt(a, b)), (p[0], an, bn)


def _spot(p, a, b, seed):
    O.spot_check(p, a, b, seed, fixed=(2305843009213693951, 4611686018427387847, 1152921504606846883,
                                       2147483647 * 1048573))


def test_large_mod_prime_spot_checks(gpu):
    """Full-size products (2^22 .. 2^26-point transforms): residues modulo
    fixed and random 61-bit primes agree, plus the top-limb and length invariants."""
    for (an, bn, s) in ((1 << 20, 1 << 20, 3), (3 << 20, 1 << 21, 5), (1 << 22, 1 << 22, 7),
                        ((1 << 24) - 5, (1 << 24) - 7, 9)):
        a = O.splitmix64(s, an)
        b = O.splitmix64(s + 1, bn)
        p = gpu.mul(a, b, ntt=True)
        _spot(p, a, b, s)
        assert p[-1] != 0 or p[-2] != 0


def test_1m_golden(gpu, golden):
    """The 1M x 1M product on both digit widths: 2^21 points over five primes
    (64-bit digits, the default) and 2^22 points over three (32-bit)."""
    rec = [r for r in golden if r["name"] == "cfg2_1Mx1M_ntt"][0]
    a, b = patterns.make(rec["gen"])
    for wide, k in ((True, 21), (False, 22)):
        prev = gpu.set_wide_digits(wide)
        try:
            assert _digest(gpu.mul(a, b, ntt=True)) == rec["sha256"], wide
            st = gpu.last_stats()
            assert st.log2_n == k and st.path == 1
        finally:
            gpu.set_wide_digits(prev)


def test_4m_golden(gpu, golden):
    """The 4M x 4M product against the reference's own digest on both digit
    widths: 2^23 points over the second five-prime set (64-bit digits, the
    default) and 2^24 points over the reference's three primes (32-bit)."""
    rec = [r for r in golden if r["name"] == "big_4Mx4M_ntt"][0]
    a, b = patterns.make(rec["gen"])
    for wide, k in ((True, 23), (False, 24)):
        prev = gpu.set_wide_digits(wide)
        try:
            assert _digest(gpu.mul(a, b, ntt=True)) == rec["sha256"], wide
            st = gpu.last_stats()
            assert st.log2_n == k and st.path == 1
        finally:
            gpu.set_wide_digits(prev)


def test_device_api_matches_host_api(gpu):
    torch = pytest.importorskip("torch")
    for (an, bn) in ((5000, 4000), (1 << 18, 1 << 18), (50, 60)):
        a = O.splitmix64(an, an)
        b = O.splitmix64(bn + 1, bn)
        ta = torch.from_numpy(a.view(np.int64)).cuda()
        tb = torch.from_numpy(b.view(np.int64)).cuda()
        to = torch.empty(an + bn, dtype=torch.int64, device="cuda")
        s = torch.cuda.current_stream().cuda_stream
        gpu.mul_device(ta.data_ptr(), an, tb.data_ptr(), bn, to.data_ptr(), s)
        gpu.stream_check(s)
        got = to.cpu().numpy().view(np.uint64)
        assert np.array_equal(got, O.mul_ntt(a, b))


def test_device_api_odd_limb_offsets(gpu):
    """Operands that start 8 bytes past a 16-byte boundary (any limb offset
    of a device array is a valid operand)."""
    torch = pytest.importorskip("torch")
    for (an, bn) in ((40000, 30001), (2049, 2039), (300, 7)):
        a = O.splitmix64(an + 5, an)
        b = O.splitmix64(bn + 6, bn)
        buf = torch.empty(an + bn + 3, dtype=torch.int64, device="cuda")
        buf[1:1 + an] = torch.from_numpy(a.view(np.int64)).cuda()
        buf[2 + an:2 + an + bn] = torch.from_numpy(b.view(np.int64)).cuda()
        to = torch.empty(an + bn + 1, dtype=torch.int64, device="cuda")
        pa, pb, po = buf.data_ptr() + 8, buf.data_ptr() + 8 * (2 + an), to.data_ptr() + 8
        gpu.mul_device(pa, an, pb, bn, po)
        gpu.stream_check()
        got = to[1:].cpu().numpy().view(np.uint64)
        assert np.array_equal(got, O.mul_ntt(a, b)), (an, bn)


def test_host_api_pinned_result_buffer(gpu):
    """Page-locked operand and result buffers: the limbs, nothing written
    past an + bn, and a result written over its own operand."""
    torch = pytest.importorskip("torch")
    import ctypes
    L = gpu.lib()
    for (an, bn) in ((1 << 20, 1 << 20), (40000, 30001), (2000, 100), (300, 7)):
        a = O.splitmix64(an + 17, an)
        b = O.splitmix64(bn + 18, bn)
        want = O.mul_ntt(a, b)
        ho = torch.full((an + bn + 1,), -1, dtype=torch.int64).pin_memory()
        po = ho.numpy().view(np.uint64)
        gpu.check(L.prec_gpu_mul_ntt(gpu._p(a), an, gpu._p(b), bn, gpu._p(po)))
        assert np.array_equal(po[:an + bn], want), (an, bn)
        assert po[an + bn] == np.uint64(0xFFFFFFFFFFFFFFFF)  # nothing past an + bn
    # result written over operand a (both in page-locked memory)
    an = bn = 50000
    a = O.splitmix64(5, an)
    b = O.splitmix64(6, bn)
    want = O.mul_ntt(a, b)
    buf = torch.zeros(an + bn, dtype=torch.int64).pin_memory()
    pb = buf.numpy().view(np.uint64)
    pb[:an] = a
    gpu.check(L.prec_gpu_mul(gpu._p(pb), an, gpu._p(b), bn, gpu._p(pb)))
    assert np.array_equal(pb, want)


def test_launch_count(gpu):
    """prec_gpu_launch_count: three kernels per prime on side streams, then
    the CRT -- 16 for a 1M-limb product on 64-bit digits (five primes), 10
    on 32-bit digits (three) -- 1 for a single-CTA product, and a batch
    graph's kernels at every replay."""
    torch = pytest.importorskip("torch")
    n = 1 << 20
    ta = torch.from_numpy(O.splitmix64(1, n).view(np.int64)).cuda()
    to = torch.empty(2 * n, dtype=torch.int64, device="cuda")
    for wide, launches in ((True, 16), (False, 10)):
        prev = gpu.set_wide_digits(wide)
        try:
            c0 = gpu.launch_count()
            gpu.mul_device(ta.data_ptr(), n, ta.data_ptr() + 8 * 7, n - 7, to.data_ptr())
            gpu.stream_check()
            assert gpu.launch_count() - c0 == launches, wide
        finally:
            gpu.set_wide_digits(prev)
    c0 = gpu.launch_count()
    gpu.mul_device(ta.data_ptr(), 100, ta.data_ptr() + 800, 90, to.data_ptr())
    gpu.stream_check()
    assert gpu.launch_count() - c0 == 1
    items = [(ta.data_ptr(), 100, ta.data_ptr() + 800, 90, to.data_ptr()),
             (ta.data_ptr(), 9000, ta.data_ptr() + 8 * 9000, 9000, to.data_ptr() + 8 * 200)]
    b = gpu.Batch(items)
    c0 = gpu.launch_count()
    b.run()
    b.run()
    gpu.stream_check()
    b.close()
    assert gpu.launch_count() - c0 == 2 * (1 + 4)  # one single-CTA class, one four-step class


def test_invalid_arguments(gpu):
    """Null pointers with nonzero sizes and zero-size device operands are
    refused with PREC_GPU_E_ARG; nothing is launched."""
    import ctypes
    L = gpu.lib()
    a = O.splitmix64(1, 8)
    out = np.zeros(16, np.uint64)
    null = ctypes.POINTER(ctypes.c_uint64)()
    c0 = gpu.launch_count()
    assert L.prec_gpu_mul(null, 8, gpu._p(a), 8, gpu._p(out)) == gpu.E_ARG
    assert L.prec_gpu_mul(gpu._p(a), 8, gpu._p(a), 8, null) == gpu.E_ARG
    assert L.prec_gpu_sqr(null, 3, gpu._p(out)) == gpu.E_ARG
    # real device buffers beside the invalid argument: were a refusal ever
    # to move, no kernel is handed an address that is not device memory
    torch = pytest.importorskip("torch")
    da = torch.zeros(5, dtype=torch.int64, device="cuda")
    db = torch.zeros(5, dtype=torch.int64, device="cuda")
    dout = torch.zeros(10, dtype=torch.int64, device="cuda")
    assert L.prec_gpu_mul_device(None, 5, db.data_ptr(), 5, dout.data_ptr(), None) == gpu.E_ARG
    assert L.prec_gpu_mul_device(da.data_ptr(), 0, db.data_ptr(), 5, dout.data_ptr(), None) == gpu.E_ARG
    assert gpu.launch_count() == c0
    # zero-length operands are a valid zero product
    assert L.prec_gpu_mul(null, 0, gpu._p(a), 8, gpu._p(out)) == gpu.OK
    assert not out[:8].any()


def test_device_calls_from_threads_on_own_streams(gpu):
    """Device-pointer products from four threads, each on its own stream
    (each thread has its own library workspace, so the products may run at
    the same time), across both digit widths and a square: all exact."""
    import threading
    torch = pytest.importorskip("torch")
    shapes = [(300000, 200000), (8192, 8192), (70000, 70000), (1 << 19, 1 << 19)]
    cases = []
    for i, (an, bn) in enumerate(shapes):
        a = O.splitmix64(60 + i, an)
        b = a if i == 2 else O.splitmix64(70 + i, bn)
        cases.append((a, b, O.mul_ntt(a, b)))
    errors = []

    def work(t):
        try:
            a, b, want = cases[t]
            s = torch.cuda.Stream()
            with torch.cuda.stream(s):
                ta = torch.from_numpy(a.view(np.int64)).cuda()
                tb = ta if b is a else torch.from_numpy(b.view(np.int64)).cuda()
                out = torch.empty(len(a) + len(b), dtype=torch.int64, device="cuda")
                for _ in range(3):
                    gpu.check(gpu.lib().prec_gpu_mul_device(ta.data_ptr(), len(a), tb.data_ptr(), len(b),
                                                            out.data_ptr(), s.cuda_stream))
                gpu.stream_check(s.cuda_stream)
                if not np.array_equal(out.cpu().numpy().view(np.uint64), want):
                    errors.append(t)
        except Exception as e:  # pragma: no cover - reported below
            errors.append(repr(e))

    th = [threading.Thread(target=work, args=(t,)) for t in range(len(cases))]
    for x in th:
        x.start()
    for x in th:
        x.join()
    assert not errors, errors


def test_host_calls_from_many_threads(gpu):
    """Host-pointer calls from eight threads at once (each thread with its own
    stream and workspace, running concurrently), across both bands and
    squares, are all exact."""
    import threading
    shapes = [(20000, 15000), (3000, 2999), (200, 300), (65536, 65536), (9000, 9000), (1, 7), (6144, 6144),
              (100000, 1000)]
    cases = []
    for i, (an, bn) in enumerate(shapes):
        a = O.splitmix64(40 + i, an)
        b = a if an == bn and i % 2 else O.splitmix64(50 + i, bn)
        cases.append((a, b, O.mul_ntt(a, b)))
    errors = []

    def work(t):
        try:
            for r in range(3):
                a, b, want = cases[(t + r) % len(cases)]
                if not np.array_equal(gpu.mul(a, b), want):
                    errors.append((t, r))
        except Exception as e:  # pragma: no cover - reported below
            errors.append(repr(e))

    th = [threading.Thread(target=work, args=(t,)) for t in range(8)]
    for x in th:
        x.start()
    for x in th:
        x.join()
    assert not errors, errors
