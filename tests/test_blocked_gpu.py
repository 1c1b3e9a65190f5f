"""GPU parity of blocked products: operands above the block size are cut into
blocks, every pair of blocks is one NTT-band product, and the partial
products are added into the result on the device (the range where the
reference's mul_ntt hands a product to mul_fft, src/mul_ntt.cpp:494-518).
A small block size puts the blocked path under the oracle; the default
2^24-limb block is checked by residues and closed forms."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

B1 = np.uint64(0xFFFFFFFFFFFFFFFF)


class _Block:
    def __init__(self, gpu, limbs):
        self.gpu, self.limbs = gpu, limbs

    def __enter__(self):
        self.prev = self.gpu.set_block_limbs(self.limbs)
        return self

    def __exit__(self, *exc):
        self.gpu.set_block_limbs(self.prev)


@pytest.mark.parametrize("an,bn", [(5000, 3000), (4097, 4096), (2049, 10), (10000, 10000), (6000, 2048),
                                   (2048, 2049), (9000, 1)])
def test_small_blocks_vs_oracle(gpu, an, bn):
    a = O.splitmix64(an * 13 + bn, an)
    b = O.splitmix64(an * 17 + bn + 1, bn)
    a[-1] |= np.uint64(1 << 63)
    b[-1] |= np.uint64(1 << 63)
    with _Block(gpu, 2048):
        got = gpu.mul(a, b, ntt=True)
        assert gpu.last_stats().path == 3
        assert gpu.ntt_log2(an, bn) == 0
    assert np.array_equal(got, O.mul_ntt(a, b))


def test_small_blocks_square_and_all_ones(gpu):
    """A blocked square, and (B^n - 1)(B^m - 1) whose partial products carry
    through every limb of the accumulation."""
    a = O.splitmix64(5, 7000)
    with _Block(gpu, 1024):
        assert np.array_equal(gpu.sqr(a), O.mul_ntt(a, a))
        for (n, m) in ((10000, 7000), (4096, 4096), (3000, 1025)):
            got = gpu.mul(np.full(n, B1), np.full(m, B1), ntt=True)
            want = np.zeros(n + m, np.uint64)
            want[0] = 1
            want[m:n] = B1
            want[n] = np.uint64(0xFFFFFFFFFFFFFFFE)
            want[n + 1:] = B1
            if n == m:
                want[n:] = B1
                want[n] = np.uint64(0xFFFFFFFFFFFFFFFE)
            assert np.array_equal(got, want), (n, m)


def test_small_blocks_device_api(gpu):
    torch = pytest.importorskip("torch")
    an, bn = 7777, 5555
    a = O.splitmix64(21, an)
    b = O.splitmix64(22, bn)
    ta = torch.from_numpy(a.view(np.int64)).cuda()
    tb = torch.from_numpy(b.view(np.int64)).cuda()
    to = torch.empty(an + bn, dtype=torch.int64, device="cuda")
    with _Block(gpu, 2000):
        gpu.mul_device(ta.data_ptr(), an, tb.data_ptr(), bn, to.data_ptr())
        gpu.stream_check()
    assert np.array_equal(to.cpu().numpy().view(np.uint64), O.mul_ntt(a, b))


def _spot(p, a, b, seed=31):
    O.spot_check(p, a, b, seed, fixed=(2305843009213693951, 4611686018427387847, 1152921504606846883))


def test_default_blocks_above_2_24_limbs(gpu):
    """Operands above 2^24 limbs (the reference's mul_fft range): residues
    modulo fixed and random 61/62-bit primes, and the all-ones closed form."""
    n = (1 << 24) + 3
    a = O.splitmix64(31, n)
    b = O.splitmix64(32, (1 << 20) + 9)
    p = gpu.mul(a, b, ntt=True)
    assert gpu.last_stats().path == 3
    _spot(p, a, b)
    assert p[-1] != 0
    p = gpu.sqr(a)
    _spot(p, a, a)
    got = gpu.mul(np.full(n, B1), np.full(n - 1, B1), ntt=True)
    m = n - 1
    assert got[0] == 1 and not got[1:m].any() and got[m:n].tolist() == [0xFFFFFFFFFFFFFFFF]
    assert got[n] == np.uint64(0xFFFFFFFFFFFFFFFE) and (got[n + 1:] == B1).all()
