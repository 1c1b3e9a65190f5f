// ntt_add.cu -- out[0 .. n) += t[0 .. nt) on the device: the accumulation
// step of a blocked product (operands above the block size are cut into
// blocks; every pair of blocks is one NTT product added into the result at
// its limb offset).
//
// Phase 1 (every block of 1024 limbs): per-limb sums with their generate
// and propagate bits, the chain resolved per warp and per block with a
// block carry-in of 0, limbs written, block aggregate published.
// Phase 2 (the last block to finish, fence + atomic counter): scans the
// aggregates, adds each nonzero block carry-in (+1 through all-ones limbs),
// then carries the final carry out of t's span into out[nt ..] until a limb
// does not wrap.  A carry past out[n - 1] sets kDevErrCarry: the blocked
// product fits its La+Lb limbs, so that never happens on valid input.
#include "ntt_engine.cuh"

namespace precgpu {

namespace {

constexpr int kAddThreads = 256;
constexpr int kAddLimbs = 4;
constexpr int kAddBlockLimbs = kAddThreads * kAddLimbs;

// scratch: [0] finished-block counter, [1 .. nblk] aggregates (bit0 G, bit1 P)
__global__ void __launch_bounds__(kAddThreads) k_add_into(uint64_t* __restrict__ out, uint64_t n,
                                                          const uint64_t* __restrict__ t, uint64_t nt,
                                                          uint32_t* __restrict__ scratch, int* err) {
    __shared__ BlockCarryShared sh;
    __shared__ uint32_t s_last;
    const uint32_t bid = blockIdx.x;
    const uint64_t m0 = (uint64_t)bid * kAddBlockLimbs + threadIdx.x * kAddLimbs;
    uint64_t v[kAddLimbs];
    uint32_t gbits = 0;
    bool c = false, P = true;
#pragma unroll
    for (int k = 0; k < kAddLimbs; ++k) {
        const uint64_t i = m0 + k;
        // past t's span: an all-ones stand-in that passes a carry through to
        // the block aggregate (and is never written)
        const uint64_t x = i < nt ? out[i] : ~0ull, y = i < nt ? __ldg(&t[i]) : 0;
        const uint64_t s = x + y;
        const bool g = s < x;
        v[k] = s;
        gbits |= (uint32_t)g << k;
        const bool all1 = s == ~0ull;
        c = g || (all1 && c);
        P = P && all1;
    }
    uint32_t* agg = scratch + 1;
    auto publish = [&](bool Gb, bool Pb) { agg[bid] = (Gb ? 1u : 0u) | (Pb ? 2u : 0u); };
    const bool cin = block_carry_in0(c, P, sh, publish);
    limbs_finish<kAddLimbs>((int64_t)m0, nt, v, gbits, cin, out);

    // ---- phase 2: the last block joins the blocks' carries
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(&scratch[0], 1u) == gridDim.x - 1 ? 1u : 0u;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const int nblk = (int)gridDim.x;
    const int per = (nblk + blockDim.x - 1) / blockDim.x;
    const int b0 = threadIdx.x * per;
    bool tG = false, tP = true;
    for (int b = b0; b < b0 + per && b < nblk; ++b) {
        const uint32_t a = __ldcg(&agg[b]);
        tG = (a & 1u) || (tG && (a & 2u));
        tP = tP && (a & 2u);
    }
    auto none = [](bool, bool) -> bool { return false; };
    bool cc = block_carry(tG, tP, sh, none);  // carry into this thread's first block
    for (int b = b0; b < b0 + per && b < nblk; ++b) {
        const uint32_t a = __ldcg(&agg[b]);
        if (cc) {
            const uint64_t end = min((uint64_t)(b + 1) * kAddBlockLimbs, nt);
            for (uint64_t m = (uint64_t)b * kAddBlockLimbs; m < end; ++m) {
                const uint64_t x = __ldcg(&out[m]) + 1;
                out[m] = x;
                if (x != 0) break;
            }
        }
        cc = (a & 1u) || (cc && (a & 2u));
    }
    // the thread holding the last block carries the final carry above t
    if (b0 < nblk && b0 + per >= nblk && cc) {
        uint64_t m = nt;
        for (; m < n; ++m) {
            const uint64_t x = __ldcg(&out[m]) + 1;
            out[m] = x;
            if (x != 0) break;
        }
        if (m == n) atomicOr(err, kDevErrCarry);
    }
}

}  // namespace

size_t add_into_scratch_words(uint64_t nt) { return (size_t)((nt + kAddBlockLimbs - 1) / kAddBlockLimbs) + 1; }

void launch_add_into(uint64_t* out, uint64_t n, const uint64_t* t, uint64_t nt, uint32_t* scratch, int* err,
                     cudaStream_t st) {
    if (nt == 0) return;
    const unsigned nblk = (unsigned)((nt + kAddBlockLimbs - 1) / kAddBlockLimbs);
    cudaMemsetAsync(scratch, 0, sizeof(uint32_t), st);
    k_add_into<<<nblk, kAddThreads, 0, st>>>(out, n, t, nt, scratch, err);
    count_launches(1);
}

}  // namespace precgpu
