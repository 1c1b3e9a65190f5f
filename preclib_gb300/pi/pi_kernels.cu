// pi_kernels.cu -- batched signed additions of the binary-splitting tree.
//
// k_top_diff: for pairs of opposite signs, the highest limb where the two
//   magnitudes differ (atomicMax over the pair's chunks) decides which one is
//   larger.
// k_signed_add: every chunk of every pair in one grid.  Each chunk adds (same
//   signs) or subtracts the smaller magnitude from the larger, resolves its
//   carries or borrows with a chunk carry-in of 0 (per thread, then ballot and
//   block scan), writes its limbs and publishes (G, P).  The last block to
//   finish (fence + atomic counter) runs a segmented scan over the chunks
//   (a pair's first chunk starts with carry 0) and adds each nonzero chunk
//   carry-in into its chunk: +1 through all-ones limbs or -1 through zero
//   limbs, rarely more than one limb.  No block waits on another.
#include "../csrc/ntt_engine.cuh"
#include "pi_device.hpp"

namespace precpi {

using precgpu::BlockCarryShared;
using precgpu::block_carry;
using precgpu::block_carry_in0;

namespace {

struct Scratch {
    long long* top;
    uint8_t* agg;
    uint32_t* counter;
};

__host__ __device__ inline Scratch carve(void* base, size_t npairs, size_t nchunks) {
    char* p = static_cast<char*>(base);
    Scratch s;
    s.top = reinterpret_cast<long long*>(p);
    p += ((npairs * sizeof(long long)) + 255) & ~(size_t)255;
    s.counter = reinterpret_cast<uint32_t*>(p);
    p += 256;
    s.agg = reinterpret_cast<uint8_t*>(p);
    return s;
}

__device__ __forceinline__ uint64_t limb(const uint64_t* v, uint32_t n, uint32_t j) { return j < n ? v[j] : 0; }

__global__ void __launch_bounds__(kAddThreads) k_top_diff(const AddPair* __restrict__ pairs,
                                                          const uint32_t* __restrict__ chunk_pair, long long* top) {
    __shared__ long long s_best[kAddThreads / 32];
    const uint32_t c = blockIdx.x;
    const uint32_t pi = chunk_pair[c];
    const AddPair P = pairs[pi];
    if (*P.sx == *P.sy) return;  // same signs: an addition, nothing to compare
    const uint32_t n = P.nx > P.ny ? P.nx : P.ny;
    const uint32_t lo = (c - P.chunk0) * kAddChunkLimbs;
    const uint32_t hi = lo + kAddChunkLimbs < n ? lo + kAddChunkLimbs : n;
    long long best = -1;
    for (uint32_t j = lo + threadIdx.x; j < hi; j += blockDim.x)
        if (limb(P.x, P.nx, j) != limb(P.y, P.ny, j)) best = (long long)j;
    for (int o = 16; o > 0; o >>= 1) {
        const long long t = __shfl_xor_sync(0xffffffffu, best, o);
        best = t > best ? t : best;
    }
    if ((threadIdx.x & 31) == 0) s_best[threadIdx.x >> 5] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < kAddThreads / 32; ++w) best = s_best[w] > best ? s_best[w] : best;
        if (best >= 0) atomicMax(&top[pi], best);
    }
}

__global__ void __launch_bounds__(kAddThreads) k_signed_add(const AddPair* __restrict__ pairs,
                                                            const uint32_t* __restrict__ chunk_pair,
                                                            uint32_t nchunks, Scratch sc) {
    __shared__ BlockCarryShared sh;
    __shared__ uint32_t s_last;
    const uint32_t c = blockIdx.x;
    const uint32_t pi = chunk_pair[c];
    const AddPair P = pairs[pi];
    const int sx = *P.sx, sy = *P.sy;
    const bool add = sx == sy;
    const long long t = add ? -1 : sc.top[pi];
    // the larger magnitude first; equal magnitudes of opposite signs give 0
    const bool x_big = add || (t >= 0 && limb(P.x, P.nx, (uint32_t)t) > limb(P.y, P.ny, (uint32_t)t));
    const bool zero = !add && t < 0;
    const uint64_t* big = x_big ? P.x : P.y;
    const uint64_t* small = x_big ? P.y : P.x;
    const uint32_t nb = x_big ? P.nx : P.ny, ns = x_big ? P.ny : P.nx;
    const uint32_t j0 = (c - P.chunk0) * kAddChunkLimbs + threadIdx.x * kAddLimbsPerThread;
    uint64_t v[kAddLimbsPerThread];
    bool carry = false, allp = true;
#pragma unroll
    for (int k = 0; k < kAddLimbsPerThread; ++k) {
        const uint32_t j = j0 + k;
        const uint64_t a = zero ? 0 : limb(big, nb, j), b = zero ? 0 : limb(small, ns, j);
        if (add) {
            const uint64_t s = a + b;
            const uint64_t r = s + (carry ? 1u : 0u);
            carry = (s < a) || (r < s);
            v[k] = r;
            allp = allp && r == ~0ull;
        } else {
            const uint64_t d = a - b;
            const uint64_t r = d - (carry ? 1u : 0u);
            carry = (a < b) || (d < (carry ? 1u : 0u));
            v[k] = r;
            allp = allp && r == 0;
        }
    }
    auto publish = [&](bool Gb, bool Pb) { sc.agg[c] = (uint8_t)((Gb ? 1u : 0u) | (Pb ? 2u : 0u)); };
    const bool cin = block_carry_in0(carry, allp, sh, publish);
    bool cc = cin;
#pragma unroll
    for (int k = 0; k < kAddLimbsPerThread; ++k) {
        const uint64_t old = v[k];
        if (cc) {
            v[k] = add ? old + 1 : old - 1;
            cc = add ? old == ~0ull : old == 0;
        }
        if (j0 + k < P.nz) P.z[j0 + k] = v[k];
    }
    if (c == P.chunk0 && threadIdx.x == 0) *P.sz = (int8_t)(zero ? 0 : (x_big ? sx : sy));

    // ---- the last block joins the chunks of every pair
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(sc.counter, 1u) == nchunks - 1 ? 1u : 0u;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const uint32_t per = (nchunks + blockDim.x - 1) / blockDim.x;
    const uint32_t q0 = threadIdx.x * per, q1 = q0 + per < nchunks ? q0 + per : nchunks;
    // this thread's run of chunks as one carry element; a pair's first chunk
    // takes no carry from before it
    bool tG = false, tP = true;
    for (uint32_t q = q0; q < q1; ++q) {
        const uint32_t a = __ldcg(&sc.agg[q]);
        const bool start = q == __ldg(&pairs[chunk_pair[q]].chunk0);
        tG = (a & 1u) || ((a & 2u) && tG && !start);
        tP = tP && (a & 2u) && !start;
    }
    auto none = [](bool, bool) -> bool { return false; };
    bool run = block_carry(tG, tP, sh, none);
    for (uint32_t q = q0; q < q1; ++q) {
        const uint32_t a = __ldcg(&sc.agg[q]);
        const AddPair Q = pairs[chunk_pair[q]];
        const bool cq = q == Q.chunk0 ? false : run;
        if (cq) {
            const bool qadd = *Q.sx == *Q.sy;
            const uint32_t lo = (q - Q.chunk0) * kAddChunkLimbs;
            const uint32_t hi = lo + kAddChunkLimbs < Q.nz ? lo + kAddChunkLimbs : Q.nz;
            for (uint32_t j = lo; j < hi; ++j) {
                const uint64_t old = __ldcg(&Q.z[j]);
                Q.z[j] = qadd ? old + 1 : old - 1;
                if (qadd ? old != ~0ull : old != 0) break;
            }
        }
        run = (a & 1u) || ((a & 2u) && cq);
    }
}

}  // namespace

static uint64_t g_launches = 0;

uint64_t signed_add_launches() { return g_launches; }

size_t signed_add_scratch_bytes(size_t npairs, size_t nchunks) {
    return (((npairs * sizeof(long long)) + 255) & ~(size_t)255) + 256 + nchunks;
}

cudaError_t signed_add_many(const AddPair* pairs, size_t npairs, const uint32_t* chunk_pair, size_t nchunks,
                            void* scratch, cudaStream_t st) {
    if (!nchunks) return cudaSuccess;
    const Scratch sc = carve(scratch, npairs, nchunks);
    cudaMemsetAsync(sc.top, 0xFF, npairs * sizeof(long long), st);  // -1: no differing limb yet
    cudaMemsetAsync(sc.counter, 0, sizeof(uint32_t), st);
    k_top_diff<<<(unsigned)nchunks, kAddThreads, 0, st>>>(pairs, chunk_pair, sc.top);
    k_signed_add<<<(unsigned)nchunks, kAddThreads, 0, st>>>(pairs, chunk_pair, (uint32_t)nchunks, sc);
    g_launches += 2;
    return cudaGetLastError();
}

}  // namespace precpi
