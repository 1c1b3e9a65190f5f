// ntt_carry.cuh -- CRT recombination and carry propagation of the four-step
// path (crt_carry_tile): the reference's ntt_crt2/ntt_crt3 and serial
// ntt_from_residues carry loop (src/mul_ntt.cpp:405-487) as one pass over
// the natural-order residues.  Shared by the carry kernel (ntt_carry.cu)
// and the batch form's persistent class kernel (ntt_class.cu).
//
// Phase 1 (every block): each thread turns 8 coefficients into 4 limbs
// (set 2: 4 coefficients of up to 150 bits, one per limb, into 4 limbs),
// the limb carry chain is resolved per warp (ballot) and per block with a
// block carry-in of 0 (one barrier), the limbs are written, and the block publishes its
// aggregate (G = carry out, P = a carry-in would pass through).
// Phase 2 (the last block to finish, found with a fence and an atomic
// counter): scans the aggregates into per-block carry-ins and adds the
// carry into the blocks that receive one -- on random data about one block
// in 64, usually a single limb.  No block ever waits on another.
#pragma once
#include "ntt_engine.cuh"

namespace precgpu {

// residue loads: COH reads through L2 only (data written earlier in the
// same launch); otherwise as before (read-only path for the vector loads)
template <bool COH>
__device__ __forceinline__ uint4 ld_work4(const uint32_t* p) {
    if constexpr (COH) return __ldcg(reinterpret_cast<const uint4*>(p));
    else return __ldg(reinterpret_cast<const uint4*>(p));
}
template <bool COH>
__device__ __forceinline__ uint32_t ld_work(const uint32_t* p) {
    if constexpr (COH) return __ldcg(p);
    else return *p;
}

// ---- set 2: one coefficient per 64-bit limb

// a coefficient c < p1..p5 < 2^150 as three words (w2 < 2^22)
struct Coef3 {
    uint64_t w0, w1;
    uint32_t w2;
};

// Garner over the five primes (the constants of Crt5Const) from the
// inverse-transform outputs y_j = (value) * a_j, a_j applied by the inverse
// column pass; then c = v0 + p0 (v1 + p1 (v2 + p2 (v3 + p3 v4))).  LAZY
// (set 2, p < 2^30): y_j in [0, 4p), running values in [0, 2p); otherwise
// (set 3, p < 2^31) y_j and the running values in [0, p).
template <bool LAZY>
__device__ __forceinline__ Coef3 crt5(const uint32_t (&y)[5], const Crt5Const& cc, const FieldArgs& f) {
    uint32_t v[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        const uint32_t p = f.pc[j].p, p2 = f.pc[j].p2;
        if constexpr (LAZY) {
            uint32_t acc = min(y[j], y[j] - p2);  // [0, 2p)
#pragma unroll
            for (int i = 0; i < j; ++i) {
                const ShoupC b = cc.b[j * (j - 1) / 2 + i];
                const uint32_t t = acc + p2 - shoup_lazy(v[i], b.w, b.wp, p);  // (0, 4p)
                acc = min(t, t - p2);
            }
            v[j] = red1(acc, p);
        } else {
            uint32_t acc = y[j];  // [0, p)
#pragma unroll
            for (int i = 0; i < j; ++i) acc = sub_mod(acc, shoup_mul(v[i], cc.b[j * (j - 1) / 2 + i], p), p);
            v[j] = acc;
        }
    }
    u128 X = (u128)((uint64_t)v[4] * f.pc[3].p + v[3]);
    X = X * f.pc[2].p + v[2];
    X = X * f.pc[1].p + v[1];  // < 2^120
    const u128 t0 = (u128)(uint64_t)X * f.pc[0].p + v[0];
    const u128 t1 = (u128)(uint64_t)(X >> 64) * f.pc[0].p + (uint64_t)(t0 >> 64);
    Coef3 c;
    c.w0 = (uint64_t)t0;
    c.w1 = (uint64_t)t1;
    c.w2 = (uint32_t)(t1 >> 64);
    return c;
}

template <bool LAZY>
__device__ __forceinline__ Coef3 coef5(const uint32_t* __restrict__ work, uint64_t N, int64_t i,
                                       const ProdArgs& args) {
    if (i < 0 || (uint64_t)i >= N) return Coef3{0, 0, 0};
    uint32_t y[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) y[j] = work[(uint64_t)(2 * j) * N + i];
    return crt5<LAZY>(y, args.crt5, args.f);
}

// sum of limb m: S_m = w0(c_m) + w1(c_(m-1)) + w2(c_(m-2)) < 2^66
__device__ __forceinline__ u128 limb_sum(const Coef3& c0, uint64_t w1_prev, uint32_t w2_prev2) {
    return (u128)c0.w0 + w1_prev + w2_prev2;
}

struct WideEdge {
    uint64_t w1;  // w1 of the warp's last coefficient
    uint32_t w2a, w2b;  // w2 of its last two coefficients
    uint32_t hi;  // S >> 64 of its last limb
};

// T[k] = S_(m0+k) for this thread's limbs and hi(S_(m0-1)); the words the
// first limbs need from below come from the lane below or, for a warp's
// lane 0, from the warp below (shared memory).  The block's thread 0 holds
// the four coefficients just below the block's first limb and outputs
// nothing, so every thread recombines exactly four coefficients (three lanes
// of warp 0 recomputing the block's edge after their own four kept the
// other warps waiting at the barrier: 3.9 stalled warps per issue).
template <bool LAZY>
__device__ __forceinline__ void wide_sums(const ProdPtrs& PP, const ProdArgs& args, int64_t m0, u128 (&T)[kCarryLimbs],
                                          uint64_t& prev_hi, WideEdge* s_edge) {
    static_assert(kCarryLimbs >= 4 && kCarryLimbs % 4 == 0, "limbs per thread: whole 16-byte loads");
    constexpr int L = kCarryLimbs;
    const uint64_t N = 1ull << args.k;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    Coef3 c[L];
    if (m0 >= 0 && (uint64_t)m0 + L <= N) {  // (block 0's thread 0 starts at -4)
#pragma unroll
        for (int h = 0; h < L / 4; ++h) {
            uint4 r[5];
#pragma unroll
            for (int j = 0; j < 5; ++j)
                r[j] = __ldg(reinterpret_cast<const uint4*>(PP.work + (uint64_t)(2 * j) * N + m0) + h);
            uint32_t y[5];
#pragma unroll
            for (int j = 0; j < 5; ++j) y[j] = r[j].x;
            c[4 * h] = crt5<LAZY>(y, args.crt5, args.f);
#pragma unroll
            for (int j = 0; j < 5; ++j) y[j] = r[j].y;
            c[4 * h + 1] = crt5<LAZY>(y, args.crt5, args.f);
#pragma unroll
            for (int j = 0; j < 5; ++j) y[j] = r[j].z;
            c[4 * h + 2] = crt5<LAZY>(y, args.crt5, args.f);
#pragma unroll
            for (int j = 0; j < 5; ++j) y[j] = r[j].w;
            c[4 * h + 3] = crt5<LAZY>(y, args.crt5, args.f);
        }
    } else {
#pragma unroll
        for (int k = 0; k < L; ++k) c[k] = coef5<LAZY>(PP.work, N, m0 + k, args);
    }
    const u128 s_last = limb_sum(c[L - 1], c[L - 2].w1, c[L - 3].w2);
    const uint32_t hi_last = (uint32_t)(s_last >> 64);
    // words from the thread below: w1(c_-1), w2(c_-1), w2(c_-2), hi(S_-1)
    uint64_t w1m1 = __shfl_up_sync(0xffffffffu, c[L - 1].w1, 1);
    uint32_t w2m1 = __shfl_up_sync(0xffffffffu, c[L - 1].w2, 1);
    uint32_t w2m2 = __shfl_up_sync(0xffffffffu, c[L - 2].w2, 1);
    uint32_t him1 = __shfl_up_sync(0xffffffffu, hi_last, 1);
    if (lane == 31) s_edge[warp] = WideEdge{c[L - 1].w1, c[L - 1].w2, c[L - 2].w2, hi_last};
    __syncthreads();
    if (lane == 0 && warp > 0) {
        const WideEdge e = s_edge[warp - 1];
        w1m1 = e.w1;
        w2m1 = e.w2a;
        w2m2 = e.w2b;
        him1 = e.hi;
    }
    T[0] = limb_sum(c[0], w1m1, w2m2);
    T[1] = limb_sum(c[1], c[0].w1, w2m1);
#pragma unroll
    for (int k = 2; k < L; ++k) T[k] = limb_sum(c[k], c[k - 1].w1, c[k - 2].w2);
    prev_hi = him1;
}

// One carry block (x, from args.crt_blk0 in a chunked CRT) of product z;
// nx: blocks of this launch (the chunk's, or every block of the product).
// scratch layout: [0] finished-block counter, [1 .. nblk] aggregates
// (bit0 G, bit1 P).  COH: the residues were written earlier in the same
// launch (the batch form's persistent class kernel) and are read through L2
// (ld.global.cg), never a non-coherent cache.
template <int SET, bool COH = false, class I>
__device__ __forceinline__ void crt_carry_tile(const ProdArgs& args, const ProdPtrs* __restrict__ batch, const I& ix) {
    __shared__ BlockCarryShared sh;
    __shared__ uint32_t s_last;
    __shared__ WideEdge s_edge[kCarryThreads / 32];
    const ProdPtrs PP = select_product_at(args, batch, ix.z());
    const uint32_t bid = args.crt_blk0 + ix.x();  // chunked CRT: blocks from crt_blk0
    if ((int)bid >= PP.nblk) return;  // batch: a shorter product of the class
    const uint64_t N = 1ull << args.k;
    const int lane = threadIdx.x & 31;
    constexpr int BL = crt_block_limbs(SET);  // limbs the block outputs
    // 64-bit digits: thread 0 takes the four coefficients below the block
    const int64_t m0 = (int64_t)bid * BL + ((int)threadIdx.x - (set_wide(SET) ? 1 : 0)) * kCarryLimbs;
    const bool edge_only = set_wide(SET) && threadIdx.x == 0;

    u128 T[kCarryLimbs];
    uint64_t prev_hi = 0;
    if constexpr (set_wide(SET)) {
        wide_sums<SET == kWideSet>(PP, args, m0, T, prev_hi, s_edge);
    } else {
        const uint32_t* __restrict__ r0 = PP.work;
        const uint32_t* __restrict__ r1 = PP.work + 2 * N;
        const uint32_t* __restrict__ r2 = PP.work + 4 * N;
        const uint64_t i0 = 2 * (uint64_t)m0;
        if (i0 + 2 * kCarryLimbs <= N) {
            uint32_t y[3][2 * kCarryLimbs];
#pragma unroll
            for (int h = 0; h < 2 * kCarryLimbs / 4; ++h) {
                const uint4 a = ld_work4<COH>(r0 + i0 + 4 * h);
                const uint4 b = ld_work4<COH>(r1 + i0 + 4 * h);
                const uint4 c = ld_work4<COH>(r2 + i0 + 4 * h);
                y[0][4 * h] = a.x; y[0][4 * h + 1] = a.y; y[0][4 * h + 2] = a.z; y[0][4 * h + 3] = a.w;
                y[1][4 * h] = b.x; y[1][4 * h + 1] = b.y; y[1][4 * h + 2] = b.z; y[1][4 * h + 3] = b.w;
                y[2][4 * h] = c.x; y[2][4 * h + 1] = c.y; y[2][4 * h + 2] = c.z; y[2][4 * h + 3] = c.w;
            }
#pragma unroll
            for (int k = 0; k < kCarryLimbs; ++k) {
                const u128 c0 = crt3_folded<SET>(y[0][2 * k], y[1][2 * k], y[2][2 * k], args.crt, args.f);
                const u128 c1 =
                    crt3_folded<SET>(y[0][2 * k + 1], y[1][2 * k + 1], y[2][2 * k + 1], args.crt, args.f);
                T[k] = c0 + (c1 << 32);
            }
        } else {
#pragma unroll
            for (int k = 0; k < kCarryLimbs; ++k) {
                u128 c[2];
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    const uint64_t i = i0 + 2 * k + e;
                    c[e] = i < N ? crt3_folded<SET>(ld_work<COH>(r0 + i), ld_work<COH>(r1 + i), ld_work<COH>(r2 + i),
                                                    args.crt, args.f)
                                 : (u128)0;
                }
                T[k] = c[0] + (c[1] << 32);
            }
        }
        // hi(T) of the limb just below this thread's first limb
        prev_hi = __shfl_up_sync(0xffffffffu, (uint64_t)(T[kCarryLimbs - 1] >> 64), 1);
        if (lane == 0) {
            prev_hi = 0;
            if (m0 > 0 && i0 - 1 < N) {
                const u128 c0 = crt3_folded<SET>(ld_work<COH>(r0 + i0 - 2), ld_work<COH>(r1 + i0 - 2),
                                                 ld_work<COH>(r2 + i0 - 2), args.crt, args.f);
                const u128 c1 = crt3_folded<SET>(ld_work<COH>(r0 + i0 - 1), ld_work<COH>(r1 + i0 - 1),
                                                 ld_work<COH>(r2 + i0 - 1), args.crt, args.f);
                prev_hi = (uint64_t)((c0 + (c1 << 32)) >> 64);
            }
        }
    }
    uint64_t v[kCarryLimbs];
    uint32_t gbits;
    bool G, P;
    limbs_from_sums<kCarryLimbs>(T, prev_hi, v, gbits, G, P);
    if (edge_only) G = false, P = true;  // no limbs: the identity of the carry scan

    uint32_t* agg = PP.scratch + 1;
    auto publish = [&](bool Gb, bool Pb) { agg[bid] = (Gb ? 1u : 0u) | (Pb ? 2u : 0u); };
    const bool cin = block_carry_in0(G, P, sh, publish);
    if (!edge_only) limbs_finish<kCarryLimbs>(m0, PP.lout, v, gbits, cin, PP.out);

    // ---- phase 2: the last block resolves the carries between blocks.
    // The barrier orders every thread's limb and aggregate stores before
    // thread 0's device-scope fence, which orders them before the counter.
    // A chunked CRT (one launch per run of blocks, in order on one stream)
    // joins each chunk on its own: the carry into the chunk comes from the
    // previous chunk's join, and its carry out goes to the next.
    const bool chunked = args.chunk_words != nullptr;
    uint32_t* counter = chunked ? &args.chunk_words[2 * args.crt_chunk] : &PP.scratch[0];
    const int blo = chunked ? args.crt_blk0 : 0;
    const int bhi = chunked ? args.crt_blk0 + (int)ix.nx() : PP.nblk;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(counter, 1u) == (uint32_t)(bhi - blo) - 1 ? 1u : 0u;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const bool cin_chunk = chunked && __ldcg(&args.chunk_words[2 * args.crt_chunk + 1]) != 0;
    const int nb = bhi - blo;
    const int per = (nb + blockDim.x - 1) / blockDim.x;  // aggregates per thread
    const int b0 = blo + threadIdx.x * per, b1 = min(b0 + per, bhi);
    const int n = b1 > b0 ? b1 - b0 : 0;  // this thread's run of blocks
    auto chunk_in = [&](bool, bool) -> bool { return cin_chunk; };
    // the carry enters block b: +1 ripples through its all-ones limbs
    auto ripple = [&](int b) {
        const uint64_t lim_end = min((uint64_t)(b + 1) * BL, PP.lout);
        for (uint64_t m = (uint64_t)b * BL; m < lim_end; ++m) {
            const uint64_t x = __ldcg(&PP.out[m]) + 1;
            PP.out[m] = x;
            if (x != 0) break;
        }
    };
    // The aggregates are loaded kAggBatch at a time in one unrolled group
    // (independent loads in flight together, not one L2 round trip each).
    constexpr int kAggBatch = 16;
    bool cout;  // the carry out of this thread's last block
    if (per <= 64) {
        // the run as bit masks (bit i: block b0 + i; G and P, with G = 0,
        // P = 1 past the run): the run's own aggregate and, once the carry
        // into it is known, the carry into each of its blocks come from one
        // carry-chain addition each (a product up to 2^24 limbs)
        uint64_t gm = 0, pm = 0;
        for (int base = 0; base < per; base += kAggBatch) {
            uint32_t h[kAggBatch];
#pragma unroll
            for (int i = 0; i < kAggBatch; ++i) h[i] = base + i < n ? __ldcg(&agg[b0 + base + i]) : 2u;
#pragma unroll
            for (int i = 0; i < kAggBatch; ++i) {
                gm |= (uint64_t)(h[i] & 1u) << (base + i);
                pm |= (uint64_t)((h[i] >> 1) & 1u) << (base + i);
            }
        }
        const u128 A = (u128)(gm | pm), B = (u128)gm;
        const uint64_t nmask = n >= 64 ? ~0ull : ((1ull << n) - 1);
        const bool tG = (uint64_t)(((A + B) ^ A ^ B) >> n) & 1;  // carry out of the run, carry-in 0
        const bool tP = (pm & nmask) == nmask;
        const bool c = block_carry(tG, tP, sh, chunk_in);  // carry into this thread's first block
        const u128 cc = (A + B + (c ? 1u : 0u)) ^ A ^ B;   // bit i: carry into block b0 + i
        for (uint64_t enter = (uint64_t)cc & nmask; enter; enter &= enter - 1) ripple(b0 + __ffsll((long long)enter) - 1);
        cout = (uint64_t)(cc >> n) & 1;
    } else {
        // longer runs: two passes over the aggregates
        bool tG = false, tP = true;
        for (int base = b0; base < b1; base += kAggBatch) {
            uint32_t h[kAggBatch];
#pragma unroll
            for (int i = 0; i < kAggBatch; ++i) h[i] = base + i < b1 ? __ldcg(&agg[base + i]) : 2u;
#pragma unroll
            for (int i = 0; i < kAggBatch; ++i) {
                tG = (h[i] & 1u) || (tG && (h[i] & 2u));
                tP = tP && (h[i] & 2u);
            }
        }
        bool c = block_carry(tG, tP, sh, chunk_in);  // carry into this thread's first block
        for (int b = b0; b < b1; ++b) {
            const uint32_t a = __ldcg(&agg[b]);
            if (c) ripple(b);
            c = (a & 1u) || (c && (a & 2u));
        }
        cout = c;
    }
    if (b0 < bhi && b1 == bhi) {  // the thread holding the last block
        if (chunked && !args.crt_last) args.chunk_words[2 * args.crt_chunk + 3] = cout ? 1u : 0u;
        else if (cout) atomicOr(args.err, kDevErrCarry);  // a product fits La+Lb limbs
    }
}

}  // namespace precgpu
