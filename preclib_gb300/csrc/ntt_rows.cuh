// ntt_rows.cuh -- row pass of the four-step NTT (rows_tile), shared by the
// row kernel (ntt_rows.cu) and the batch form's persistent class kernel
// (ntt_class.cu).
//
// For `rows` row slots of one prime: the remaining DIF stages of both
// operands' rows (the last log2(N2) stages of ntt_forward,
// src/mul_ntt.cpp:193-255), the pointwise product (mul_ntt.cpp:364-373)
// and the first DIT stages of the product row (ntt_inverse,
// mul_ntt.cpp:257-311).  The bottom five stages of both directions and the
// product run in registers without a shared-memory round trip in between.
// The four-step twiddles are the column passes' (the inverse one measured
// 1-2% faster at 2^21 points in the inverse column pass, where it shares the
// loop over a thread's 32 slots with the forward one's pattern).
#pragma once
#include "ntt_engine.cuh"

namespace precgpu {

// MR: pass radix cap.  With MR = 6 a 2^11-point row runs as a radix-64 and
// a radix-32 pass (no middle pass); the radix-64 top pass then takes the two
// operands one after the other (64 values in registers, not 128).
// One tile of the row pass: row slots [x*rows, (x+1)*rows) of prime
// args.prime0 + y of product z.  COH: the work rows were written earlier in
// the same launch (the batch form's persistent class kernel), so they are
// read through L2 (ld.global.cg), never a non-coherent cache.
template <int SET, int M, bool SQ, int MR, bool COH = false, class I>
__device__ __forceinline__ void rows_tile(const ProdArgs& args, const ProdPtrs* __restrict__ batch, const I& ix,
                                          uint32_t* sm) {
    constexpr int NP = sch_np(M, MR);
    static_assert(NP >= 2, "row transforms have at least two passes");
    constexpr int AS = astride_for(M);
    const ProdPtrs P = select_product_at(args, batch, ix.z());
    const int prime = args.prime0 + ix.y();
    const PrimeC pc = args.f.pc[prime];
    const uint2* __restrict__ twf = args.f.tf[prime];
    const uint2* __restrict__ twi = args.f.ti[prime];
    const int rows = args.rows;
    uint32_t* __restrict__ A = P.work + ((uint64_t)(prime * 2) << args.k);
    const uint32_t* __restrict__ B = A + (1ull << args.k);
    const uint32_t row0 = ix.x() * rows;
    constexpr int NA = SQ ? 1 : 2;  // a square transforms its one operand only

    {   // top DIF pass of A (and B) straight from HBM (shared twiddles).
        // (Staging the rows into shared memory first by 4-byte asynchronous
        // copies -- the padding leaves no 16-byte alignment -- measured slower
        // on GB300: 78 against 70 us at 2^21 points.)
        using G = Geom<M, 0, MR>;
        constexpr bool SEQ = !SQ && G::R > 32;  // operands one after the other
        constexpr int NT = SEQ ? 1 : NA;        // operands per item
        constexpr int items = 1 << G::LGI;
        for (int w = threadIdx.x; w < (rows * items) * (SEQ ? 2 : 1); w += blockDim.x) {
            const int op = SEQ ? w / (rows * items) : 0;
            const int wi = SEQ ? w - op * (rows * items) : w;
            const int r = wi >> G::LGI;
            const uint32_t u = wi & (items - 1);
            const uint64_t roff = ((uint64_t)(row0 + r) << M) + G::base(u);
            const uint32_t* __restrict__ src = op ? B : A;
            uint32_t x[NT][G::R];
#pragma unroll
            for (int q = 0; q < G::R; ++q) {
                if constexpr (COH) {
                    x[0][q] = __ldcg(src + roff + ((uint32_t)q << G::LO));
                    if constexpr (NT == 2) x[1][q] = __ldcg(B + roff + ((uint32_t)q << G::LO));
                } else {
                    x[0][q] = src[roff + ((uint32_t)q << G::LO)];
                    if constexpr (NT == 2) x[1][q] = B[roff + ((uint32_t)q << G::LO)];
                }
            }
            regs_pass<SET, M, 0, false, NT, MR>(x, u, twf, pc);
            uint32_t* s = sm + 2 * r * AS + op * AS + G::pbase(u);
#pragma unroll
            for (int q = 0; q < G::R; ++q) {
                s[q * G::QS] = x[0][q];
                if constexpr (NT == 2) s[AS + q * G::QS] = x[1][q];
            }
        }
        __syncthreads();
    }
    if constexpr (SQ) row_passes<SET, M, 1, NP - 2, false, 1, MR>(sm, 2 * AS, rows, twf, pc);
    else row_passes<SET, M, 1, NP - 2, false, 2, MR>(sm, AS, 2 * rows, twf, pc);
    {   // bottom: last DIF stages, product, first DIT stages
        using G = Geom<M, NP - 1, MR>;
        static_assert(G::LO == 0 && G::RB == 5, "bottom pass covers bits 0..4");
        for (int w = threadIdx.x; w < (rows << G::LGI); w += blockDim.x) {
            const int r = w >> G::LGI;
            const uint32_t u = w & ((1u << G::LGI) - 1);
            uint32_t* s = sm + 2 * r * AS + 33 * u;
            uint32_t x[NA][32];
#pragma unroll
            for (int q = 0; q < 32; ++q) {
                x[0][q] = s[q];
                if constexpr (!SQ) x[NA - 1][q] = s[AS + q];
            }
            regs_pass<SET, M, NP - 1, false, NA, MR>(x, u, twf, pc);
            uint32_t y[1][32];
#pragma unroll
            for (int q = 0; q < 32; ++q) y[0][q] = Ar<SET>::mul(x[0][q], x[NA - 1][q], pc);
            regs_pass<SET, M, NP - 1, true, 1, MR>(y, u, twi, pc);
#pragma unroll
            for (int q = 0; q < 32; ++q) s[q] = y[0][q];
        }
        __syncthreads();
    }
    row_passes<SET, M, NP - 2, 1, true, 1, MR>(sm, 2 * AS, rows, twi, pc);
    {   // top DIT pass, straight to HBM
        using G = Geom<M, 0, MR>;
        for (int w = threadIdx.x; w < (rows << G::LGI); w += blockDim.x) {
            const int r = w >> G::LGI;
            const uint32_t u = w & ((1u << G::LGI) - 1);
            const uint32_t* s = sm + 2 * r * AS + G::pbase(u);
            uint32_t x[1][G::R];
#pragma unroll
            for (int q = 0; q < G::R; ++q) x[0][q] = s[q * G::QS];
            regs_pass<SET, M, 0, true, 1, MR>(x, u, twi, pc);
            // in the forward range: the inverse column pass multiplies by the
            // inverse four-step twiddle first
            uint32_t* __restrict__ dst = A + ((uint64_t)(row0 + r) << M) + G::base(u);
#pragma unroll
            for (int q = 0; q < G::R; ++q) dst[(uint32_t)q << G::LO] = Ar<SET>::half(x[0][q], pc);
        }
    }
}

}  // namespace precgpu
