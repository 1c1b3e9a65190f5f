// ntt_rows.cu -- row pass of the four-step NTT.
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
// pass radix cap of the row transforms (radix-8/16 passes: two operands'
// radix-64 items would not fit the register budget)
#ifndef PREC_ROWS_MAXRB
#define PREC_ROWS_MAXRB 4
#endif
#ifndef PREC_SCH_MAXRB
#define PREC_SCH_MAXRB PREC_ROWS_MAXRB
#endif
#include "ntt_engine.cuh"

// threads of a row-pass CTA (rows x 2^(M-5)), at most 256: one 2^11-point
// row per 64-thread CTA syncs only its own two warps (13% faster than four
// rows per 256-thread CTA on GB300)
#ifndef PREC_ROWS_THREADS
#define PREC_ROWS_THREADS 64
#endif

namespace precgpu {

// MR: pass radix cap.  With MR = 6 a 2^11-point row runs as a radix-64 and
// a radix-32 pass (no middle pass); the radix-64 top pass then takes the two
// operands one after the other (64 values in registers, not 128).
template <int SET, int M, bool SQ, int MR>
__global__ void __launch_bounds__(256, MR == 6 ? 2 : PREC_ROWS_MINB) k_rows(ProdArgs args, const ProdPtrs* __restrict__ batch) {
    extern __shared__ uint32_t sm[];
    constexpr int NP = sch_np(M, MR);
    static_assert(NP >= 2, "row transforms have at least two passes");
    constexpr int AS = astride_for(M);
    const ProdPtrs P = select_product(args, batch);
    const int prime = args.prime0 + blockIdx.y;
    const PrimeC pc = args.f.pc[prime];
    const uint2* __restrict__ twf = args.f.tf[prime];
    const uint2* __restrict__ twi = args.f.ti[prime];
    const int rows = args.rows;
    uint32_t* __restrict__ A = P.work + ((uint64_t)(prime * 2) << args.k);
    const uint32_t* __restrict__ B = A + (1ull << args.k);
    const uint32_t row0 = blockIdx.x * rows;
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
                x[0][q] = src[roff + ((uint32_t)q << G::LO)];
                if constexpr (NT == 2) x[1][q] = B[roff + ((uint32_t)q << G::LO)];
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

// ---------------------------------------------------------------------------

static size_t row_smem(int m, int rows) { return (size_t)rows * 2 * astride_for(m) * sizeof(uint32_t); }

// rows per CTA: PREC_ROWS_THREADS / 2^(M-5), fewer when the transform has
// too few rows to fill the GPU, never under one warp
int ntt_row_threads(int k2, int n1, int* rows_out) {
    int rows = PREC_ROWS_THREADS >> (k2 - 5);
    if (rows < 1) rows = 1;
    const int sms = device_sm_count();
    while (rows > 1 && (n1 / rows) * kPrimes < 2 * sms) rows >>= 1;
    int min_rows = k2 >= 10 ? 1 : (1 << (10 - k2));  // >= 32 threads
    if (rows < min_rows) rows = min_rows;
    if (rows > n1) rows = n1;
    *rows_out = rows;
    return rows << (k2 - 5);
}

// (set, M, radix cap): the cap changes the schedule of 2^10- and 2^11-point rows only
#define PREC_ROWS1(X, SQ)                                                                                      \
    X(0, 7, SQ, 4) X(0, 8, SQ, 4) X(0, 9, SQ, 4) X(0, 10, SQ, 4) X(0, 10, SQ, 6) X(0, 11, SQ, 4) X(0, 11, SQ, 6) \
    X(0, 12, SQ, 4) X(1, 13, SQ, 4)
#define PREC_ROWS(X) PREC_ROWS1(X, false) PREC_ROWS1(X, true)

void launch_rows(int set, const ProdArgs& a, cudaStream_t st, const ProdPtrs* batch, int count, int nprimes) {
    if (nprimes <= 0) nprimes = kSetPrimes[set];
    set = set_base(set);  // sets 2 and 3: the same kernel on their residues
    const int m = a.k2;
    const dim3 grid((1u << a.k1) / a.rows, nprimes, count);
    const int threads = a.rows << (m - 5);
    const size_t smem = row_smem(m, a.rows);
    const int mr = row_radix_cap(m, a.rmr);
#define X(S, MM, SQ, RR)                                                                  \
    if (set == S && m == MM && (a.square != 0) == SQ && mr == RR) {                       \
        launch_kernel(k_rows<S, MM, SQ, RR>, grid, threads, smem, st, a, batch);                 \
        count_launches(1);                                                              \
        return;                                                                         \
    }
    PREC_ROWS(X)
#undef X
}

int configure_rows() {
    cudaError_t e = cudaSuccess;
#define X(S, MM, SQ, RR)                                                                                      \
    if (!e) e = cudaFuncSetAttribute(k_rows<S, MM, SQ, RR>, cudaFuncAttributeMaxDynamicSharedMemorySize,     \
                                     (int)row_smem(MM, 256 >> (MM - 5) > 0 ? 256 >> (MM - 5) : 1));
    PREC_ROWS(X)
#undef X
    return (int)e;
}

}  // namespace precgpu
