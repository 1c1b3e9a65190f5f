// ntt_cols.cuh -- column passes of the four-step NTT (index i = i1*N2 + i2).
//
// k_fwd_cols: for C adjacent columns i2 of one operand and one prime, the
//   limbs are read as 32-bit digits (sets 2 and 3: whole 64-bit limbs) (the
//   reference's ntt_digits and mont_in, src/mul_ntt.cpp:331-342, 357-360,
//   fused into the load), reduced, run through a DIF transform over i1 (the
//   first log2(N1) stages of ntt_forward, mul_ntt.cpp:193-255) and
//   multiplied by the four-step twiddle w_N^(i2*k1).  Output row slot s
//   holds frequency k1 = bitrev(s).
// k_inv_cols: the inverse four-step twiddle w_N^-(i2*k1) times the prime's
//   CRT scale (CrtConst/Crt5Const::fold: the Garner constant that would
//   otherwise cost the CRT one product per prime and coefficient), then the
//   DIT transform over the row slots (the last stages of ntt_inverse,
//   mul_ntt.cpp:257-329) back to natural coefficient order.
// Both generate their twiddles as running Montgomery powers over a thread's
// 32 slots of one column (twiddle32).
// Columns are interleaved in shared memory (element i of column c at
// P(i)*C + c); a warp covers C columns x 32/C items, so every global access
// moves whole 32-byte sectors.
// Template parameters: SET prime set, M = log2 N1 (column length), C
// columns per CTA (launched with 32*C threads), MR the pass radix cap (MR = 6: a 2^11-point column runs
// as a radix-64 and a radix-32 pass; MR = 4: radix-8, -8, -32), K2 =
// log2 N2 (the row length, the stride between a column's elements) as a
// constant, or 0: from the arguments.  The instantiated (SET, M, C, MR)
// configurations are PREC_COLS_CONFIGS, with K2 = 0; the autotuner picks C
// and MR per transform length.  The default configuration of every
// transform length also has a K2 instantiation (PREC_COLS_*_K2_CONFIGS,
// ntt_cols_fwd_k2.cu, ntt_cols_inv_k2.cu).  Its global addresses are a
// constant offset from one base per item.  At 2^21 points on the 64-bit plan
// the forward columns measured 71.5 -> 63.1 us, and the inverse columns
// 34.8 -> 32.8 us.
#pragma once
#include "ntt_engine.cuh"

namespace precgpu {


// Top DIF pass of a digit tile whose upper half (rows 2^(M-1) and up) is
// zero -- every operand of at most N/2 digits, i.e. both operands of a
// balanced product: only the lower half is staged and reduced, and the
// first stage (x, 0) -> (x, x*w) needs one twiddle product per pair.
// Set 2 stages 64-bit limbs as two words per element (stage_limbs): the
// element's digit is read from its row and the row 2^(M-1) above it.
template <int SET, int M, int C, int MR>
__device__ __forceinline__ void col_top_upper_zero(uint32_t* sm, const uint2* __restrict__ tw, const PrimeC& c) {
    using G = Geom<M, 0, MR>;
    static_assert(G::LO >= 5, "the top pass of a multi-pass transform");
    constexpr int H = G::R / 2;
    for (int w = threadIdx.x; w < (C << G::LGI); w += blockDim.x) {
        const int col = w & (C - 1);
        const uint32_t u = w / C;
        const uint32_t ulo = u & G::LOMASK;
        uint32_t* s = sm + G::pbase(u) * C + col;
        uint32_t x[1][G::R];
#pragma unroll
        for (int q = 0; q < H; ++q) {
            uint32_t d;
            if constexpr (set_wide(SET)) d = Ar<SET>::digit64(s[q * G::QS * C], s[(q + H) * G::QS * C], c);
            else d = Ar<SET>::digit(s[q * G::QS * C], c);
            const uint2 wq = __ldg(&tw[(1u << (G::LO + G::RB - 1)) + (ulo | ((uint32_t)q << G::LO))]);
            x[0][q] = d;
            x[0][q + H] = Ar<SET>::twiddle(d, wq, c);
        }
        dif_regs<SET, G::LO, G::RB, 1, G::RB - 2>(x, ulo, tw, c);
#pragma unroll
        for (int q = 0; q < G::R; ++q) s[q * G::QS * C] = x[0][q];
    }
}

// The forward column pass: column group x (C columns) and y = prime*2 +
// operand (or just the prime for a square or a launch of one operand) of
// product z; nx = column groups per (prime, operand).
template <int SET, int M, int C, int MR, int K2 = 0>
__global__ void __launch_bounds__(256, cols_minb(M, MR)) k_fwd_cols(ProdArgs args, const ProdPtrs* __restrict__ batch) {
    extern __shared__ uint32_t sm[];
#define PREC_K2 K2
#define PREC_TILE_X blockIdx.x
#define PREC_TILE_Y blockIdx.y
#define PREC_TILE_NX gridDim.x
#define PREC_TILE_PRODUCT select_product(args, batch)
#include "ntt_cols_fwd_body.inc"
#undef PREC_K2
#undef PREC_TILE_X
#undef PREC_TILE_Y
#undef PREC_TILE_NX
#undef PREC_TILE_PRODUCT
}

// The forward column pass of one prime of a 64-bit-digit product, software
// pipelined: each CTA takes every gridDim.x-th column group of its (prime,
// operand) and stages the next group's limbs into a second tile buffer while
// it transforms the current one.  The single product's per-prime chains
// launch it (five launches side by side) for the 1M x 1M class: there it
// measured 0.1782 -> 0.1741-0.1751 ms, and with both kernels compiled for
// the constant row length 0.1690 -> 0.1672 ms (2 or 4 tiles per CTA: 0.1679,
// 0.1685-0.1692).  As one launch over all primes the one-tile kernel stays
// faster (71 against 77 us), and on set 3's 4M x 4M it measured slower.
constexpr int kFwdPipeTiles = 3;  // column groups per CTA
template <int SET, int M, int C, int MR, int K2>
__global__ void __launch_bounds__(256, 3) k_fwd_cols_pipe(ProdArgs args, const ProdPtrs* __restrict__ batch) {
    static_assert(set_wide(SET), "64-bit digits: whole limbs staged");
    static_assert(K2 > 0, "a constant row length");
    extern __shared__ uint32_t sm[];
    constexpr int NP = sch_np(M, MR);
    constexpr int TW = C * astride_for(M);  // words per tile buffer
    const ProdPtrs P = select_product(args, batch);
    const bool one = args.square || args.operand_only;
    const int prime = args.prime0 + (one ? blockIdx.y : blockIdx.y >> 1);
    const int operand = args.operand_only ? args.operand_only - 1 : (one ? 0 : blockIdx.y & 1);
    const PrimeC pc = args.f.pc[prime];
    const uint2* __restrict__ tw = args.f.tf[prime];
    constexpr uint32_t N2 = 1u << K2;
    constexpr int KK = M + K2;  // log2 of the transform length
    constexpr int nbx = (int)(N2 / C);
    if (args.publish && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) *args.publish = P;
    const uint64_t nl = operand ? P.lb : P.la;
    if (nl > (1ull << (KK - 1))) {  // the plan puts both operands in the lower half
        if (threadIdx.x == 0) atomicOr(args.err, kDevErrPlan);
        return;
    }
    const uint64_t* src = operand ? P.b : P.a;
    uint32_t* __restrict__ dst = P.work + ((uint64_t)(prime * 2 + operand) << KK);
    uint32_t* cur = sm;
    uint32_t* nxt = sm + TW;
    int bx = blockIdx.x;
    if (bx < nbx) stage_limbs_issue<M, C>(cur, src, N2, (uint64_t)bx * C, nl);
    for (; bx < nbx; bx += gridDim.x) {
        const int bn = bx + gridDim.x;
        if (bn < nbx) {
            stage_limbs_issue<M, C>(nxt, src, N2, (uint64_t)bn * C, nl);
            cp_async_wait<1>();  // this tile's group done, the next one in flight
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        // the carry kernel's look-back words start at zero
        if (blockIdx.y == 0 && args.prime0 == 0) {
            for (int i = bx * blockDim.x + threadIdx.x; i <= P.nblk; i += nbx * blockDim.x) P.scratch[i] = 0;
        }
        const uint32_t c0 = (uint32_t)bx * C;
        col_top_upper_zero<SET, M, C, MR>(cur, tw, pc);
        __syncthreads();
        col_passes<SET, M, 1, NP - 2, false, C, MR>(cur, tw, pc);
        {   // bottom pass with the four-step twiddle, straight to HBM
            using G = Geom<M, NP - 1, MR>;
            static_assert(G::LO == 0 && G::RB == 5, "bottom pass covers bits 0..4");
            const double ip = 4294967296.0 / (double)pc.p;  // 2^32 / p for twiddle32_shoup
            for (int w = threadIdx.x; w < (C << G::LGI); w += blockDim.x) {
                const int col = w & (C - 1);
                const uint32_t u = w / C;
                const uint32_t* s = cur + (33 * u) * C + col;
                const uint32_t i2 = c0 + col;
                const uint32_t t = fourstep_twiddle<SET>(args.f, prime, i2 * brev_bits(u, M - 5), KK);
                const uint32_t g = fourstep_twiddle<SET>(args.f, prime, i2 << (M - 5), KK);
                uint32_t x[1][32];
#pragma unroll
                for (int q = 0; q < 32; ++q) x[0][q] = s[q * C];
                regs_pass<SET, M, NP - 1, false, 1, MR>(x, u, tw, pc);
                twiddle32_shoup<SET>(x[0], t, g, pc, ip);
#pragma unroll
                for (int q = 0; q < 32; ++q) dst[(uint64_t)(32 * u + q) * N2 + i2] = x[0][q];
            }
        }
        __syncthreads();  // every thread is done with `cur` before it is refilled
        uint32_t* t = cur;
        cur = nxt;
        nxt = t;
    }
}

// One tile of the forward column pass at the indices ix (a persistent kernel's).
template <int SET, int M, int C, int MR>
__device__ __forceinline__ void fwd_cols_tile(const ProdArgs& args, const ProdPtrs* __restrict__ batch,
                                              const TileIdx& ix, uint32_t* sm) {
#define PREC_K2 0
#define PREC_TILE_X ix.bx
#define PREC_TILE_Y ix.by
#define PREC_TILE_NX ix.nbx
#define PREC_TILE_PRODUCT select_product_at(args, batch, ix.bz)
#include "ntt_cols_fwd_body.inc"
#undef PREC_K2
#undef PREC_TILE_X
#undef PREC_TILE_Y
#undef PREC_TILE_NX
#undef PREC_TILE_PRODUCT
}

// The inverse column pass: column group x, prime args.prime0 + y of
// product z.
template <int SET, int M, int C, int MR, int K2 = 0>
__global__ void __launch_bounds__(256, cols_minb(M, MR)) k_inv_cols(ProdArgs args, const ProdPtrs* __restrict__ batch) {
    extern __shared__ uint32_t sm[];
#define PREC_K2 K2
#define PREC_TILE_X blockIdx.x
#define PREC_TILE_Y blockIdx.y
#define PREC_TILE_PRODUCT select_product(args, batch)
#include "ntt_cols_inv_body.inc"
#undef PREC_K2
#undef PREC_TILE_X
#undef PREC_TILE_Y
#undef PREC_TILE_PRODUCT
}

// One tile of the inverse column pass at the indices ix.
template <int SET, int M, int C, int MR>
__device__ __forceinline__ void inv_cols_tile(const ProdArgs& args, const ProdPtrs* __restrict__ batch,
                                              const TileIdx& ix, uint32_t* sm) {
#define PREC_K2 0
#define PREC_TILE_X ix.bx
#define PREC_TILE_Y ix.by
#define PREC_TILE_PRODUCT select_product_at(args, batch, ix.bz)
#include "ntt_cols_inv_body.inc"
#undef PREC_K2
#undef PREC_TILE_X
#undef PREC_TILE_Y
#undef PREC_TILE_PRODUCT
}

// ---------------------------------------------------------------------------

#define PREC_COLS_CONFIGS(X)                                                                            \
    X(0, 6, 4, 6) X(0, 6, 8, 6) X(0, 7, 4, 6) X(0, 7, 8, 6) X(0, 8, 4, 6) X(0, 8, 8, 6) X(0, 9, 4, 6)     \
    X(0, 9, 8, 6) X(0, 10, 4, 4) X(0, 10, 8, 4) X(0, 10, 4, 6) X(0, 10, 8, 6) X(0, 11, 4, 4)              \
    X(0, 11, 8, 4) X(0, 11, 4, 6) X(0, 11, 8, 6) X(1, 11, 4, 4) X(1, 11, 8, 4) X(1, 11, 4, 6)             \
    X(1, 11, 8, 6) X(1, 12, 4, 6) X(1, 13, 4, 6) X(1, 10, 4, 6) X(1, 10, 8, 6)

// the forward column kernels of sets 2 and 3 (64-bit digits) in the
// (M, C, MR) configurations of sets 0 and 1; their other kernels are set 0's
// and set 1's
#define PREC_COLS_WIDE_CONFIGS(X)                                                                       \
    X(2, 6, 4, 6) X(2, 6, 8, 6) X(2, 7, 4, 6) X(2, 7, 8, 6) X(2, 8, 4, 6) X(2, 8, 8, 6) X(2, 9, 4, 6)     \
    X(2, 9, 8, 6) X(2, 10, 4, 4) X(2, 10, 8, 4) X(2, 10, 4, 6) X(2, 10, 8, 6) X(2, 11, 4, 4)              \
    X(2, 11, 8, 4) X(2, 11, 4, 6) X(2, 11, 8, 6) X(3, 10, 4, 6) X(3, 10, 8, 6) X(3, 11, 4, 4)             \
    X(3, 11, 8, 4) X(3, 11, 4, 6) X(3, 11, 8, 6) X(3, 12, 4, 6)

// (SET, M, C, MR, K2) of the default configurations (sets 0 and 2: N1 =
// 2^floor(k/2); sets 1 and 3: N2 = 2^13), compiled with a constant row
// length.  The inverse columns of sets 2 and 3 are set 0's and set 1's.
#define PREC_COLS_FWD_K2_CONFIGS(X)                                                                        \
    X(0, 6, 8, 6, 7) X(0, 7, 8, 6, 7) X(0, 7, 8, 6, 8) X(0, 8, 8, 6, 8) X(0, 8, 8, 6, 9) X(0, 9, 8, 6, 9)   \
    X(0, 9, 8, 6, 10) X(0, 10, 8, 6, 10) X(0, 10, 8, 6, 11) X(0, 11, 8, 6, 11) X(0, 11, 8, 6, 12)           \
    X(2, 9, 8, 6, 9) X(2, 9, 8, 6, 10) X(2, 10, 8, 6, 10) X(2, 10, 8, 6, 11) X(2, 11, 8, 6, 11)             \
    X(1, 11, 8, 6, 13) X(1, 12, 4, 6, 13) X(1, 13, 4, 6, 13) X(3, 10, 8, 6, 13) X(3, 11, 8, 6, 13)         \
    X(3, 12, 4, 6, 13)
#define PREC_COLS_INV_K2_CONFIGS(X)                                                                        \
    X(0, 6, 8, 6, 7) X(0, 7, 8, 6, 7) X(0, 7, 8, 6, 8) X(0, 8, 8, 6, 8) X(0, 8, 8, 6, 9) X(0, 9, 8, 6, 9)   \
    X(0, 9, 8, 6, 10) X(0, 10, 8, 6, 10) X(0, 10, 8, 6, 11) X(0, 11, 8, 6, 11) X(0, 11, 8, 6, 12)           \
    X(1, 10, 8, 6, 13) X(1, 11, 8, 6, 13) X(1, 12, 4, 6, 13) X(1, 13, 4, 6, 13)

inline size_t col_smem(int m, int cg) { return (size_t)cg * astride_for(m) * sizeof(uint32_t); }

// the K2 instantiations (ntt_cols_fwd_k2.cu, ntt_cols_inv_k2.cu): launch the
// one matching (set, a.k1, cg, mr, a.k2) and return true, or return false.
// one_prime: a single product's launch for one prime (the per-prime chains)
bool launch_fwd_cols_k2(int set, const ProdArgs& a, int cg, int mr, dim3 grid, size_t smem, cudaStream_t st,
                        const ProdPtrs* batch, bool one_prime);
bool launch_inv_cols_k2(int set, const ProdArgs& a, int cg, int mr, dim3 grid, size_t smem, cudaStream_t st,
                        const ProdPtrs* batch);
int configure_fwd_cols_k2();
int configure_inv_cols_k2();

}  // namespace precgpu
