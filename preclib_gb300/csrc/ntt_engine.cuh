// ntt_engine.cuh -- device-side transform engine shared by the NTT kernels.
//
// A sub-transform of 2^M points lives in shared memory with one spare word
// per 32 (padded index P(i) = i + i/32) and is processed in register passes
// of radix 2^RB over index bits [LO, LO+RB).  The pass schedule is fixed at
// compile time: the lowest pass always covers bits 0..4 (RB = 5), every
// other pass starts at bit 5 or above.  With that schedule the 32 lanes of
// a warp touch 32 distinct banks in every pass, and every shared-memory
// address is a per-thread base plus an immediate offset.
#pragma once
#include <cuda_runtime.h>

#include "ntt_field.cuh"
#include "ntt_kernels.cuh"

// minimum resident 256-thread CTAs per SM the transform kernels are
// compiled for (register budget 65536 / (256 * n))
#ifndef PREC_ROWS_MINB
#define PREC_ROWS_MINB 3
#endif
// column kernels: 4 CTAs (64 registers) unless a radix-64 pass of a
// 2^11-point column holds 64 values per thread (3 CTAs, 85 registers: at 64
// those kernels spill 300-450 bytes)
#ifndef PREC_COLS_MINB
#define PREC_COLS_MINB 4
#endif
#ifndef PREC_COLS_MINB_R64
#define PREC_COLS_MINB_R64 3
#endif
__host__ __device__ constexpr int cols_minb(int m, int mr) {
    return m >= 11 && mr == 6 ? PREC_COLS_MINB_R64 : PREC_COLS_MINB;
}
// unroll factor of the item loops of the shared-memory passes
#ifndef PREC_PASS_UNROLL
#define PREC_PASS_UNROLL 1
#endif

namespace precgpu {

typedef unsigned __int128 u128;

constexpr int kPassUnroll = PREC_PASS_UNROLL;

// ---------------------------------------------------------------------------
// compile-time pass schedule (t = 0 is the top pass, t = np-1 the bottom)
// ---------------------------------------------------------------------------
#ifndef PREC_SCH_MAXRB
#define PREC_SCH_MAXRB 4
#endif
// passes above the bottom one cover at most mr bits each (the radix cap;
// PREC_SCH_MAXRB is the default of the translation unit)
__host__ __device__ constexpr int sch_np(int m, int mr = PREC_SCH_MAXRB) {
    return m <= 5 ? 1 : 1 + (m - 5 + mr - 1) / mr;
}
__host__ __device__ constexpr int sch_rb(int m, int t, int mr = PREC_SCH_MAXRB) {
    return m <= 5 ? m
                  : (t == sch_np(m, mr) - 1
                         ? 5
                         : (m - 5) / (sch_np(m, mr) - 1) + (t < (m - 5) % (sch_np(m, mr) - 1) ? 1 : 0));
}
__host__ __device__ constexpr int sch_lo(int m, int t, int mr = PREC_SCH_MAXRB) {
    return t < 0 ? m : sch_lo(m, t - 1, mr) - sch_rb(m, t, mr);
}

__host__ __device__ constexpr int padded(int n) { return n + (n >> 5); }

// words per array in shared memory (== 4 mod 8)
__host__ __device__ constexpr int astride_for(int m) { return ((padded(1 << m) + 7) & ~7) + 4; }

template <int M, int T, int MR = PREC_SCH_MAXRB>
struct Geom {
    static constexpr int RB = sch_rb(M, T, MR);
    static constexpr int LO = sch_lo(M, T, MR);
    static constexpr int R = 1 << RB;
    static constexpr int LGI = M - RB;  // log2 of items per array
    static constexpr uint32_t LOMASK = (1u << LO) - 1;
    // padded distance between consecutive elements of one item
    static constexpr uint32_t QS = LO >= 5 ? (1u << LO) + (1u << (LO - 5)) : 1u;
    static __device__ __forceinline__ uint32_t base(uint32_t u) {
        return ((u >> LO) << (LO + RB)) | (u & LOMASK);
    }
    static __device__ __forceinline__ uint32_t pbase(uint32_t u) {
        const uint32_t b = base(u);
        return b + (b >> 5);
    }
};

// ---------------------------------------------------------------------------
// register passes
// ---------------------------------------------------------------------------

// DIF stages over bits BTOP+LO .. LO of NA arrays held in registers
// (BTOP = RB-1: all RB stages); element q of an item sits at index
// base + (q << LO); ulo = base & LOMASK.
template <int SET, int LO, int RB, int NA, int BTOP = RB - 1>
__device__ __forceinline__ void dif_regs(uint32_t (&x)[NA][1 << RB], uint32_t ulo, const uint2* __restrict__ tw,
                                         const PrimeC& c) {
#pragma unroll
    for (int bb = BTOP; bb >= 0; --bb) {
        const int h = 1 << bb;
        if constexpr (LO == 0) {
#pragma unroll
            for (int j = 0; j < h; j += 2) {
                uint2 w0 = make_uint2(1, 0), w1 = w0;
                if (h >= 2) {
                    const uint4 v = __ldg(reinterpret_cast<const uint4*>(tw + (1u << bb) + j));
                    w0 = make_uint2(v.x, v.y);
                    w1 = make_uint2(v.z, v.w);
                }
#pragma unroll
                for (int q0 = 0; q0 < (1 << RB); q0 += 2 * h) {
#pragma unroll
                    for (int a = 0; a < NA; ++a) {
                        if (j == 0) Ar<SET>::dif1(x[a][q0], x[a][q0 + h], c);
                        else Ar<SET>::dif(x[a][q0 + j], x[a][q0 + j + h], w0, c);
                        if (h >= 2) Ar<SET>::dif(x[a][q0 + j + 1], x[a][q0 + j + 1 + h], w1, c);
                    }
                }
            }
        } else {
#pragma unroll
            for (int q = 0; q < (1 << RB); ++q) {
                if (q & h) continue;
                const uint32_t j = ulo | ((uint32_t)(q & (h - 1)) << LO);
                const uint2 w = __ldg(&tw[(1u << (LO + bb)) + j]);
#pragma unroll
                for (int a = 0; a < NA; ++a) Ar<SET>::dif(x[a][q], x[a][q + h], w, c);
            }
        }
    }
}

// DIT stages over bits LO .. LO+RB-1.
template <int SET, int LO, int RB, int NA>
__device__ __forceinline__ void dit_regs(uint32_t (&x)[NA][1 << RB], uint32_t ulo, const uint2* __restrict__ tw,
                                         const PrimeC& c) {
#pragma unroll
    for (int bb = 0; bb < RB; ++bb) {
        const int h = 1 << bb;
        if constexpr (LO == 0) {
#pragma unroll
            for (int j = 0; j < h; j += 2) {
                uint2 w0 = make_uint2(1, 0), w1 = w0;
                if (h >= 2) {
                    const uint4 v = __ldg(reinterpret_cast<const uint4*>(tw + (1u << bb) + j));
                    w0 = make_uint2(v.x, v.y);
                    w1 = make_uint2(v.z, v.w);
                }
#pragma unroll
                for (int q0 = 0; q0 < (1 << RB); q0 += 2 * h) {
#pragma unroll
                    for (int a = 0; a < NA; ++a) {
                        if (j == 0) Ar<SET>::dit1(x[a][q0], x[a][q0 + h], c);
                        else Ar<SET>::dit(x[a][q0 + j], x[a][q0 + j + h], w0, c);
                        if (h >= 2) Ar<SET>::dit(x[a][q0 + j + 1], x[a][q0 + j + 1 + h], w1, c);
                    }
                }
            }
        } else {
#pragma unroll
            for (int q = 0; q < (1 << RB); ++q) {
                if (q & h) continue;
                const uint32_t j = ulo | ((uint32_t)(q & (h - 1)) << LO);
                const uint2 w = __ldg(&tw[(1u << (LO + bb)) + j]);
#pragma unroll
                for (int a = 0; a < NA; ++a) Ar<SET>::dit(x[a][q], x[a][q + h], w, c);
            }
        }
    }
}

template <int SET, int M, int T, bool DIT, int NA, int MR = PREC_SCH_MAXRB>
__device__ __forceinline__ void regs_pass(uint32_t (&x)[NA][Geom<M, T, MR>::R], uint32_t u,
                                          const uint2* __restrict__ tw, const PrimeC& c) {
    using G = Geom<M, T, MR>;
    if constexpr (DIT) dit_regs<SET, G::LO, G::RB, NA>(x, u & G::LOMASK, tw, c);
    else dif_regs<SET, G::LO, G::RB, NA>(x, u & G::LOMASK, tw, c);
}

// ---------------------------------------------------------------------------
// shared-memory passes
// ---------------------------------------------------------------------------

// Row layout: array a at sm + a*astride, element i at P(i).  Items of NA
// arrays share twiddle loads.  narr must be a multiple of NA.
template <int SET, int M, int T, bool DIT, int NA, int MR = PREC_SCH_MAXRB>
__device__ __forceinline__ void row_pass(uint32_t* sm, int astride, int narr, const uint2* __restrict__ tw,
                                         const PrimeC& c) {
    using G = Geom<M, T, MR>;
    const int total = (narr / NA) << G::LGI;
#pragma unroll kPassUnroll
    for (int w = threadIdx.x; w < total; w += blockDim.x) {
        const uint32_t u = w & ((1u << G::LGI) - 1);
        const int g = w >> G::LGI;
        uint32_t* s = sm + g * NA * astride + G::pbase(u);
        uint32_t x[NA][G::R];
#pragma unroll
        for (int a = 0; a < NA; ++a)
#pragma unroll
            for (int q = 0; q < G::R; ++q) x[a][q] = s[a * astride + q * G::QS];
        regs_pass<SET, M, T, DIT, NA, MR>(x, u, tw, c);
#pragma unroll
        for (int a = 0; a < NA; ++a)
#pragma unroll
            for (int q = 0; q < G::R; ++q) s[a * astride + q * G::QS] = x[a][q];
    }
}

// 16-byte asynchronous copy global -> shared; bytes past src_bytes (0..16)
// are zero-filled and not read
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, int src_bytes) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(s), "l"(gmem), "r"(src_bytes) : "memory");
}
// 4-byte asynchronous copy (src_bytes 0 or 4; 0 zero-fills without reading)
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem, int src_bytes) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(s), "l"(gmem), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// waits until at most N of this thread's committed groups are pending
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Stages rows [0, 2^M) x columns [c0, c0+C) of a row-major u32 matrix with
// row length `ld` into the column layout (element i of column c at
// P(i)*C + c); `valid` = number of meaningful elements of the matrix
// (row-major index), the rest read as zero.  16-byte copies when the
// matrix starts on a 16-byte boundary (ld and c0 are multiples of 4), else
// 4-byte copies: operand limb arrays are only guaranteed 8-byte aligned.
// stage_rows issues the copies of rows [r0, r1) only and commits them as
// one group (cp_async_wait<n> then waits for all but the last n groups).
template <int M, int C>
__device__ __forceinline__ void stage_rows(uint32_t* sm, const uint32_t* __restrict__ g, uint64_t ld, uint64_t c0,
                                           uint64_t valid, int r0, int r1) {
    constexpr int Q = C / 4;
    if (((uintptr_t)g & 15) == 0) {
        for (int w = r0 * Q + threadIdx.x; w < r1 * Q; w += blockDim.x) {
            const int r = w / Q, h = w % Q;
            const uint64_t idx = (uint64_t)r * ld + c0 + 4 * h;
            const int bytes = idx >= valid ? 0 : (valid - idx >= 4 ? 16 : (int)(valid - idx) * 4);
            cp_async16(sm + padded(r) * C + 4 * h, bytes ? g + idx : g, bytes);
        }
    } else {
        for (int w = r0 * C + threadIdx.x; w < r1 * C; w += blockDim.x) {
            const int r = w / C, col = w % C;
            const uint64_t idx = (uint64_t)r * ld + c0 + col;
            const bool in = idx < valid;
            cp_async4(sm + padded(r) * C + col, in ? g + idx : g, in ? 4 : 0);
        }
    }
    cp_async_commit();
}

// Whole 64-bit limbs (set 2) of an operand in the lower half of the tile:
// rows i1 < 2^(M-1) of C columns; the low word of limb i1*ld + c0 + col
// goes to row i1 and the high word to row i1 + 2^(M-1), the two elements
// the top pass pairs anyway (limbs past `valid` read as zero).
// Both words go by 4-byte asynchronous copies, all of a thread's copies in
// flight at once (a load-then-store loop waited out the memory latency once
// per limb: on GB300 that staging took 44% of the forward column pass).
template <int M, int C>
__device__ __forceinline__ void stage_limbs(uint32_t* sm, const uint64_t* __restrict__ g, uint64_t ld, uint64_t c0,
                                            uint64_t valid) {
    constexpr int H = 1 << (M - 1);
    const uint32_t* __restrict__ g32 = reinterpret_cast<const uint32_t*>(g);
    for (int w = threadIdx.x; w < H * C; w += blockDim.x) {
        const int r = w / C, col = w % C;
        const uint64_t idx = (uint64_t)r * ld + c0 + col;
        const bool in = idx < valid;
        const uint32_t* src = in ? g32 + 2 * idx : g32;  // 0 bytes read (zero fill) past the operand
        cp_async4(sm + padded(r) * C + col, src, in ? 4 : 0);
        cp_async4(sm + padded(r + H) * C + col, in ? src + 1 : g32, in ? 4 : 0);
    }
    cp_async_commit();
    cp_async_wait<0>();
}

// stage_limbs without the wait: the copies of one tile as one committed
// group, left in flight (the pipelined forward columns prefetch the next tile)
template <int M, int C>
__device__ __forceinline__ void stage_limbs_issue(uint32_t* sm, const uint64_t* __restrict__ g, uint64_t ld,
                                                  uint64_t c0, uint64_t valid) {
    constexpr int H = 1 << (M - 1);
    const uint32_t* __restrict__ g32 = reinterpret_cast<const uint32_t*>(g);
    for (int w = threadIdx.x; w < H * C; w += blockDim.x) {
        const int r = w / C, col = w % C;
        const uint64_t idx = (uint64_t)r * ld + c0 + col;
        const bool in = idx < valid;
        const uint32_t* src = in ? g32 + 2 * idx : g32;  // 0 bytes read (zero fill) past the operand
        cp_async4(sm + padded(r) * C + col, src, in ? 4 : 0);
        cp_async4(sm + padded(r + H) * C + col, in ? src + 1 : g32, in ? 4 : 0);
    }
    cp_async_commit();
}

template <int M, int C>
__device__ __forceinline__ void stage_cols(uint32_t* sm, const uint32_t* __restrict__ g, uint64_t ld, uint64_t c0,
                                           uint64_t valid) {
    stage_rows<M, C>(sm, g, ld, c0, valid, 0, 1 << M);
    cp_async_wait<0>();
}

// Column layout: C interleaved columns, element i of column c at
// P(i)*C + c; lanes cover C adjacent columns (twiddle loads broadcast).
// DIGIT: the values are raw 32-bit digits, reduced on load.  Items
// [w0, w1) of the pass (w1 < 0: all C << LGI items).
template <int SET, int M, int T, bool DIT, int C, bool DIGIT = false, int MR = PREC_SCH_MAXRB>
__device__ __forceinline__ void col_pass(uint32_t* sm, const uint2* __restrict__ tw, const PrimeC& c, int w0 = 0,
                                         int w1 = -1) {
    using G = Geom<M, T, MR>;
    const int total = w1 < 0 ? (C << G::LGI) : w1;
#pragma unroll kPassUnroll
    for (int w = w0 + threadIdx.x; w < total; w += blockDim.x) {
        const int col = w & (C - 1);
        const uint32_t u = w / C;
        uint32_t* s = sm + G::pbase(u) * C + col;
        uint32_t x[1][G::R];
#pragma unroll
        for (int q = 0; q < G::R; ++q) x[0][q] = DIGIT ? Ar<SET>::digit(s[q * G::QS * C], c) : s[q * G::QS * C];
        regs_pass<SET, M, T, DIT, 1, MR>(x, u, tw, c);
#pragma unroll
        for (int q = 0; q < G::R; ++q) s[q * G::QS * C] = x[0][q];
    }
}

// Middle passes T in [T0, T1] (ascending for DIF, descending for DIT).
template <int SET, int M, int T, int TEND, bool DIT, int NA, int MR = PREC_SCH_MAXRB>
__device__ __forceinline__ void row_passes(uint32_t* sm, int astride, int narr, const uint2* __restrict__ tw,
                                           const PrimeC& c) {
    if constexpr (DIT ? (T >= TEND) : (T <= TEND)) {
        row_pass<SET, M, T, DIT, NA, MR>(sm, astride, narr, tw, c);
        __syncthreads();
        row_passes<SET, M, DIT ? T - 1 : T + 1, TEND, DIT, NA, MR>(sm, astride, narr, tw, c);
    }
}

template <int SET, int M, int T, int TEND, bool DIT, int C, int MR = PREC_SCH_MAXRB>
__device__ __forceinline__ void col_passes(uint32_t* sm, const uint2* __restrict__ tw, const PrimeC& c) {
    if constexpr (DIT ? (T >= TEND) : (T <= TEND)) {
        col_pass<SET, M, T, DIT, C, false, MR>(sm, tw, c);
        __syncthreads();
        col_passes<SET, M, DIT ? T - 1 : T + 1, TEND, DIT, C, MR>(sm, tw, c);
    }
}

// bit reversal of the low `bits` bits
__device__ __forceinline__ uint32_t brev_bits(uint32_t x, int bits) { return bits ? __brev(x) >> (32 - bits) : 0u; }

__host__ __device__ constexpr int brev5(int q) {
    return ((q & 1) << 4) | ((q & 2) << 2) | (q & 4) | ((q & 8) >> 2) | ((q & 16) >> 4);
}

// w^e * 2^32 mod p (Montgomery form, [0, 2p)) for a root w of order
// N = 2^k, e < N; two-level table over the set's largest root.
template <int SET>
__device__ __forceinline__ uint32_t fourstep_twiddle(const FieldArgs& f, int prime, uint32_t e, int k) {
    const uint32_t E = e << (f.max_log2 - k);
    const uint32_t hi = __ldg(&f.twhi[prime][E >> kTwLevelBits]);
    const uint32_t lo = __ldg(&f.twlo[prime][E & ((1u << kTwLevelBits) - 1)]);
    return Ar<SET>::mul(hi, lo, f.pc[prime]);
}

// x[brev5(j)] *= t * g^j for j = 0 .. 31 (t, g in Montgomery form; [0, 2p)
// under set 0's arithmetic): the four-step twiddles of a thread's 32 slots
// of one column as a running power.  (Four interleaved chains stepping by
// g^4 measured no faster on GB300: the chain is not latency-bound.)
template <int SET>
__device__ __forceinline__ void twiddle32(uint32_t (&x)[32], uint32_t t, uint32_t g, const PrimeC& pc) {
#pragma unroll
    for (int j = 0; j < 32; ++j) {
        const int q = brev5(j);
        x[q] = Ar<SET>::mul(x[q], t, pc);
        if (j < 31) t = Ar<SET>::mul(t, g, pc);
    }
}

// twiddle32 with the chain's step t*g as a Shoup product (one high and two
// low products instead of Montgomery's two wide and one low): g goes to
// plain form below p, and its quotient floor(g 2^32 / p) comes from the
// double estimate g * ip (ip = 2^32 / p; error far below 1) and one
// correction.  Used by the pipelined forward columns (1M x 1M 0.1679 ->
// 0.1661-0.1675 ms); in the other column kernels it measured slower (the
// inverse kernels spilled 16-20 bytes more).
template <int SET>
__device__ __forceinline__ void twiddle32_shoup(uint32_t (&x)[32], uint32_t t, uint32_t g, const PrimeC& pc,
                                                double ip) {
    const uint32_t gp = red1(mont_lazy(g, 1u, pc), pc.p);
    uint32_t gq = (uint32_t)((double)gp * ip);
    const int64_t r = (int64_t)((uint64_t)gp << 32) - (int64_t)((uint64_t)gq * pc.p);
    if (r < 0) --gq;
    else if (r >= (int64_t)pc.p) ++gq;
#pragma unroll
    for (int j = 0; j < 32; ++j) {
        const int q = brev5(j);
        x[q] = Ar<SET>::mul(x[q], t, pc);
        if (j < 31) t = shoup_lazy(t, gp, gq, pc.p);
    }
}

// ---------------------------------------------------------------------------
// CRT and carries
// ---------------------------------------------------------------------------

// Garner recombination of the three inverse-transform outputs (any value
// below 2^32 of each residue class) into the exact coefficient below
// p1*p2*p3, with the transform scale folded into the constants
// (src/mul_ntt.cpp:405-424 recombines its primes the same way).
__device__ __forceinline__ u128 crt3(uint32_t y1, uint32_t y2, uint32_t y3, const CrtConst& cc, const FieldArgs& f) {
    const uint32_t p1 = f.pc[0].p, p2 = f.pc[1].p, p3 = f.pc[2].p;
    const uint32_t v1 = shoup_mul(y1, cc.s1, p1);
    const uint32_t v2 = sub_mod(shoup_mul(y2, cc.k22, p2), shoup_mul(v1, cc.k21, p2), p2);
    uint32_t v3 = sub_mod(shoup_mul(y3, cc.k33, p3), shoup_mul(v1, cc.k31, p3), p3);
    v3 = sub_mod(v3, shoup_mul(v2, cc.k32, p3), p3);
    const uint64_t t = (uint64_t)v2 + (uint64_t)p2 * v3;
    return (u128)t * p1 + v1;
}

// crt3 of the four-step path: the inverse column pass has already
// multiplied y_j by s1, k22, k33 (CrtConst::fold), so y_j is v1's, and
// v2's and v3's first term.  Set 0 leaves y_j in [0, 4p), set 1 in [0, p).
template <int SET>
__device__ __forceinline__ u128 crt3_folded(uint32_t y1, uint32_t y2, uint32_t y3, const CrtConst& cc,
                                            const FieldArgs& f) {
    const uint32_t p1 = f.pc[0].p, p2 = f.pc[1].p, p3 = f.pc[2].p;
    if constexpr (SET == 0) {
        y1 = red1(red1(y1, f.pc[0].p2), p1);
        y2 = red1(red1(y2, f.pc[1].p2), p2);
        y3 = red1(red1(y3, f.pc[2].p2), p3);
    }
    const uint32_t v1 = y1;
    const uint32_t v2 = sub_mod(y2, shoup_mul(v1, cc.k21, p2), p2);
    uint32_t v3 = sub_mod(y3, shoup_mul(v1, cc.k31, p3), p3);
    v3 = sub_mod(v3, shoup_mul(v2, cc.k32, p3), p3);
    const uint64_t t = (uint64_t)v2 + (uint64_t)p2 * v3;
    return (u128)t * p1 + v1;
}

// Carry-in of every lane from the lanes' (G, P) bits: the chain
// c_{t+1} = G_t | (P_t & c_t) is the carry chain of the sum A + B with
// A = G|P, B = G (G and P are disjoint), so the carry into lane t is bit t
// of (A + B + cin) ^ A ^ B.
__device__ __forceinline__ uint64_t carry_chain(uint32_t G, uint32_t P, bool cin) {
    const uint64_t A = (uint64_t)(G | P), B = (uint64_t)G;
    return (A + B + (cin ? 1u : 0u)) ^ A ^ B;  // bit t: carry into t; bit 32: carry out
}

struct BlockCarryShared {
    uint32_t wg[32], wp[32];
    uint32_t block_cin;
};

// Block-wide carry resolution: every thread holds (G, P) of its limbs; the
// block aggregate (Gb, Pb) goes to cin_fn (thread 0 only), which returns
// the block's carry-in; returns the thread's carry-in.
template <class CinFn>
__device__ __forceinline__ bool block_carry(bool G, bool P, BlockCarryShared& sh, CinFn cin_fn) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = (blockDim.x + 31) >> 5;
    const uint32_t gm = __ballot_sync(0xffffffffu, G);
    const uint32_t pm = __ballot_sync(0xffffffffu, P);
    if (lane == 0) {
        sh.wg[warp] = (uint32_t)(carry_chain(gm, pm, false) >> 32) & 1;
        sh.wp[warp] = pm == 0xffffffffu;
    }
    __syncthreads();
    if (warp == 0) {
        const bool wG = lane < nwarps ? sh.wg[lane] != 0 : false;
        const bool wP = lane < nwarps ? sh.wp[lane] != 0 : true;
        const uint32_t real = nwarps >= 32 ? 0xffffffffu : ((1u << nwarps) - 1);
        const uint32_t bg = __ballot_sync(0xffffffffu, wG) & real;
        const uint32_t bp = __ballot_sync(0xffffffffu, wP) & real;
        const uint64_t c0 = carry_chain(bg, bp, false);
        const bool Gb = (c0 >> nwarps) & 1;
        const bool Pb = bp == real;
        uint32_t bcin = 0;
        if (lane == 0) bcin = cin_fn(Gb, Pb) ? 1u : 0u;
        bcin = __shfl_sync(0xffffffffu, bcin, 0);
        const uint64_t cw = carry_chain(bg, bp, bcin != 0);
        __syncwarp();
        if (lane < nwarps) sh.wg[lane] = (uint32_t)(cw >> lane) & 1;  // carry into warp `lane`
    }
    __syncthreads();
    const bool wcin = sh.wg[warp] != 0;
    const uint64_t cl = carry_chain(gm, pm, wcin);
    return (cl >> lane) & 1;
}

// Block-wide carry resolution with a block carry-in of 0, one barrier:
// every warp derives its own carry-in from the warp aggregates below it;
// thread 0 hands the block aggregate (Gb, Pb) to publish.  Returns the
// thread's carry-in.
template <class PublishFn>
__device__ __forceinline__ bool block_carry_in0(bool G, bool P, BlockCarryShared& sh, PublishFn publish) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = (blockDim.x + 31) >> 5;
    const uint32_t gm = __ballot_sync(0xffffffffu, G);
    const uint32_t pm = __ballot_sync(0xffffffffu, P);
    if (lane == 0) {
        sh.wg[warp] = (uint32_t)(carry_chain(gm, pm, false) >> 32) & 1;
        sh.wp[warp] = pm == 0xffffffffu;
    }
    __syncthreads();
    bool c = false;  // carry into this warp
    for (int w = 0; w < warp; ++w) c = sh.wg[w] || (sh.wp[w] && c);
    if (threadIdx.x == 0) {
        bool Gb = false, Pb = true;
        for (int w = 0; w < nwarps; ++w) {
            Gb = sh.wg[w] || (sh.wp[w] && Gb);
            Pb = Pb && sh.wp[w];
        }
        publish(Gb, Pb);
    }
    return (carry_chain(gm, pm, c) >> lane) & 1;
}

// Limbs of one thread: T_k = c_{2k} + c_{2k+1} * 2^32 folds the 32-bit
// digit convolution onto 64-bit limbs (T < 2^123); limb value
// v_k = lo64(T_k) + hi(T_{k-1}) with generate bit g_k.  Returns (G, P):
// the carry out with carry-in 0, and whether a carry-in passes through.
template <int L>
__device__ __forceinline__ void limbs_from_sums(const u128 (&T)[L], uint64_t prev_hi, uint64_t (&v)[L],
                                                uint32_t& gbits, bool& G, bool& P) {
    gbits = 0;
    bool c = false;
    P = true;
#pragma unroll
    for (int k = 0; k < L; ++k) {
        const uint64_t hi_prev = k == 0 ? prev_hi : (uint64_t)(T[k - 1] >> 64);
        const u128 s = (u128)(uint64_t)T[k] + hi_prev;
        v[k] = (uint64_t)s;
        const bool g = (uint64_t)(s >> 64) != 0;
        gbits |= (uint32_t)g << k;
        const bool all1 = v[k] == ~0ull;
        c = g || (all1 && c);
        P = P && all1;
    }
    G = c;
}

template <int L>
__device__ __forceinline__ void limbs_finish(int64_t m0, uint64_t lout, const uint64_t (&v)[L], uint32_t gbits,
                                             bool cin, uint64_t* out) {
    bool c = cin;
#pragma unroll
    for (int k = 0; k < L; ++k) {
        const uint64_t r = v[k] + (c ? 1u : 0u);
        const bool g = (gbits >> k) & 1;
        c = g || (v[k] == ~0ull && c);
        if (m0 + k < (int64_t)lout) out[m0 + k] = r;
    }
}

}  // namespace precgpu
