// ntt_kernels.cu -- sm_103a kernels of the large-operand multiply (NTT band).
//
// Replaces the hot loops of preclib's src/mul_ntt.cpp:
//   ntt_digits (331-342)           -> fused into the first column pass load
//   mont_in + zero padding (357-360) -> fused into the same load
//   ntt_forward (193-255)          -> column pass + row pass (four-step)
//   pointwise mont_mul (364-373)   -> fused into the row pass
//   ntt_inverse (257-329)          -> row pass + inverse column pass
//   ntt_crt2/3 + from_residues (405-487) -> CRT + decoupled look-back carry
//
// A transform of N = 2^k points (k >= 13) is split N = N1 * N2 (N1 = 2^k1
// column length, N2 = 2^k2 row length, k1 = k/2).  Index i = i1*N2 + i2:
//   fwd column pass : DIF over i1 for 8 adjacent columns i2 per CTA, then the
//                     four-step twiddle w_N^(i2*k1); output row slot s holds
//                     k1 = bitrev(s).  Digits are split from the limbs here.
//   row pass        : DIF over i2 of operand rows A and B, pointwise product,
//                     DIT back over the row, twiddle w_N^-(i2*k1).
//   inv column pass : DIT over the row slots -> natural coefficient order.
//   CRT + carry     : three residues -> 90-bit coefficient -> limbs, carries
//                     resolved by a single-pass decoupled look-back scan.
// Every HBM access moves whole 32-byte sectors (8 columns x 4 bytes) or
// 16-byte vectors; sub-transforms run in shared memory in radix-2^r register
// passes (r <= 4) over a padded layout (one spare word per 32).
#include <cuda_runtime.h>

#include "ntt_kernels.cuh"

namespace precgpu {

typedef unsigned __int128 u128;

__constant__ PrimeC c_prime[kPrimes];
__constant__ TableSet c_tab;

constexpr int kColGroup = 8;        // adjacent columns per column-pass CTA
constexpr int kColGroupWide = 4;    // used when the column length is 2^13
constexpr int kCarryThreads = 256;
constexpr int kCarryLimbs = 4;      // limbs per thread in the carry kernel
constexpr int kSpinLimit = 1 << 20; // bounded look-back wait
constexpr int kSmallMaxLog2 = 12;

__device__ __forceinline__ int padi(int i) { return i + (i >> 5); }

__host__ __device__ __forceinline__ int astride_for(int m) {
    int p = (1 << m) + ((1 << m) >> 5);
    p = (p + 7) & ~7;
    return p + 4;  // == 4 mod 8: columns 4 apart fall 16 banks apart
}

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(uint32_t* p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// ---------------------------------------------------------------------------
// shared-memory sub-transform engine
// ---------------------------------------------------------------------------

// One radix-2^RB pass of a forward (DIF) transform of length 2^m over bits
// [lo, lo+RB) of `narr` arrays laid out `astride` words apart; NA arrays
// share each twiddle load.
template <int RB, int NA>
__device__ __forceinline__ void dif_pass(uint32_t* s, int astride, int m, int lo, int narr,
                                         const uint2* __restrict__ tw, uint32_t p) {
    constexpr int R = 1 << RB;
    const int lg_items = m - RB;
    const int total = (narr / NA) << lg_items;
    const int lomask = (1 << lo) - 1;
    for (int w = threadIdx.x; w < total; w += blockDim.x) {
        const int u = w & ((1 << lg_items) - 1);
        const int ag = w >> lg_items;
        const int ulo = u & lomask;
        const int base = ((u >> lo) << (lo + RB)) | ulo;
        uint32_t x[NA][R];
#pragma unroll
        for (int a = 0; a < NA; ++a)
#pragma unroll
            for (int q = 0; q < R; ++q) x[a][q] = s[(ag * NA + a) * astride + padi(base + (q << lo))];
#pragma unroll
        for (int bb = RB - 1; bb >= 0; --bb) {
            const int h = 1 << bb;
#pragma unroll
            for (int q = 0; q < R; ++q) {
                if (q & h) continue;
                const int j = ulo | ((q & (h - 1)) << lo);
                const uint2 t = __ldg(&tw[(1 << (lo + bb)) + j]);
#pragma unroll
                for (int a = 0; a < NA; ++a) bfly_dif(x[a][q], x[a][q + h], t, p);
            }
        }
#pragma unroll
        for (int a = 0; a < NA; ++a)
#pragma unroll
            for (int q = 0; q < R; ++q) s[(ag * NA + a) * astride + padi(base + (q << lo))] = x[a][q];
    }
}

// One radix-2^RB pass of an inverse (DIT) transform over bits [lo, lo+RB).
template <int RB, int NA>
__device__ __forceinline__ void dit_pass(uint32_t* s, int astride, int m, int lo, int narr,
                                         const uint2* __restrict__ tw, uint32_t p) {
    constexpr int R = 1 << RB;
    const int lg_items = m - RB;
    const int total = (narr / NA) << lg_items;
    const int lomask = (1 << lo) - 1;
    for (int w = threadIdx.x; w < total; w += blockDim.x) {
        const int u = w & ((1 << lg_items) - 1);
        const int ag = w >> lg_items;
        const int ulo = u & lomask;
        const int base = ((u >> lo) << (lo + RB)) | ulo;
        uint32_t x[NA][R];
#pragma unroll
        for (int a = 0; a < NA; ++a)
#pragma unroll
            for (int q = 0; q < R; ++q) x[a][q] = s[(ag * NA + a) * astride + padi(base + (q << lo))];
#pragma unroll
        for (int bb = 0; bb < RB; ++bb) {
            const int h = 1 << bb;
#pragma unroll
            for (int q = 0; q < R; ++q) {
                if (q & h) continue;
                const int j = ulo | ((q & (h - 1)) << lo);
                const uint2 t = __ldg(&tw[(1 << (lo + bb)) + j]);
#pragma unroll
                for (int a = 0; a < NA; ++a) bfly_dit(x[a][q], x[a][q + h], t, p);
            }
        }
#pragma unroll
        for (int a = 0; a < NA; ++a)
#pragma unroll
            for (int q = 0; q < R; ++q) s[(ag * NA + a) * astride + padi(base + (q << lo))] = x[a][q];
    }
}

// Pass schedule of a length-2^m transform: ceil(m/4) passes, bits spread
// evenly, the larger passes at the low bits (top-down: [3,4,4] for m = 11).
__device__ __forceinline__ int pass_bits(int m, int t, int np) {
    const int base = m / np, extra = m % np;
    return base + (t >= np - extra ? 1 : 0);
}

template <int NA>
__device__ void dif_engine(uint32_t* s, int astride, int m, int narr, const uint2* __restrict__ tw,
                           uint32_t p) {
    const int np = (m + 3) >> 2;
    int hi = m;
    for (int t = 0; t < np; ++t) {
        const int rb = pass_bits(m, t, np);
        const int lo = hi - rb;
        switch (rb) {
            case 1: dif_pass<1, NA>(s, astride, m, lo, narr, tw, p); break;
            case 2: dif_pass<2, NA>(s, astride, m, lo, narr, tw, p); break;
            case 3: dif_pass<3, NA>(s, astride, m, lo, narr, tw, p); break;
            default: dif_pass<4, NA>(s, astride, m, lo, narr, tw, p); break;
        }
        __syncthreads();
        hi = lo;
    }
}

template <int NA>
__device__ void dit_engine(uint32_t* s, int astride, int m, int narr, const uint2* __restrict__ tw,
                           uint32_t p) {
    const int np = (m + 3) >> 2;
    int lo = 0;
    for (int t = np - 1; t >= 0; --t) {
        const int rb = pass_bits(m, t, np);
        switch (rb) {
            case 1: dit_pass<1, NA>(s, astride, m, lo, narr, tw, p); break;
            case 2: dit_pass<2, NA>(s, astride, m, lo, narr, tw, p); break;
            case 3: dit_pass<3, NA>(s, astride, m, lo, narr, tw, p); break;
            default: dit_pass<4, NA>(s, astride, m, lo, narr, tw, p); break;
        }
        __syncthreads();
        lo += rb;
    }
}

// w_N^e * 2^32 mod p (Montgomery form) for N = 2^k, e < N
__device__ __forceinline__ uint32_t fourstep_twiddle(int prime, uint32_t e, int k, const PrimeC& c) {
    const uint32_t E = e << (kMaxLog2N - k);
    const uint32_t hi = __ldg(&c_tab.twhi[prime][E >> kTwLevelBits]);
    const uint32_t lo = __ldg(&c_tab.twlo[prime][E & ((1u << kTwLevelBits) - 1)]);
    return mont_mul(hi, lo, c);
}

// ---------------------------------------------------------------------------
// CRT and carries
// ---------------------------------------------------------------------------

// Garner recombination of the three inverse-transform outputs y_j into the
// exact coefficient x < p1*p2*p3, with the transform's scale R*N^-1 folded
// into the constants (mul_ntt.cpp:405-424 recombine two or three primes
// the same way, without the folding).
__device__ __forceinline__ u128 crt3(uint32_t y1, uint32_t y2, uint32_t y3, const CrtConst& cc) {
    const uint32_t p1 = c_prime[0].p, p2 = c_prime[1].p, p3 = c_prime[2].p;
    const uint32_t v1 = shoup_mul(y1, cc.s1, p1);
    const uint32_t v2 = sub_mod(shoup_mul(y2, cc.k22, p2), shoup_mul(v1, cc.k21, p2), p2);
    uint32_t v3 = sub_mod(shoup_mul(y3, cc.k33, p3), shoup_mul(v1, cc.k31, p3), p3);
    v3 = sub_mod(v3, shoup_mul(v2, cc.k32, p3), p3);
    const uint64_t t = (uint64_t)v2 + (uint64_t)p2 * v3;
    return (u128)t * p1 + v1;
}

// Limb m of the product before carries: T_m = c_{2m} + c_{2m+1} * 2^32 (the
// 32-bit digit convolution folded onto 64-bit limbs); T_m < 2^123.
template <class Fetch>
__device__ __forceinline__ u128 limb_sum(int64_t m, const Fetch& fetch, const CrtConst& cc) {
    if (m < 0) return 0;
    uint32_t y0[3], y1[3];
    fetch(2 * m, y0);
    fetch(2 * m + 1, y1);
    const u128 c0 = crt3(y0[0], y0[1], y0[2], cc);
    const u128 c1 = crt3(y1[0], y1[1], y1[2], cc);
    return c0 + (c1 << 32);
}

// Per-thread part of the carry resolution: limbs m0 .. m0+L-1 get
// v_m = lo64(T_m) + hi(T_{m-1}) with generate bit g_m; returns the thread's
// (G, P): carry out with carry-in 0, and whether a carry-in passes through.
template <int L, class Fetch>
__device__ __forceinline__ void thread_limbs(int64_t m0, const Fetch& fetch, const CrtConst& cc,
                                             uint64_t (&v)[L], uint32_t& gbits, bool& G, bool& P) {
    u128 prev = limb_sum(m0 - 1, fetch, cc);
    gbits = 0;
    bool c = false;
    P = true;
#pragma unroll
    for (int k = 0; k < L; ++k) {
        const u128 cur = limb_sum(m0 + k, fetch, cc);
        const u128 s = (u128)(uint64_t)cur + (uint64_t)(prev >> 64);
        v[k] = (uint64_t)s;
        const bool g = (uint64_t)(s >> 64) != 0;
        gbits |= (uint32_t)g << k;
        const bool all1 = v[k] == ~0ull;
        c = g || (all1 && c);
        P = P && all1;
        prev = cur;
    }
    G = c;
}

// Applies the thread's carry-in and writes its limbs.
template <int L>
__device__ __forceinline__ void thread_finish(int64_t m0, uint64_t lout, const uint64_t (&v)[L],
                                              uint32_t gbits, bool cin, uint64_t* out) {
    bool c = cin;
#pragma unroll
    for (int k = 0; k < L; ++k) {
        const uint64_t r = v[k] + (c ? 1u : 0u);
        const bool g = (gbits >> k) & 1;
        c = g || (v[k] == ~0ull && c);
        if (m0 + k < (int64_t)lout) out[m0 + k] = r;
    }
}

// Carry-in of every lane from the lanes' (G, P) bits: the chain
// c_{t+1} = G_t | (P_t & c_t) is the carry chain of the sum A + B with
// A = G|P, B = G (G and P are disjoint), so the carry into lane t is bit t
// of (A + B + cin) ^ A ^ B.
__device__ __forceinline__ uint64_t carry_chain(uint32_t G, uint32_t P, bool cin) {
    const uint64_t A = (uint64_t)(G | P), B = (uint64_t)G;
    return (A + B + (cin ? 1u : 0u)) ^ A ^ B;  // bit t: carry into t; bit 32: carry out
}

// Block-wide carry resolution.  Each thread holds (G, P); returns the
// thread's carry-in given `block_cin_fn` which maps the block aggregate
// (Gb, Pb) to the block carry-in (called by thread 0 only).
struct BlockCarryShared {
    uint32_t wg[32], wp[32];
    uint32_t block_cin;
};

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
        const uint32_t bg = __ballot_sync(0xffffffffu, wG);
        const uint32_t bp = __ballot_sync(0xffffffffu, wP);
        // block aggregate over the real warps
        const uint32_t real = nwarps >= 32 ? 0xffffffffu : ((1u << nwarps) - 1);
        const uint64_t c0 = carry_chain(bg & real, bp & real, false);
        const bool Gb = (c0 >> nwarps) & 1;
        const bool Pb = (bp & real) == real;
        uint32_t bcin = 0;
        if (lane == 0) bcin = cin_fn(Gb, Pb) ? 1u : 0u;
        bcin = __shfl_sync(0xffffffffu, bcin, 0);
        const uint64_t cw = carry_chain(bg & real, bp & real, bcin != 0);
        if (lane < nwarps) sh.wg[lane] = (uint32_t)(cw >> lane) & 1;  // carry into warp `lane`
    }
    __syncthreads();
    const bool wcin = sh.wg[warp] != 0;
    const uint64_t cl = carry_chain(gm, pm, wcin);
    return (cl >> lane) & 1;
}

// ---------------------------------------------------------------------------
// multi-pass kernels
// ---------------------------------------------------------------------------

// forward column pass: limbs -> 32-bit digits -> mod p -> DIF over i1 ->
// four-step twiddle.  grid (N2/CG, 6): y = prime*2 + operand.
template <int CG>
__global__ void __launch_bounds__(256) k_fwd_cols(ProdArgs args) {
    extern __shared__ uint32_t sm[];
    const int prime = blockIdx.y >> 1, operand = blockIdx.y & 1;
    const PrimeC pc = c_prime[prime];
    const int k1 = args.k1, k2 = args.k2;
    const int N1 = 1 << k1;
    const uint64_t N2 = 1ull << k2, N = 1ull << args.k;
    const int astride = astride_for(k1);
    const int c0 = blockIdx.x * CG;
    constexpr int Q = CG / 4;  // 4-digit (2-limb) groups per row

    // the carry kernel's look-back words start at zero
    if (blockIdx.y == 0) {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= args.nblk; i += gridDim.x * blockDim.x)
            args.scratch[i] = 0;
    }

    const uint64_t* src = operand ? args.b : args.a;
    const uint64_t L = operand ? args.lb : args.la;
    for (int w = threadIdx.x; w < N1 * Q; w += blockDim.x) {
        const int r = w / Q, h = w % Q;
        const uint64_t limb = ((uint64_t)r * N2 + c0 + 4 * h) >> 1;
        const uint64_t l0 = limb < L ? __ldg(&src[limb]) : 0;
        const uint64_t l1 = limb + 1 < L ? __ldg(&src[limb + 1]) : 0;
        uint32_t* d = sm + (4 * h) * astride + padi(r);
        d[0] = reduce_u32((uint32_t)l0, pc);
        d[astride] = reduce_u32((uint32_t)(l0 >> 32), pc);
        d[2 * astride] = reduce_u32((uint32_t)l1, pc);
        d[3 * astride] = reduce_u32((uint32_t)(l1 >> 32), pc);
    }
    __syncthreads();
    dif_engine<2>(sm, astride, k1, CG, c_tab.tf[prime], pc.p);

    uint32_t* dst = args.work + (uint64_t)blockIdx.y * N;
    for (int w = threadIdx.x; w < N1 * Q; w += blockDim.x) {
        const int s = w / Q, h = w % Q;
        const uint32_t kk = __brev((uint32_t)s) >> (32 - k1);
        uint32_t o[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int c = 4 * h + t;
            const uint32_t i2 = (uint32_t)(c0 + c);
            const uint32_t tw = fourstep_twiddle(prime, i2 * kk, args.k, pc);
            o[t] = mont_mul(sm[c * astride + padi(s)], tw, pc);
        }
        *reinterpret_cast<uint4*>(dst + (uint64_t)s * N2 + c0 + 4 * h) = make_uint4(o[0], o[1], o[2], o[3]);
    }
}

// row pass: DIF of the A and B rows, pointwise product, DIT of the product
// row, inverse four-step twiddle.  grid (N1, 3).
__global__ void __launch_bounds__(256) k_rows(ProdArgs args) {
    extern __shared__ uint32_t sm[];
    const int prime = blockIdx.y;
    const PrimeC pc = c_prime[prime];
    const int k2 = args.k2, k1 = args.k1;
    const int N2 = 1 << k2;
    const uint64_t N = 1ull << args.k;
    const int astride = astride_for(k2);
    const int s = blockIdx.x;
    uint32_t* rowA = args.work + (uint64_t)(prime * 2) * N + (uint64_t)s * N2;
    const uint32_t* rowB = args.work + (uint64_t)(prime * 2 + 1) * N + (uint64_t)s * N2;

    for (int w = threadIdx.x; w < N2 / 4; w += blockDim.x) {
        const uint4 va = *reinterpret_cast<const uint4*>(rowA + 4 * w);
        const uint4 vb = *reinterpret_cast<const uint4*>(rowB + 4 * w);
        sm[padi(4 * w + 0)] = va.x;
        sm[padi(4 * w + 1)] = va.y;
        sm[padi(4 * w + 2)] = va.z;
        sm[padi(4 * w + 3)] = va.w;
        sm[astride + padi(4 * w + 0)] = vb.x;
        sm[astride + padi(4 * w + 1)] = vb.y;
        sm[astride + padi(4 * w + 2)] = vb.z;
        sm[astride + padi(4 * w + 3)] = vb.w;
    }
    __syncthreads();
    dif_engine<2>(sm, astride, k2, 2, c_tab.tf[prime], pc.p);
    for (int i = threadIdx.x; i < N2; i += blockDim.x)
        sm[padi(i)] = mont_mul(sm[padi(i)], sm[astride + padi(i)], pc);
    __syncthreads();
    dit_engine<1>(sm, astride, k2, 1, c_tab.ti[prime], pc.p);

    const uint32_t kk = __brev((uint32_t)s) >> (32 - k1);
    const uint32_t Nmask = (uint32_t)(N - 1);
    for (int w = threadIdx.x; w < N2 / 4; w += blockDim.x) {
        uint32_t o[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const uint32_t i2 = 4 * w + t;
            const uint32_t e = (0u - i2 * kk) & Nmask;
            o[t] = mont_mul(sm[padi(i2)], fourstep_twiddle(prime, e, args.k, pc), pc);
        }
        *reinterpret_cast<uint4*>(rowA + 4 * w) = make_uint4(o[0], o[1], o[2], o[3]);
    }
}

// inverse column pass: DIT over the row slots of CG adjacent columns; the
// output is the natural coefficient order.  grid (N2/CG, 3).
template <int CG>
__global__ void __launch_bounds__(256) k_inv_cols(ProdArgs args) {
    extern __shared__ uint32_t sm[];
    const int prime = blockIdx.y;
    const PrimeC pc = c_prime[prime];
    const int k1 = args.k1;
    const int N1 = 1 << k1;
    const uint64_t N2 = 1ull << args.k2, N = 1ull << args.k;
    const int astride = astride_for(k1);
    const int c0 = blockIdx.x * CG;
    constexpr int Q = CG / 4;
    uint32_t* base = args.work + (uint64_t)(prime * 2) * N;

    for (int w = threadIdx.x; w < N1 * Q; w += blockDim.x) {
        const int s = w / Q, h = w % Q;
        const uint4 v = *reinterpret_cast<const uint4*>(base + (uint64_t)s * N2 + c0 + 4 * h);
        uint32_t* d = sm + (4 * h) * astride + padi(s);
        d[0] = v.x;
        d[astride] = v.y;
        d[2 * astride] = v.z;
        d[3 * astride] = v.w;
    }
    __syncthreads();
    dit_engine<2>(sm, astride, k1, CG, c_tab.ti[prime], pc.p);
    for (int w = threadIdx.x; w < N1 * Q; w += blockDim.x) {
        const int r = w / Q, h = w % Q;
        const uint32_t* d = sm + (4 * h) * astride + padi(r);
        *reinterpret_cast<uint4*>(base + (uint64_t)r * N2 + c0 + 4 * h) =
            make_uint4(d[0], d[astride], d[2 * astride], d[3 * astride]);
    }
}

// CRT + carry: one pass over the natural-order residues.  Block order is
// taken from a ticket counter so that a block only waits on blocks that
// already run; every wait is bounded.
__global__ void __launch_bounds__(kCarryThreads) k_crt_carry(ProdArgs args) {
    __shared__ BlockCarryShared sh;
    __shared__ uint32_t s_ticket;
    if (threadIdx.x == 0) s_ticket = atomicAdd(&args.scratch[0], 1u);
    __syncthreads();
    const uint32_t bid = s_ticket;
    const uint64_t N = 1ull << args.k;
    const uint32_t* r0 = args.work;
    const uint32_t* r1 = args.work + 2 * N;
    const uint32_t* r2 = args.work + 4 * N;
    auto fetch = [&](int64_t i, uint32_t (&y)[3]) {
        if ((uint64_t)i < N) {
            y[0] = r0[i];
            y[1] = r1[i];
            y[2] = r2[i];
        } else {
            y[0] = y[1] = y[2] = 0;
        }
    };
    const int64_t m0 = (int64_t)bid * (kCarryThreads * kCarryLimbs) + threadIdx.x * kCarryLimbs;
    uint64_t v[kCarryLimbs];
    uint32_t gbits;
    bool G, P;
    thread_limbs<kCarryLimbs>(m0, fetch, args.crt, v, gbits, G, P);

    uint32_t* status = args.scratch + 1;
    auto cin_fn = [&](bool Gb, bool Pb) -> bool {
        // status word: bit0 aggregate ready, bit1 inclusive ready,
        // bit2 G (or inclusive carry out), bit3 P
        if (bid == 0) {
            st_release(&status[0], 2u | (Gb ? 4u : 0u));
            return false;
        }
        if (!Pb) st_release(&status[bid], 2u | (Gb ? 4u : 0u));  // carry out known already
        else st_release(&status[bid], 1u | (Gb ? 4u : 0u) | 8u);
        bool accG = false, accP = true;
        bool cin = false;
        for (int64_t j = (int64_t)bid - 1; j >= 0; --j) {
            uint32_t st = 0;
            int spins = 0;
            while (((st = ld_acquire(&status[j])) & 3u) == 0) {
                if (++spins > kSpinLimit) {
                    atomicOr(args.err, kDevErrTimeout);
                    st = 2u;  // give up: treat as carry 0, error reported
                    break;
                }
                __nanosleep(100);
            }
            const bool g = (st & 4u) != 0;
            if (st & 2u) {
                cin = accG || (accP && g);
                break;
            }
            const bool p = (st & 8u) != 0;
            accG = accG || (accP && g);
            accP = accP && p;
        }
        if (Pb) st_release(&status[bid], 2u | ((Gb || cin) ? 4u : 0u));
        return cin;
    };
    const bool cin = block_carry(G, P, sh, cin_fn);
    thread_finish<kCarryLimbs>(m0, args.lout, v, gbits, cin, args.out);
    // the very last block's carry out must be zero
    if (bid + 1 == gridDim.x && threadIdx.x == blockDim.x - 1) {
        bool c = cin;
        for (int k = 0; k < kCarryLimbs; ++k) c = ((gbits >> k) & 1) || (v[k] == ~0ull && c);
        if (c) atomicOr(args.err, kDevErrCarry);
    }
}

// ---------------------------------------------------------------------------
// single-CTA path: whole product in shared memory, N <= 2^12
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(256) k_small(const SmallDesc* __restrict__ descs, SmallDesc single) {
    extern __shared__ uint32_t sm[];
    __shared__ BlockCarryShared sh;
    const SmallDesc d = descs ? descs[blockIdx.x] : single;
    const int k = d.k;
    const int N = 1 << k;
    const int astride = astride_for(k);
    uint32_t* A = sm;
    uint32_t* B = sm + astride;
    uint32_t* res = sm + 2 * astride;  // 3 arrays of residues
    for (int prime = 0; prime < kPrimes; ++prime) {
        const PrimeC pc = c_prime[prime];
        for (int i = threadIdx.x; i < N; i += blockDim.x) {
            const uint64_t limb = (uint64_t)(i >> 1);
            const int sh32 = (i & 1) * 32;
            const uint32_t xa = limb < d.la ? (uint32_t)(__ldg(&d.a[limb]) >> sh32) : 0u;
            const uint32_t xb = limb < d.lb ? (uint32_t)(__ldg(&d.b[limb]) >> sh32) : 0u;
            A[padi(i)] = reduce_u32(xa, pc);
            B[padi(i)] = reduce_u32(xb, pc);
        }
        __syncthreads();
        dif_engine<2>(A, astride, k, 2, c_tab.tf[prime], pc.p);
        for (int i = threadIdx.x; i < N; i += blockDim.x) A[padi(i)] = mont_mul(A[padi(i)], B[padi(i)], pc);
        __syncthreads();
        dit_engine<1>(A, astride, k, 1, c_tab.ti[prime], pc.p);
        for (int i = threadIdx.x; i < N; i += blockDim.x) res[prime * astride + padi(i)] = A[padi(i)];
        __syncthreads();
    }
    auto fetch = [&](int64_t i, uint32_t (&y)[3]) {
        if (i < N) {
            const int pi = padi((int)i);
            y[0] = res[pi];
            y[1] = res[astride + pi];
            y[2] = res[2 * astride + pi];
        } else {
            y[0] = y[1] = y[2] = 0;
        }
    };
    // lout <= N/2 + 1 limbs; each thread takes a run of L limbs per round
    constexpr int L = 8;
    bool carry = false;  // carry into the current round
    for (int64_t r0 = 0; r0 < (int64_t)d.lout; r0 += (int64_t)blockDim.x * L) {
        const int64_t m0 = r0 + threadIdx.x * L;
        uint64_t v[L];
        uint32_t gbits;
        bool G, P;
        thread_limbs<L>(m0, fetch, d.crt, v, gbits, G, P);
        bool next = false;
        const bool cin = block_carry(G, P, sh, [&](bool Gb, bool Pb) {
            next = Gb || (Pb && carry);
            sh.block_cin = next ? 1u : 0u;
            return carry;
        });
        thread_finish<L>(m0, d.lout, v, gbits, cin, d.out);
        __syncthreads();
        carry = sh.block_cin != 0;
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

void ntt_set_tables(const PrimeC* primes, const TableSet& tabs) {
    cudaMemcpyToSymbol(c_prime, primes, sizeof(PrimeC) * kPrimes);
    cudaMemcpyToSymbol(c_tab, &tabs, sizeof(TableSet));
}

int ntt_small_max_log2() { return kSmallMaxLog2; }
int ntt_carry_block_limbs() { return kCarryThreads * kCarryLimbs; }

size_t ntt_small_smem_bytes(int k) { return (size_t)5 * astride_for(k) * sizeof(uint32_t); }

static size_t cols_smem(int k1) {
    const int cg = k1 >= 13 ? kColGroupWide : kColGroup;
    return (size_t)cg * astride_for(k1) * sizeof(uint32_t);
}

int ntt_configure_kernels() {
    cudaError_t e;
    const int big = 200 * 1024;
    if ((e = cudaFuncSetAttribute(k_fwd_cols<kColGroup>, cudaFuncAttributeMaxDynamicSharedMemorySize, big))) return e;
    if ((e = cudaFuncSetAttribute(k_fwd_cols<kColGroupWide>, cudaFuncAttributeMaxDynamicSharedMemorySize, big))) return e;
    if ((e = cudaFuncSetAttribute(k_inv_cols<kColGroup>, cudaFuncAttributeMaxDynamicSharedMemorySize, big))) return e;
    if ((e = cudaFuncSetAttribute(k_inv_cols<kColGroupWide>, cudaFuncAttributeMaxDynamicSharedMemorySize, big))) return e;
    if ((e = cudaFuncSetAttribute(k_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, big))) return e;
    if ((e = cudaFuncSetAttribute(k_small, cudaFuncAttributeMaxDynamicSharedMemorySize, big))) return e;
    return 0;
}

void ntt_launch_small(const SmallDesc* d_descs, const SmallDesc* single, int count, int k, cudaStream_t st) {
    SmallDesc one{};
    if (single) one = *single;
    k_small<<<count, 256, ntt_small_smem_bytes(k), st>>>(d_descs, one);
}

void ntt_launch_4step(const ProdArgs& args, cudaStream_t st) {
    const int k1 = args.k1, k2 = args.k2;
    const int cg = k1 >= 13 ? kColGroupWide : kColGroup;
    const size_t csm = cols_smem(k1);
    const dim3 gcol((1u << k2) / cg, 2 * kPrimes);
    if (cg == kColGroup) k_fwd_cols<kColGroup><<<gcol, 256, csm, st>>>(args);
    else k_fwd_cols<kColGroupWide><<<gcol, 256, csm, st>>>(args);
    const int row_threads = (1 << k2) / 16 >= 256 ? 256 : ((1 << k2) / 16 < 32 ? 32 : (1 << k2) / 16);
    k_rows<<<dim3(1u << k1, kPrimes), row_threads, (size_t)2 * astride_for(k2) * sizeof(uint32_t), st>>>(args);
    const dim3 gicol((1u << k2) / cg, kPrimes);
    if (cg == kColGroup) k_inv_cols<kColGroup><<<gicol, 256, csm, st>>>(args);
    else k_inv_cols<kColGroupWide><<<gicol, 256, csm, st>>>(args);
    k_crt_carry<<<args.nblk, kCarryThreads, 0, st>>>(args);
}

}  // namespace precgpu
