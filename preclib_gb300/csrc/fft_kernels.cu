// fft_kernels.cu -- FP64 FFT band (193 .. 6144 limbs) of the multiply.
//
// Replaces preclib's mul_fft (src/mul_fft.cpp:340-394) with the same method
// -- both operands packed as the real and imaginary parts of one complex
// FP64 FFT (fft_load_digits, 234-246), the two spectra separated and
// multiplied (fft_pair_convolution, 248-305), one inverse FFT, rounding to
// the nearest integer (307-309, 364-376) and a signed carry back to limbs
// (fft_from_digits, 311-338) -- laid out for many SMs:
//
//  digits   balanced b-bit digits (|d| <= 2^(b-1)), b chosen per transform
//           length from a worst-case error bound (host side); every digit
//           is computed on its own: d_i = raw_i - 2^b t_i + t_{i-1} with
//           t_j = [raw_j >= 2^(b-1)], so no carry chain is needed.
//  twiddles one table of e^(2 pi i e / 2^16), e < 2^15, from sincospi()
//           (the reference builds per-stage tables by a recurrence,
//           mul_fft.cpp:57-76).
//  four-step N = N1 * N2:
//    k_fft_fwd_cols  digits -> column DIF over i1 -> twiddle w^-(i2 k1)
//    k_fft_rows      rows k1 and N1-k1 together: row DIF, separation and
//                    product (P_-k = conj P_k), row DIT, twiddle w^(i2 k1)
//    k_fft_inv_cols  column DIT -> x/N -> nearest integer, max distance
//    k_fft_carry     limbs from the signed coefficients (blocks, then the
//                    last block joins their carries); writes nothing when
//                    the max distance exceeds 0.25.
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "fft_kernels.cuh"
#include "ntt_kernels.cuh"

namespace precgpu {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 conj2(double2 a) { return make_double2(a.x, -a.y); }

// w_N^e = e^(2 pi i e / N) for 0 <= e < N, N = 2^k <= 2^16
__device__ __forceinline__ double2 root(const double2* __restrict__ tw, uint32_t e, int k) {
    const uint32_t half = 1u << (k - 1);
    const double2 w = __ldg(&tw[(e & (half - 1)) << (kFftMaxLog2 - k)]);
    return (e & half) ? make_double2(-w.x, -w.y) : w;
}

__device__ __forceinline__ int fpad(int i) { return i + (i >> 4); }  // 16-byte elements, 1 spare per 16

// raw b-bit digit i of an n-limb operand (zero past its top)
__device__ __forceinline__ uint32_t raw_digit(const uint64_t* __restrict__ a, uint64_t n, int b, uint64_t i) {
    const uint64_t bit = (uint64_t)b * i;
    const uint64_t limb = bit >> 6;
    const int sh = (int)(bit & 63);
    uint64_t v = limb < n ? __ldg(&a[limb]) >> sh : 0;
    if (sh + b > 64 && limb + 1 < n) v |= __ldg(&a[limb + 1]) << (64 - sh);
    return (uint32_t)(v & ((1ull << b) - 1));
}

// balanced digit i (|d| <= 2^(b-1)) of an operand with `nd` digits
__device__ __forceinline__ double bal_digit(const uint64_t* __restrict__ a, uint64_t n, int b, uint64_t i, uint64_t nd) {
    if (i >= nd) return 0.0;
    const uint32_t half = 1u << (b - 1);
    const uint32_t r = raw_digit(a, n, b, i);
    const int t_in = i > 0 && raw_digit(a, n, b, i - 1) >= half ? 1 : 0;
    const int t_out = r >= half ? 1 : 0;
    return (double)((int64_t)r - ((int64_t)t_out << b) + t_in);
}

// One register pass: stages over bits lo .. lo+RB-1 of `narr` arrays of 2^m
// points in shared memory (array stride `as`, element i at fpad(i)); item u
// holds elements base + (q << lo), q < 2^RB.  DIF (forward, sign -1,
// natural -> bit-reversed) runs the pass's stages from its top bit down, DIT
// (inverse, sign +1, bit-reversed -> natural) from its bottom bit up; the
// stage at bit b pairs i and i + 2^b with twiddle w_(2^(b+1))^(i mod 2^b).
template <bool DIT, int RB>
__device__ __forceinline__ void fft_pass(double2* s, int as, int narr, int m, int lo, const double2* __restrict__ tw) {
    const int lgper = m - RB;
    const uint32_t lomask = (1u << lo) - 1;
    for (int w = threadIdx.x; w < (narr << lgper); w += blockDim.x) {
        const int a = w >> lgper;
        const uint32_t u = w & ((1u << lgper) - 1);
        const uint32_t base = ((u >> lo) << (lo + RB)) | (u & lomask);
        const uint32_t ulo = u & lomask;
        double2* row = s + a * as;
        double2 x[1 << RB];
#pragma unroll
        for (int q = 0; q < (1 << RB); ++q) x[q] = row[fpad((int)(base + ((uint32_t)q << lo)))];
#pragma unroll
        for (int t = 0; t < RB; ++t) {
            const int bb = DIT ? t : RB - 1 - t;
            const int h = 1 << bb;
#pragma unroll
            for (int q = 0; q < (1 << RB); ++q) {
                if (q & h) continue;
                const uint32_t j = ulo | ((uint32_t)(q & (h - 1)) << lo);
                const double2 X = x[q], Y = x[q + h];
                double2 r = make_double2(1.0, 0.0);
                if (j) {
                    r = root(tw, j << (m - 1 - (lo + bb)), m);
                    if (!DIT) r.y = -r.y;
                }
                if (DIT) {
                    const double2 tt = j ? cmul(Y, r) : Y;
                    x[q] = cadd(X, tt);
                    x[q + h] = csub(X, tt);
                } else {
                    x[q] = cadd(X, Y);
                    const double2 d = csub(X, Y);
                    x[q + h] = j ? cmul(d, r) : d;
                }
            }
        }
#pragma unroll
        for (int q = 0; q < (1 << RB); ++q) row[fpad((int)(base + ((uint32_t)q << lo)))] = x[q];
    }
}

template <bool DIT>
__device__ __forceinline__ void fft_pass_rb(int rb, double2* s, int as, int narr, int m, int lo,
                                            const double2* __restrict__ tw) {
    if (rb == 3) fft_pass<DIT, 3>(s, as, narr, m, lo, tw);
    else if (rb == 2) fft_pass<DIT, 2>(s, as, narr, m, lo, tw);
    else fft_pass<DIT, 1>(s, as, narr, m, lo, tw);
}

// the whole 2^m-point transform of `narr` arrays in passes of up to radix
// 2^PREC_FFT_MAX_RB, one barrier per pass; DIF from the top bits, DIT from the
// bottom bits.  Radix 2 is the default: at 2^15 points radix-4 and radix-8
// passes measured 10% and 30% slower (more registers per thread, the same
// FP64 work, and these kernels are bound by the FP64 pipe and by latency).
#ifndef PREC_FFT_MAX_RB
#define PREC_FFT_MAX_RB 1
#endif
constexpr int kFftMaxRb = PREC_FFT_MAX_RB;

template <bool DIT>
__device__ void fft_stages(double2* s, int as, int narr, int m, const double2* __restrict__ tw) {
    if (!DIT) {
        for (int top = m; top > 0;) {
            const int rb = top < kFftMaxRb ? top : kFftMaxRb;
            fft_pass_rb<false>(rb, s, as, narr, m, top - rb, tw);
            __syncthreads();
            top -= rb;
        }
    } else {
        for (int lo = 0; lo < m;) {
            const int rb = m - lo < kFftMaxRb ? m - lo : kFftMaxRb;
            fft_pass_rb<true>(rb, s, as, narr, m, lo, tw);
            __syncthreads();
            lo += rb;
        }
    }
}

__device__ __forceinline__ uint32_t bitrev(uint32_t x, int bits) { return bits ? __brev(x) >> (32 - bits) : 0u; }

// forward column pass: grid N2/C CTAs, C adjacent columns each
template <int C>
__global__ void __launch_bounds__(256) k_fft_fwd_cols(FftArgs f, FftArgs* publish) {
    extern __shared__ double2 fsm[];
    // the product's arguments for the three kernels after this one
    if (blockIdx.x == 0 && threadIdx.x == 0) *publish = f;
    const int N1 = 1 << f.k1;
    const uint32_t N2 = 1u << f.k2;
    const int as = fpad(N1) + 1;
    const uint32_t c0 = blockIdx.x * C;
    // the product's max distance starts at 0 (the previous product's readers
    // are earlier in stream order)
    if (blockIdx.x == 0 && threadIdx.x == 0) *f.maxdist = 0.0;
    for (int w = threadIdx.x; w < C * N1; w += blockDim.x) {
        const int col = w % C, i1 = w / C;
        const uint64_t i = (uint64_t)i1 * N2 + c0 + col;
        fsm[col * as + fpad(i1)] = make_double2(bal_digit(f.a, f.la, f.b, i, f.da), bal_digit(f.bp, f.lb, f.b, i, f.db));
    }
    __syncthreads();
    fft_stages<false>(fsm, as, C, f.k1, f.tw);
    for (int w = threadIdx.x; w < C * N1; w += blockDim.x) {
        const int col = w % C, s = w / C;
        const uint32_t k1 = bitrev((uint32_t)s, f.k1);
        const uint32_t i2 = c0 + col;
        double2 r = root(f.tw, (i2 * k1) & ((1u << f.k) - 1), f.k);
        r.y = -r.y;
        f.work[(uint64_t)s * N2 + i2] = cmul(fsm[col * as + fpad(s)], r);
    }
}

// row pass: CTA r handles frequency rows k1 = r and N1 - r (one row when
// they coincide); grid N1/2 + 1
__global__ void __launch_bounds__(256) k_fft_rows(const FftArgs* __restrict__ fa) {
    const FftArgs f = *fa;
    extern __shared__ double2 fsm[];
    const int N1 = 1 << f.k1, N2 = 1 << f.k2;
    const int as = fpad(N2) + 1;
    const uint32_t ka = blockIdx.x, kb = (N1 - blockIdx.x) & (N1 - 1);
    const int nrow = ka == kb ? 1 : 2;
    const uint32_t sa = bitrev(ka, f.k1), sb = bitrev(kb, f.k1);
    double2* rowp[2] = {f.work + (uint64_t)sa * N2, f.work + (uint64_t)sb * N2};
    for (int w = threadIdx.x; w < nrow * N2; w += blockDim.x) {
        const int r = w / N2, t = w % N2;
        fsm[r * as + fpad(t)] = rowp[r][t];
    }
    __syncthreads();
    fft_stages<false>(fsm, as, nrow, f.k2, f.tw);
    // separation of the packed spectra and product; slot t holds k2 = bitrev(t)
    double2 prod[8];  // at most 2 * N2 / blockDim = 8 elements per thread
    int cnt = 0;
    for (int w = threadIdx.x; w < nrow * N2; w += blockDim.x, ++cnt) {
        const int r = w / N2, t = w % N2;
        const uint32_t k1 = r ? kb : ka;
        const uint32_t k2 = bitrev((uint32_t)t, f.k2);
        const uint32_t pk2 = (N2 - k2 - (k1 != 0 ? 1u : 0u)) & (N2 - 1);
        const int pr = (nrow == 1) ? 0 : 1 - r;  // the partner row
        const double2 F = fsm[r * as + fpad(t)];
        const double2 G = conj2(fsm[pr * as + fpad(bitrev(pk2, f.k2))]);  // conj(F_-k)
        const double2 A = make_double2(0.5 * (F.x + G.x), 0.5 * (F.y + G.y));
        // B = (F - conj F_-k) / 2i
        const double2 D = csub(F, G);
        const double2 B = make_double2(0.5 * D.y, -0.5 * D.x);
        prod[cnt] = cmul(A, B);
    }
    __syncthreads();
    cnt = 0;
    for (int w = threadIdx.x; w < nrow * N2; w += blockDim.x, ++cnt) {
        const int r = w / N2, t = w % N2;
        fsm[r * as + fpad(t)] = prod[cnt];
    }
    __syncthreads();
    fft_stages<true>(fsm, as, nrow, f.k2, f.tw);
    for (int w = threadIdx.x; w < nrow * N2; w += blockDim.x) {
        const int r = w / N2, i2 = w % N2;
        const uint32_t k1 = r ? kb : ka;
        const double2 rt = root(f.tw, (i2 * k1) & ((1u << f.k) - 1), f.k);
        rowp[r][i2] = cmul(fsm[r * as + fpad(i2)], rt);
    }
}

// inverse column pass, scaling, rounding; grid N2/C
template <int C>
__global__ void __launch_bounds__(256) k_fft_inv_cols(const FftArgs* __restrict__ fa) {
    const FftArgs f = *fa;
    extern __shared__ double2 fsm[];
    __shared__ double s_max[8];
    const int N1 = 1 << f.k1;
    const uint32_t N2 = 1u << f.k2;
    const int as = fpad(N1) + 1;
    const uint32_t c0 = blockIdx.x * C;
    for (int w = threadIdx.x; w < C * N1; w += blockDim.x) {
        const int col = w % C, s = w / C;
        fsm[col * as + fpad(s)] = f.work[(uint64_t)s * N2 + c0 + col];
    }
    __syncthreads();
    // block 0 alone reads the first element; the carry kernel's counter
    // lives there and starts at 0
    if (blockIdx.x == 0 && threadIdx.x == 0) *reinterpret_cast<unsigned long long*>(f.work) = 0ull;
    fft_stages<true>(fsm, as, C, f.k1, f.tw);
    const double inv_n = 1.0 / (double)(1u << f.k);
    double dmax = 0.0;
    for (int w = threadIdx.x; w < C * N1; w += blockDim.x) {
        const int col = w % C, i1 = w / C;
        const double v = fsm[col * as + fpad(i1)].x * inv_n;
        const double r = rint(v);
        double d = fabs(v - r);
        if (!isfinite(v)) d = INFINITY;
        dmax = fmax(dmax, d);
        f.coef[(uint64_t)i1 * N2 + c0 + col] = (long long)r;
    }
    for (int o = 16; o > 0; o >>= 1) dmax = fmax(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
    if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = dmax;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < (int)(blockDim.x >> 5); ++i) dmax = fmax(dmax, s_max[i]);
        // non-negative doubles order like their bit patterns
        atomicMax(reinterpret_cast<unsigned long long*>(f.maxdist), (unsigned long long)__double_as_longlong(dmax));
    }
}

// signed carry: one CTA of 1024 threads, limbs of the product from the
// rounded coefficients c_i (value sum c_i 2^(b i)).  A limb's sum
// S_m = sum of c_i 2^(b i - 64 m) over the coefficients starting in it is a
// signed 128-bit value; v_m = lo64(S_m) + hi(S_{m-1}) = u_m + g_m 2^64 with
// g_m in {-1, 0, 1}, and the carry chain c_{m+1} = g_m + floor((u_m + c_m)
// / 2^64) stays in {-1, 0, 1}.  Each thread composes the chain of its limbs
// into a map {-1,0,1} -> {-1,0,1}; the block scans the maps.
typedef __int128 i128;

__device__ __forceinline__ i128 limb_sum_s(const long long* __restrict__ c, uint64_t ncoef, int b, int64_t m) {
    if (m < 0) return 0;
    const uint64_t lo_bit = (uint64_t)m * 64;
    uint64_t i = (lo_bit + b - 1) / b;
    i128 s = 0;
    for (; i < ncoef && (uint64_t)b * i < lo_bit + 64; ++i)
        s += (i128)((unsigned __int128)(i128)c[i] << ((uint64_t)b * i - lo_bit));  // two's complement shift
    return s;
}

__device__ __forceinline__ int chain_step(uint64_t u, int g, int cin, uint64_t* out_limb) {
    const uint64_t r = u + (uint64_t)(int64_t)cin;
    if (out_limb) *out_limb = r;
    int fl = 0;
    if (cin < 0 && u == 0) fl = -1;
    if (cin > 0 && u == ~0ull) fl = 1;
    return g + fl;
}

// Carry maps {-1,0,1} -> {-1,0,1} packed as three 2-bit fields (value + 1).
constexpr uint32_t kMapIdentity = 0u | (1u << 2) | (2u << 4);
__device__ __forceinline__ int map_apply(uint32_t m, int x) { return (int)((m >> (2 * (x + 1))) & 3u) - 1; }
// g after f
__device__ __forceinline__ uint32_t map_compose(uint32_t g, uint32_t f) {
    uint32_t r = 0;
#pragma unroll
    for (int x = -1; x <= 1; ++x) r |= (uint32_t)(map_apply(g, map_apply(f, x)) + 1) << (2 * (x + 1));
    return r;
}

#ifndef PREC_FFT_CARRY_THREADS
#define PREC_FFT_CARRY_THREADS 256
#endif
#ifndef PREC_FFT_CARRY_LIMBS
#define PREC_FFT_CARRY_LIMBS 2
#endif
constexpr int kFftCarryThreads = PREC_FFT_CARRY_THREADS;
constexpr int kFftCarryLimbs = PREC_FFT_CARRY_LIMBS;  // limbs per thread
constexpr int kFftCarryBlockLimbs = kFftCarryThreads * kFftCarryLimbs;

// Phase 1 (every block): the block's limbs from the signed coefficient sums,
// the carry chain inside the block resolved with a block carry-in of 0
// (maps composed by warp shuffles and a block scan), limbs written -- below
// La+Lb to the output, above it to scratch -- and the block's composed map
// published.  Phase 2 (the last block to finish, fence + atomic counter):
// loads the block maps into shared memory (one load per thread, all in
// flight at once), composes them in order, adds each nonzero block carry-in
// into its block (+1 ripples through all-ones limbs, -1 through zero limbs;
// rare), and checks that every limb past La+Lb and the final carry are zero.
// scratch (the transform buffer, free by now): [0] counter, [1 .. nblk]
// block maps, then the limbs from La+Lb up.
__global__ void __launch_bounds__(kFftCarryThreads) k_fft_carry(const FftArgs* __restrict__ fa) {
    const FftArgs f = *fa;
    __shared__ uint32_t s_wmap[kFftCarryThreads / 32];
    __shared__ uint32_t s_bmap[kFftCarryThreads];
    __shared__ uint32_t s_last;
    const double dist = *f.maxdist;
    if (!(dist <= 0.25)) {  // also NaN / inf: nothing is written
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(f.err, kDevErrFftRound);
        return;
    }
    // Balanced digits can place signed contributions past the product's
    // La+Lb limbs (they cancel a borrow that runs up to them), so the chain
    // covers every limb a coefficient reaches; those limbs must end as 0.
    const int64_t Lout = (int64_t)f.lout;
    const int64_t Lcoef = (int64_t)(((uint64_t)f.b * f.ncoef + 63) / 64) + 2;
    const int64_t L = Lcoef > Lout ? Lcoef : Lout;
    const int nblk = (int)((L + kFftCarryBlockLimbs - 1) / kFftCarryBlockLimbs);
    uint64_t* scr = reinterpret_cast<uint64_t*>(f.work);
    uint32_t* counter = reinterpret_cast<uint32_t*>(scr);
    uint64_t* bmap = scr + 1;
    uint64_t* high = scr + 1 + nblk;  // limbs Lout .. L-1
    auto limb_ref = [&](int64_t m) -> uint64_t& { return m < Lout ? f.out[m] : high[m - Lout]; };

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // a graph launch uses the largest grid of the transform length: blocks
    // past this product's limbs only take part in the count below
    const bool idle = (int)blockIdx.x >= nblk;
    const int64_t m0 = (int64_t)blockIdx.x * kFftCarryBlockLimbs + (int64_t)threadIdx.x * kFftCarryLimbs;
    uint64_t u[kFftCarryLimbs];
    int g[kFftCarryLimbs];
    if (!idle) {
        i128 prev = limb_sum_s(f.coef, f.ncoef, f.b, m0 - 1);
#pragma unroll
        for (int k = 0; k < kFftCarryLimbs; ++k) {
            const i128 cur = m0 + k < L ? limb_sum_s(f.coef, f.ncoef, f.b, m0 + k) : (i128)0;
            const i128 v = (i128)(uint64_t)cur + (prev >> 64);
            u[k] = (uint64_t)v;
            g[k] = (int)(v >> 64);
            prev = cur;
        }
    }
    // this thread's chain as a map of its carry-in
    uint32_t tmap = 0;
#pragma unroll
    for (int x = -1; x <= 1; ++x) {
        int c = x;
#pragma unroll
        for (int k = 0; k < kFftCarryLimbs; ++k)
            if (m0 + k < L) c = chain_step(u[k], g[k], c, nullptr);
        tmap |= (uint32_t)((c < -1 ? -1 : (c > 1 ? 1 : c)) + 1) << (2 * (x + 1));
    }
    // inclusive scan of the maps over the warp, then over the warps
    uint32_t inc = tmap;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t o = __shfl_up_sync(0xffffffffu, inc, d);
        if (lane >= d) inc = map_compose(inc, o);
    }
    if (lane == 31) s_wmap[warp] = inc;
    __syncthreads();
    uint32_t below = kMapIdentity;  // warps before this one
    for (int w = 0; w < warp; ++w) below = map_compose(s_wmap[w], below);
    uint32_t excl = __shfl_up_sync(0xffffffffu, inc, 1);
    if (lane == 0) excl = kMapIdentity;
    const int cin = map_apply(map_compose(excl, below), 0);
    {
        int c = cin;
#pragma unroll
        for (int k = 0; k < kFftCarryLimbs; ++k) {
            if (m0 + k >= L) break;
            uint64_t limb;
            c = chain_step(u[k], g[k], c, &limb);
            limb_ref(m0 + k) = limb;
        }
    }
    if (threadIdx.x == 0 && !idle) {
        uint32_t bm = kMapIdentity;
        for (int w = 0; w < kFftCarryThreads / 32; ++w) bm = map_compose(s_wmap[w], bm);
        bmap[blockIdx.x] = bm;
    }
    // ---- phase 2: the last block resolves the carries between blocks
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(counter, 1u) == (uint32_t)gridDim.x - 1 ? 1u : 0u;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    // (one L2 round trip per block map, in the serial loop below, made this
    // kernel 14 us long at 3000 x 3000 limbs)
    const bool staged = nblk <= kFftCarryThreads;
    if (staged && (int)threadIdx.x < nblk) s_bmap[threadIdx.x] = (uint32_t)__ldcg(&bmap[threadIdx.x]);
    __syncthreads();
    if (threadIdx.x == 0) {
        int c = 0;
        for (int bk = 0; bk < nblk; ++bk) {
            if (c != 0) {
                const int64_t e = (int64_t)(bk + 1) * kFftCarryBlockLimbs < L ? (int64_t)(bk + 1) * kFftCarryBlockLimbs : L;
                for (int64_t m = (int64_t)bk * kFftCarryBlockLimbs; m < e; ++m) {
                    uint64_t& x = limb_ref(m);
                    const uint64_t old = __ldcg(&x);
                    x = old + (uint64_t)(int64_t)c;
                    if (c > 0 ? old != ~0ull : old != 0) break;
                }
            }
            c = map_apply(staged ? s_bmap[bk] : (uint32_t)__ldcg(&bmap[bk]), c);
        }
        if (c != 0) atomicOr(f.err, kDevErrCarry);
    }
    __syncthreads();
    // a product fits La+Lb limbs: everything above must be zero
    for (int64_t m = Lout + threadIdx.x; m < L; m += blockDim.x)
        if (__ldcg(&high[m - Lout]) != 0) atomicOr(f.err, kDevErrCarry);
}

// e^(2 pi i e / 2^16) for e < 2^15
__global__ void k_fft_table(double2* tw) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < (1 << (kFftMaxLog2 - 1))) {
        double s, c;
        sincospi((double)e / (double)(1 << (kFftMaxLog2 - 1)), &s, &c);
        tw[e] = make_double2(c, s);
    }
}

// ---------------------------------------------------------------------------

#ifndef PREC_FFT_COLS
#define PREC_FFT_COLS 1
#endif
constexpr int kFftCols = PREC_FFT_COLS;  // columns per column-pass CTA

size_t fft_table_bytes() { return (size_t)sizeof(double2) << (kFftMaxLog2 - 1); }

void fft_build_table(double2* tw, cudaStream_t st) {
    k_fft_table<<<(1 << (kFftMaxLog2 - 1)) / 256, 256, 0, st>>>(tw);
    count_launches(1);
}

static size_t cols_smem(int k1) { return (size_t)kFftCols * (fpad_host(1 << k1) + 1) * sizeof(double2); }
static size_t rows_smem(int k2) { return (size_t)2 * (fpad_host(1 << k2) + 1) * sizeof(double2); }

int fft_configure_kernels() {
    cudaError_t e = cudaFuncSetAttribute(k_fft_fwd_cols<kFftCols>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)cols_smem(kFftMaxLog2 - kFftMaxLog2 / 2));
    if (!e) e = cudaFuncSetAttribute(k_fft_inv_cols<kFftCols>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)cols_smem(kFftMaxLog2 - kFftMaxLog2 / 2));
    if (!e) e = cudaFuncSetAttribute(k_fft_rows, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)rows_smem(kFftMaxLog2 - kFftMaxLog2 / 2));
    return (int)e;
}

static int carry_blocks(uint64_t b, uint64_t ncoef, uint64_t lout) {
    const int64_t lcoef = (int64_t)((b * ncoef + 63) / 64) + 2;
    const int64_t L = lcoef > (int64_t)lout ? lcoef : (int64_t)lout;
    return (int)((L + kFftCarryBlockLimbs - 1) / kFftCarryBlockLimbs);
}

// The first kernel takes the product's arguments by value (launch
// parameters: no copy in the stream) and stores them at d_args, where the
// other three read them.
static void launch4(const FftArgs& f, FftArgs* d_args, int nblk, cudaStream_t st, cudaEvent_t* ev) {
    if (ev) cudaEventRecord(ev[0], st);
    const int ncol = (1 << f.k2) / kFftCols;
    launch_kernel(k_fft_fwd_cols<kFftCols>, ncol, 256, cols_smem(f.k1), st, f, d_args);
    if (ev) cudaEventRecord(ev[1], st);
    launch_kernel(k_fft_rows, (1 << f.k1) / 2 + 1, 256, rows_smem(f.k2), st, d_args);
    if (ev) cudaEventRecord(ev[2], st);
    launch_kernel(k_fft_inv_cols<kFftCols>, ncol, 256, cols_smem(f.k1), st, d_args);
    if (ev) cudaEventRecord(ev[3], st);
    launch_kernel(k_fft_carry, nblk, kFftCarryThreads, 0, st, d_args);
    count_launches(4);
    if (ev) cudaEventRecord(ev[4], st);
}

// One graph per (column, row) length and argument buffer (each library
// lane has its own), its carry grid the length's largest (16-bit digits;
// the extra blocks idle).  A replay sets the first node's parameters to
// the product's arguments.  (An upload of the arguments by a copy in the
// stream measured 8 us slower per product when the caller's operands were
// page-locked.)  The map is shared by the lanes (g_fft_mu); a graph is
// only replayed by its own lane, one product at a time.
struct FftGraph {
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t first = nullptr;  // k_fft_fwd_cols
    cudaKernelNodeParams params{};
    cudaGraph_t graph = nullptr;  // kept: a node's parameters are set through its graph's node handle
};
typedef std::tuple<int, int, const FftArgs*> FftGraphKey;
static std::map<FftGraphKey, FftGraph> g_fft_graphs;
static std::mutex g_fft_mu;

void fft_release_graphs(const FftArgs* d_args) {
    std::lock_guard<std::mutex> lk(g_fft_mu);
    for (auto it = g_fft_graphs.begin(); it != g_fft_graphs.end();) {
        if (d_args && std::get<2>(it->first) != d_args) {
            ++it;
            continue;
        }
        cudaGraphExecDestroy(it->second.exec);
        cudaGraphDestroy(it->second.graph);
        it = g_fft_graphs.erase(it);
    }
}

int fft_launch(const FftArgs& f, FftArgs* d_args, cudaStream_t st, cudaEvent_t* ev, cudaStream_t cap) {
    cudaError_t e;
    if (ev || !cap) {
        launch4(f, d_args, carry_blocks(f.b, f.ncoef, f.lout), st, ev);
        return (int)cudaGetLastError();
    }
    const FftGraphKey key(f.k1, f.k2, d_args);
    std::map<FftGraphKey, FftGraph>::iterator it;
    {
        std::lock_guard<std::mutex> lk(g_fft_mu);
        it = g_fft_graphs.find(key);
    }
    if (it == g_fft_graphs.end()) {
        // the four launches as a chain of kernel nodes (explicit
        // construction: no stream capture)
        GraphRecorder rec;
        if ((e = cudaGraphCreate(&rec.graph, 0)) != cudaSuccess) return (int)e;
        const uint64_t before = launches_this_thread();
        thread_recorder() = &rec;
        launch4(f, d_args, carry_blocks(16, 1ull << (f.k1 + f.k2), 0), cap, nullptr);
        thread_recorder() = nullptr;
        uncount_launches(launches_this_thread() - before);  // recorded: counted at every replay
        cudaGraph_t g = rec.graph;
        e = rec.err;
        FftGraph fg;
        // the forward column node: the first recorded
        fg.first = rec.first;
        if (e == cudaSuccess && fg.first) e = cudaGraphKernelNodeGetParams(fg.first, &fg.params);
        if (e == cudaSuccess && !fg.first) e = cudaErrorInvalidValue;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&fg.exec, g, 0);
        if (e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return (int)e;
        }
        fg.graph = g;
        std::lock_guard<std::mutex> lk(g_fft_mu);
        it = g_fft_graphs.emplace(key, fg).first;
    }
    FftGraph& fg = it->second;
    FftArgs* pub = d_args;
    void* params[2] = {const_cast<FftArgs*>(&f), &pub};
    cudaKernelNodeParams kp = fg.params;
    kp.kernelParams = params;
    kp.extra = nullptr;
    if ((e = cudaGraphExecKernelNodeSetParams(fg.exec, fg.first, &kp)) != cudaSuccess) return (int)e;
    e = cudaGraphLaunch(fg.exec, st);
    if (e == cudaSuccess) count_launches(4);
    return (int)e;
}

}  // namespace precgpu
