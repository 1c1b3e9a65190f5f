// ntt_field.cuh -- 32-bit modular arithmetic for the three NTT primes.
//
// The residue ring follows preclib's NTT band (src/mul_ntt.cpp:29-34): the
// primes 469762049 = 7*2^26+1, 1811939329 = 27*2^26+1, 2013265921 =
// 15*2^27+1 with generators 3, 13, 31.  Their 2-adicity (26) caps the
// transform at 2^26 points, the reference's own cap (mul_ntt.cpp:28).
// Unlike the reference (16-bit digits, two primes), this library feeds
// 32-bit digits and recombines all three primes: a coefficient of the
// digit convolution is below min(da,db)*(2^32-1)^2 < p1*p2*p3 (~2^90.47)
// for min(da,db) <= 2^25, which every transform up to 2^26 points meets.
//
// Multiplication methods (all on the 32-bit integer pipes):
//  * Shoup's precomputed-quotient product for twiddles known in advance:
//    x*w mod p = x*w - umulhi(x, w')*p with w' = floor(w*2^32/p), exact
//    in [0, 2p) for any x < 2^32 (V. Shoup, NTL; D. Harvey, "Faster
//    arithmetic for number-theoretic transforms", 2014).
//  * Montgomery's REDC for products of two variables (pointwise product,
//    generated four-step twiddles): a*b*2^-32 mod p (P. Montgomery 1985).
// Residues are kept fully reduced in [0, p); p < 2^31 so every sum of two
// residues and every x - y + p fits in 32 bits.
#pragma once
#include <cstdint>

#ifndef PREC_HD
#define PREC_HD __host__ __device__ __forceinline__
#endif

namespace precgpu {

constexpr int kPrimes = 3;
constexpr int kMaxLog2N = 26;      // 2-adicity of the smallest prime
constexpr int kMaxSubLog2 = 13;    // largest shared-memory sub-transform
constexpr int kTwLevelBits = 13;   // two-level four-step twiddle table split

// Shoup constant pair (w, floor(w * 2^32 / p)).
struct ShoupC {
    uint32_t w, wp;
};

// Per-prime constants, resident in __constant__ memory.
struct PrimeC {
    uint32_t p;       // modulus
    uint32_t pinv;    // -p^{-1} mod 2^32 (Montgomery)
    uint32_t one_wp;  // floor(2^32 / p): Shoup constant of 1, reduces x < 2^32
    uint32_t pad;
};

__device__ __forceinline__ uint32_t red1(uint32_t x, uint32_t p) {
    // x in [0, 2p) -> [0, p): unsigned min picks x - p unless it wrapped
    return min(x, x - p);
}

__device__ __forceinline__ uint32_t add_mod(uint32_t a, uint32_t b, uint32_t p) {
    return red1(a + b, p);
}

__device__ __forceinline__ uint32_t sub_mod(uint32_t a, uint32_t b, uint32_t p) {
    return red1(a - b + p, p);
}

// Shoup product, result in [0, 2p)
__device__ __forceinline__ uint32_t shoup_lazy(uint32_t x, uint32_t w, uint32_t wp, uint32_t p) {
    uint32_t q = __umulhi(x, wp);
    return x * w - q * p;
}

__device__ __forceinline__ uint32_t shoup_mul(uint32_t x, ShoupC c, uint32_t p) {
    return red1(shoup_lazy(x, c.w, c.wp, p), p);
}

// x < 2^32 -> x mod p
__device__ __forceinline__ uint32_t reduce_u32(uint32_t x, const PrimeC& c) {
    return red1(x - __umulhi(x, c.one_wp) * c.p, c.p);
}

// Montgomery product a*b*2^-32 mod p for a, b < p (p < 2^31).
__device__ __forceinline__ uint32_t mont_mul(uint32_t a, uint32_t b, const PrimeC& c) {
    uint64_t t = (uint64_t)a * b;
    uint32_t m = (uint32_t)t * c.pinv;
    uint64_t u = (t + (uint64_t)m * c.p) >> 32;  // < 2p
    return red1((uint32_t)u, c.p);
}

// Gentleman-Sande (DIF) butterfly: (x, y) -> (x + y, (x - y) * w)
__device__ __forceinline__ void bfly_dif(uint32_t& x, uint32_t& y, uint2 w, uint32_t p) {
    uint32_t s = x + y;
    uint32_t d = x - y + p;
    x = red1(s, p);
    y = red1(shoup_lazy(d, w.x, w.y, p), p);
}

// Cooley-Tukey (DIT) butterfly: (x, y) -> (x + y*w, x - y*w)
__device__ __forceinline__ void bfly_dit(uint32_t& x, uint32_t& y, uint2 w, uint32_t p) {
    uint32_t t = red1(shoup_lazy(y, w.x, w.y, p), p);
    uint32_t s = x + t;
    uint32_t d = x - t + p;
    x = red1(s, p);
    y = red1(d, p);
}

}  // namespace precgpu
