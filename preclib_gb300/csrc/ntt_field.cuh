// ntt_field.cuh -- 32-bit modular arithmetic for the NTT prime sets.
//
// Two sets of three NTT primes recombined by CRT from 32-bit digits (the
// reference feeds 16-bit digits to two of its primes, src/mul_ntt.cpp:29-34,
// 331-342, 489-492), and one set of five primes for whole 64-bit limbs:
//
//  set 0 (transforms up to 2^23 points): 998244353 = 119*2^23+1,
//        897581057 = 107*2^23+1, 880803841 = 105*2^23+1; generators 3, 3, 26.
//        All below 2^30, so residues may live lazily in [0, 2p) / [0, 4p)
//        (D. Harvey, "Faster arithmetic for number-theoretic transforms",
//        J. Symb. Comp. 2014): a butterfly needs no final correction.
//        p1*p2*p3 ~ 2^89.35 > 2^22 * (2^32-1)^2 bounds every coefficient
//        when min(da, db) <= 2^22 digits, which 2^23 points guarantee.
//  set 1 (2^24 .. 2^26 points): the reference's primes 469762049 =
//        7*2^26+1, 1811939329 = 27*2^26+1, 2013265921 = 15*2^27+1 with
//        generators 3, 13, 31; above 2^30, so residues are kept fully
//        reduced in [0, p).  p1*p2*p3 ~ 2^90.47 > 2^25 * (2^32-1)^2.
//  set 2 (2^13 .. 2^22 points, digits = 64-bit limbs): 998244353,
//        985661441 = 235*2^22+1, 943718401 = 225*2^22+1,
//        935329793 = 223*2^22+1, 918552577 = 219*2^22+1; generators 3, 3, 7,
//        3, 5.  All below 2^30 (set 0's lazy arithmetic).  The product
//        ~2^149.16 exceeds 2344425 * (2^64-1)^2, so every coefficient is
//        exact when min(la, lb) <= 2^21 limbs, which 2^22 points with both
//        operands in the lower half guarantee.  Half the points of a 32-bit
//        digit transform: 5 transforms of N/2 points per operand instead of
//        3 of N, about 17% fewer butterflies.
//  set 3 (2^23 .. 2^25 points, digits = 64-bit limbs): 2113929217 =
//        63*2^25+1, 2013265921, 1811939329, 1711276033 = 51*2^25+1,
//        1107296257 = 33*2^25+1; generators 5, 31, 13, 29, 10.  Above 2^30:
//        set 1's reduced arithmetic.  The product ~2^153.36 exceeds
//        42941745 * (2^64-1)^2 >= min(la, lb) (2^24 at most) * (2^64-1)^2.
//
// Multiplication methods (all on the 32-bit integer pipes):
//  * Shoup's precomputed-quotient product for twiddles known in advance:
//    x*w mod p = x*w - umulhi(x, w')*p with w' = floor(w*2^32/p), in
//    [0, 2p) for any x < 2^32 (V. Shoup, NTL).
//  * Montgomery's REDC for products of two variables (pointwise product,
//    generated four-step twiddles): a*b*2^-32 mod p in [0, 2p) whenever
//    a*b < p*2^32 (P. Montgomery, Math. Comp. 1985).
#pragma once
#include <cstdint>

namespace precgpu {

constexpr int kPrimes = 3;     // primes of sets 0 and 1
constexpr int kMaxPrimes = 5;  // primes of set 2
constexpr int kSets = 4;
constexpr int kSetMaxLog2[kSets] = {23, 26, 22, 25};  // 2-adicity cap of each set
constexpr int kSetPrimes[kSets] = {3, 3, 5, 5};
constexpr int kMaxLog2 = 26;                          // longest transform of any set
constexpr int kWideSet = 2;                           // 64-bit digits up to 2^22 points (set 0's arithmetic)
constexpr int kWideSetL = 3;                          // 64-bit digits, 2^23 .. 2^25 points (set 1's arithmetic)

// 64-bit digits over five primes
__host__ __device__ constexpr bool set_wide(int s) { return s >= kWideSet; }
// the three-prime set whose arithmetic and row / inverse-column kernels a set shares
__host__ __device__ constexpr int set_base(int s) { return s >= kWideSet ? s - kWideSet : s; }
constexpr int kMaxSubLog2 = 13;               // largest shared-memory sub-transform
constexpr int kTwLevelBits = 13;              // low level of the four-step twiddle table

// Shoup constant pair (w, floor(w * 2^32 / p)).
struct ShoupC {
    uint32_t w, wp;
};

// Per-prime constants.
struct PrimeC {
    uint32_t p;       // modulus
    uint32_t pinv;    // -p^{-1} mod 2^32 (Montgomery)
    uint32_t one_wp;  // floor(2^32 / p): Shoup constant of 1
    uint32_t p2;      // 2p
    uint32_t r32;     // 2^32 mod p
    uint32_t r32p;    // its Shoup constant floor(r32 * 2^32 / p)
};

#ifdef __CUDACC__

__device__ __forceinline__ uint32_t red1(uint32_t x, uint32_t m) {
    // x in [0, 2m) -> [0, m): unsigned min picks x - m unless it wrapped
    return min(x, x - m);
}

__device__ __forceinline__ uint32_t shoup_lazy(uint32_t x, uint32_t w, uint32_t wp, uint32_t p) {
    const uint32_t q = __umulhi(x, wp);
    return x * w - q * p;  // [0, 2p)
}

__device__ __forceinline__ uint32_t shoup_mul(uint32_t x, ShoupC c, uint32_t p) {
    return red1(shoup_lazy(x, c.w, c.wp, p), p);
}

__device__ __forceinline__ uint32_t sub_mod(uint32_t a, uint32_t b, uint32_t p) {
    return red1(a - b + p, p);
}

// REDC of a*b (a*b < p*2^32): a*b*2^-32 mod p in [0, 2p)
__device__ __forceinline__ uint32_t mont_lazy(uint32_t a, uint32_t b, const PrimeC& c) {
    const uint64_t t = (uint64_t)a * b;
    const uint32_t m = (uint32_t)t * c.pinv;
    return (uint32_t)((t + (uint64_t)m * c.p) >> 32);
}

// Arithmetic policy of a prime set.
template <int SET>
struct Ar;

// set 0: lazy.  Forward (DIF) values in [0, 2p); inverse (DIT) values in
// [0, 4p); products of two variables take operands below 2p.
template <>
struct Ar<0> {
    // a 32-bit digit into the forward range [0, 2p)
    static __device__ __forceinline__ uint32_t digit(uint32_t x, const PrimeC& c) {
        return x - __umulhi(x, c.one_wp) * c.p;
    }
    // Gentleman-Sande: (x, y) -> (x + y, (x - y) w); in and out in [0, 2p)
    static __device__ __forceinline__ void dif(uint32_t& x, uint32_t& y, uint2 w, const PrimeC& c) {
        const uint32_t s = x + y;
        const uint32_t t = x - y + c.p2;
        x = min(s, s - c.p2);
        y = shoup_lazy(t, w.x, w.y, c.p);
    }
    static __device__ __forceinline__ void dif1(uint32_t& x, uint32_t& y, const PrimeC& c) {  // w = 1
        const uint32_t s = x + y;
        const uint32_t t = x - y + c.p2;
        x = min(s, s - c.p2);
        y = min(t, t - c.p2);
    }
    // Cooley-Tukey: (x, y) -> (x + y w, x - y w); in and out in [0, 4p)
    static __device__ __forceinline__ void dit(uint32_t& x, uint32_t& y, uint2 w, const PrimeC& c) {
        const uint32_t xr = min(x, x - c.p2);
        const uint32_t t = shoup_lazy(y, w.x, w.y, c.p);
        x = xr + t;
        y = xr - t + c.p2;
    }
    static __device__ __forceinline__ void dit1(uint32_t& x, uint32_t& y, const PrimeC& c) {
        const uint32_t xr = min(x, x - c.p2);
        const uint32_t yr = min(y, y - c.p2);
        x = xr + yr;
        y = xr - yr + c.p2;
    }
    // product of two operands below 2p -> [0, 2p)
    static __device__ __forceinline__ uint32_t mul(uint32_t a, uint32_t b, const PrimeC& c) {
        return mont_lazy(a, b, c);
    }
    // x * w for a table twiddle, any 32-bit x -> [0, 2p)
    static __device__ __forceinline__ uint32_t twiddle(uint32_t x, uint2 w, const PrimeC& c) {
        return shoup_lazy(x, w.x, w.y, c.p);
    }
    // inverse-range value [0, 4p) -> forward range [0, 2p)
    static __device__ __forceinline__ uint32_t half(uint32_t x, const PrimeC& c) {
        return min(x, x - c.p2);
    }
};

// set 2: set 0's arithmetic; a digit is a whole 64-bit limb hi*2^32 + lo
template <>
struct Ar<2> : Ar<0> {
    static __device__ __forceinline__ uint32_t digit64(uint32_t lo, uint32_t hi, const PrimeC& c) {
        const uint32_t l = lo - __umulhi(lo, c.one_wp) * c.p;  // [0, 2p)
        const uint32_t h = shoup_lazy(hi, c.r32, c.r32p, c.p);  // [0, 2p)
        const uint32_t s = l + h;                                // [0, 4p)
        return min(s, s - c.p2);
    }
};

// set 1: fully reduced in [0, p) everywhere (p up to 2^31).
template <>
struct Ar<1> {
    static __device__ __forceinline__ uint32_t digit(uint32_t x, const PrimeC& c) {
        return red1(x - __umulhi(x, c.one_wp) * c.p, c.p);
    }
    static __device__ __forceinline__ void dif(uint32_t& x, uint32_t& y, uint2 w, const PrimeC& c) {
        const uint32_t s = x + y;
        const uint32_t d = x - y + c.p;
        x = red1(s, c.p);
        y = red1(shoup_lazy(d, w.x, w.y, c.p), c.p);
    }
    static __device__ __forceinline__ void dif1(uint32_t& x, uint32_t& y, const PrimeC& c) {
        const uint32_t s = x + y;
        const uint32_t d = x - y + c.p;
        x = red1(s, c.p);
        y = red1(d, c.p);
    }
    static __device__ __forceinline__ void dit(uint32_t& x, uint32_t& y, uint2 w, const PrimeC& c) {
        const uint32_t t = red1(shoup_lazy(y, w.x, w.y, c.p), c.p);
        const uint32_t s = x + t;
        const uint32_t d = x - t + c.p;
        x = red1(s, c.p);
        y = red1(d, c.p);
    }
    static __device__ __forceinline__ void dit1(uint32_t& x, uint32_t& y, const PrimeC& c) {
        const uint32_t s = x + y;
        const uint32_t d = x - y + c.p;
        x = red1(s, c.p);
        y = red1(d, c.p);
    }
    static __device__ __forceinline__ uint32_t mul(uint32_t a, uint32_t b, const PrimeC& c) {
        return red1(mont_lazy(a, b, c), c.p);
    }
    static __device__ __forceinline__ uint32_t twiddle(uint32_t x, uint2 w, const PrimeC& c) {
        return red1(shoup_lazy(x, w.x, w.y, c.p), c.p);
    }
    static __device__ __forceinline__ uint32_t half(uint32_t x, const PrimeC&) { return x; }
};

// set 3: set 1's arithmetic; a digit is a whole 64-bit limb hi*2^32 + lo
template <>
struct Ar<3> : Ar<1> {
    static __device__ __forceinline__ uint32_t digit64(uint32_t lo, uint32_t hi, const PrimeC& c) {
        const uint32_t l = red1(lo - __umulhi(lo, c.one_wp) * c.p, c.p);    // [0, p)
        const uint32_t h = red1(shoup_lazy(hi, c.r32, c.r32p, c.p), c.p);  // [0, p)
        return red1(l + h, c.p);                                             // l + h < 2p < 2^32
    }
};

#endif  // __CUDACC__

}  // namespace precgpu
