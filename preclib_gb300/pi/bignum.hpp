// bignum.hpp -- natural numbers for the pi program: host-side linear
// arithmetic (add, subtract, shift, compare, single-limb multiply and
// divide) and the Newton-based operations built on a multiply backend
// (reciprocal, exact division, integer square root, decimal conversion).
//
// Every product above the backend's host threshold goes to the backend;
// the pi program's backend is the GPU library (pi_gpu.cpp), and many
// independent products of one step (a binary-splitting level, a level of
// the decimal conversion) are handed over together as one batch.
#pragma once
#include <cstddef>
#include <cstdint>
#include <functional>
#include <memory>
#include <string>
#include <vector>

namespace precpi {

using u64 = uint64_t;
using u128 = unsigned __int128;

// Limb buffers of at least kBigBytes are kept for reuse when freed (up to a
// bound): the Newton steps and the conversion levels allocate and free
// numbers of nearly the same sizes over and over, and the C library maps
// fresh pages for every allocation of that size (a fault and a kernel zero
// fill per page).  Smaller buffers use the C library's heap.
constexpr size_t kBigBytes = (size_t)32 << 20;
void* big_alloc(size_t bytes);
void big_free(void* p) noexcept;

template <class T>
struct LimbAlloc {
    using value_type = T;
    LimbAlloc() = default;
    template <class U>
    LimbAlloc(const LimbAlloc<U>&) noexcept {}
    T* allocate(size_t n) {
        if (n * sizeof(T) >= kBigBytes) return static_cast<T*>(big_alloc(n * sizeof(T)));
        return std::allocator<T>().allocate(n);
    }
    void deallocate(T* p, size_t n) noexcept {
        if (n * sizeof(T) >= kBigBytes) big_free(p);
        else std::allocator<T>().deallocate(p, n);
    }
    template <class U>
    bool operator==(const LimbAlloc<U>&) const noexcept {
        return true;
    }
    template <class U>
    bool operator!=(const LimbAlloc<U>&) const noexcept {
        return false;
    }
};
using Limbs = std::vector<u64, LimbAlloc<u64>>;

// little-endian limbs, no zero top limb (zero = empty)
struct Nat {
    Limbs d;
    Nat() = default;
    explicit Nat(u64 v) {
        if (v) d.push_back(v);
    }
    bool zero() const { return d.empty(); }
    size_t size() const { return d.size(); }
};

// Products: one at a time or many independent ones (the batch form).
struct MulBackend {
    virtual ~MulBackend() = default;
    // out = a * b (a or b may be zero); a and b may be the same object
    virtual void mul(const Nat& a, const Nat& b, Nat& out) = 0;
    // out[i] = *a[i] * *b[i]
    virtual void mul_many(const std::vector<const Nat*>& a, const std::vector<const Nat*>& b,
                          std::vector<Nat>& out) = 0;
};

void set_backend(MulBackend* be);
MulBackend& backend();

// host threads for the linear work (and small products)
void parallel_for(size_t n, const std::function<void(size_t)>& fn);

void normalize(Nat& x);
int cmp(const Nat& a, const Nat& b);
size_t bitlen(const Nat& a);
Nat add(const Nat& a, const Nat& b);
Nat sub(const Nat& a, const Nat& b);  // a >= b
void add_in(Nat& a, const Nat& b);    // a += b
void sub_in(Nat& a, const Nat& b);    // a -= b, a >= b
Nat shl(const Nat& a, size_t bits);
Nat shr(const Nat& a, size_t bits);
Nat pow2(size_t bits);
Nat mul_u64(const Nat& a, u64 b);
u64 divmod_u64(Nat& a, u64 b);  // a /= b, returns a mod b
// schoolbook product on the host (small operands)
void mul_school(const u64* a, size_t an, const u64* b, size_t bn, u64* out);

Nat mul(const Nat& a, const Nat& b);
Nat sqr(const Nat& a);
Nat pow_u64(u64 base, size_t e);

// Reciprocal: X with |X - 2^(bitlen(D) + p) / D| <= 4, p >= 1.
Nat recip(const Nat& D, size_t p);
// exact floor division and remainder (D > 0)
void divmod(const Nat& N, const Nat& D, Nat& q, Nat& r);
// the same with X = recip(D, P) computed ahead (P >= bitlen(N) - bitlen(D) + 34)
void divmod_recip(const Nat& N, const Nat& D, const Nat& X, size_t P, Nat& q, Nat& r);
// floor(sqrt(n))
Nat isqrt(const Nat& n);
// Y with |Y - 2^(e/2 + p) / sqrt(n)| <= 4, for even e >= bitlen(n)
// (the Newton inverse square root isqrt is built on)
Nat invsqrt(const Nat& n, size_t e, size_t p);

// Digits per leaf of the decimal conversion (divide and conquer down to
// numbers below 10^L, each then converted by repeated division by 10^19)
#ifndef PI_LEAF_DIGITS
#define PI_LEAF_DIGITS 2048
#endif
constexpr size_t kDecimalLeafDigits = PI_LEAF_DIGITS;

// The powers 10^(L * 2^j), j < levels (L = the leaf size in digits), and
// their reciprocals: all that decimal conversion needs besides x, so a
// caller that knows the size of x can build them ahead of time.
struct DecimalPowers {
    std::vector<Nat> pw;     // 10^(L * 2^j)
    std::vector<Nat> rx;     // recip(pw[j], bitlen(pw[j]) + 34)
    std::vector<size_t> P;   // that precision
};
// levels the conversion of a number of `digits` decimal digits splits into
int decimal_levels(size_t digits);
DecimalPowers decimal_powers(int levels);

// Exact decimal digits of x, padded with leading zeros to at least
// `width` characters; `pre` (optional) holds powers built ahead of time
// (any number of levels; missing ones are computed here).
std::string to_decimal(const Nat& x, size_t width, const DecimalPowers* pre = nullptr);

}  // namespace precpi
