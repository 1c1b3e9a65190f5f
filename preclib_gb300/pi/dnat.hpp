// dnat.hpp -- natural numbers resident in device memory, for the Newton
// steps of the pi program (reciprocal, exact division, integer square root)
// and the powers of ten of its decimal conversion.
//
// bignum.hpp's Newton operations keep their iterates in host memory, and
// every product goes host -> device -> host through prec_gpu_mul: at 10^8
// digits a top-level product moves ~170 MB over the link for ~1.5 ms of
// device work.  Here the iterates stay on the device: products run through
// prec_gpu_mul_device on the math object's stream, and the linear steps
// (shifts, additions, subtractions, comparisons) are device kernels.  Only
// a few bytes come back per step (the top limbs that fix a result's exact
// length, a comparison's sign).  The algorithms and their error bounds are
// those of bignum.cpp; the results of the exact operations (quotient and
// remainder, integer square root) are the same numbers.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "bignum.hpp"

namespace precpi {

class DevMath;

// kernels this module launched (the signed additions are counted by
// signed_add_launches, the products by prec_gpu_launch_count)
uint64_t dnat_launches();

// little-endian limbs in device memory, no zero top limb (zero: n == 0);
// bits = bitlen.  Memory is stream-ordered on `st` (the stream it was made
// on, or the one it was handed to with DevMath::adopt).
struct DNat {
    u64* d = nullptr;
    size_t n = 0;
    size_t bits = 0;
    cudaStream_t st = nullptr;
    DNat() = default;
    DNat(const DNat&) = delete;
    DNat& operator=(const DNat&) = delete;
    DNat(DNat&& o) noexcept { *this = static_cast<DNat&&>(o); }
    DNat& operator=(DNat&& o) noexcept;
    ~DNat();
    bool zero() const { return n == 0; }
};

// bignum.hpp's DecimalPowers on the device: pw[j] = 10^(L * 2^j), rx[j] its
// reciprocal at precision P[j] = bitlen(pw[j]) + 34 (L = kDecimalLeafDigits)
struct DevDecimalPowers {
    std::vector<DNat> pw, rx;
    std::vector<size_t> P;
};

class DevMath {
public:
    explicit DevMath(cudaStream_t st);
    ~DevMath();
    DevMath(const DevMath&) = delete;
    DevMath& operator=(const DevMath&) = delete;
    cudaStream_t stream() const { return st_; }

    DNat upload(const Nat& x);
    Nat download(const DNat& x);
    // a number made on another math object's stream, after that stream's
    // work on it is complete (its owner synchronised): frees go to this stream
    void adopt(DNat& x) { x.st = st_; }

    DNat copy(const DNat& a);
    DNat pow2(size_t bits);
    DNat shr(const DNat& a, size_t bits);
    DNat shl(const DNat& a, size_t bits);
    DNat mul(const DNat& a, const DNat& b);
    DNat sqr(const DNat& a) { return mul(a, a); }
    DNat mul_u64(const DNat& a, u64 v);
    DNat pow_u64(u64 base, size_t e);  // base^e by squarings on the device
    DNat add(const DNat& a, const DNat& b);
    DNat sub(const DNat& a, const DNat& b);  // a >= b
    // |a - b|; sign of a - b in *sign (-1, 0, 1)
    DNat absdiff(const DNat& a, const DNat& b, int* sign);
    int cmp(const DNat& a, const DNat& b);

    // bignum.hpp's Newton operations on device numbers (same contracts)
    DNat recip(const DNat& D, size_t p);
    // the conversion's powers and reciprocals (bignum.hpp's decimal_powers)
    DevDecimalPowers decimal_powers(int levels);
    // powers made on another math object's stream, after it synchronised
    void adopt(DevDecimalPowers& p);
    // the decimal digits of x without leading zeros ("0" for zero), as
    // bignum.hpp's to_decimal: the same divide and conquer on the powers
    // (pw holds at least decimal_levels(digits of x) levels), every level's
    // pieces split on the device in one pass, the leaves converted by one
    // kernel; only the digit text comes back (ddec.cu)
    std::string to_decimal(const DNat& x, const DevDecimalPowers& pw);
    void divmod_recip(const DNat& N, const DNat& D, const DNat& X, size_t P, DNat* q, DNat* r);
    DNat isqrt(const DNat& n);

    // device kernels and products issued (for the program's summary)
    size_t products = 0, syncs = 0;

private:
    DNat alloc(size_t limbs);
    // exact length and bit length of x's first `limbs` limbs (reads the top
    // limbs back: one synchronisation)
    void fix_size(DNat& x, size_t limbs);
    DNat signed_sum(const DNat& a, int sa, const DNat& b, int sb, int* sign);
    DNat invsqrt(const DNat& n, size_t e, size_t p);

    cudaStream_t st_;
    u64* h_top_ = nullptr;     // pinned read-back of top limbs / flags
    void* dev_ = nullptr;      // one pair descriptor, its signs, the compare word
    void* scratch_ = nullptr;  // the add kernels' scratch and chunk table
    size_t scratch_cap_ = 0;
};

}  // namespace precpi
