// prec_gpu_precn.cpp -- preclib's mul_ntt and mul_fft, computed on the GPU.
//
// preclib's dispatcher reaches its two large-operand multipliers through
// the free functions mul_ntt and mul_fft, called by name
// (src/mul_basic.cpp:203, 264, 268; also src/mul_ssa.cpp and the test
// programs).  This file defines both with the same C++ signatures on top of
// the C ABI of libprecgpu, so a preclib build that leaves out
// src/mul_ntt.cpp and src/mul_fft.cpp (see link_preclib.sh beside this
// file) runs every product of the two bands on the GPU, with operator*,
// precn_sqr, division, sqrt and the pi program unchanged.
//
// Contract kept from the replaced functions (src/mul_ntt.cpp:494-518,
// src/mul_fft.cpp:386-394):
//   * the result is returned by value, normalised (no zero top limb), and
//     zero is rsiz 0 with a[0] = 0 and asiz >= 1 (init_basic.cpp:47-52);
//   * the limb array is malloc/realloc memory owned by the precn_t
//     (freed by ~precn_t, init_basic.cpp:133);
//   * failures do not return: the reference aborts (mul_ntt.cpp:135-136),
//     and so does this file, after naming the library's error code;
//   * with COUNT_FFTS the rounding statistics of mul_fft (mul_fft.cpp:32-38,
//     359-382) are kept from the library's per-product maximum distance.
// Sizes the reference hands to its schoolbook code (<= 192 limbs) are
// computed on the GPU as well: there is no CPU path here.
//
// Needs preclib's prec.hpp on the include path and links against
// libprecgpu (include/prec_gpu.h).
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "prec.hpp"
#include "prec_gpu.h"

#if defined(COUNT_FFTS) && COUNT_FFTS
// weak, so a build that keeps the reference's mul_fft.cpp under another
// name links its own definitions instead
__attribute__((weak)) uint64_t total_fftmuls = 0;
__attribute__((weak)) uint64_t danger_fftmuls = 0;
__attribute__((weak)) uint64_t danger_fftmuls_1_4 = 0;
__attribute__((weak)) uint64_t danger_fftmuls_3_8 = 0;
__attribute__((weak)) double max_fft_rounding_error = 0.0;
#endif

namespace {

using gpu_mul_fn = int (*)(const uint64_t*, size_t, const uint64_t*, size_t, uint64_t*);

[[noreturn]] void fail(const char* who, int rc) {
    std::fprintf(stderr, "prec_gpu: %s: %s (code %d)\n", who, prec_gpu_strerror(rc), rc);
    std::abort();
}

void count_fft(const prec_gpu_stats_t& st) {
#if defined(COUNT_FFTS) && COUNT_FFTS
    if (st.path != 2) return;  // only FP64-band products have a distance
    const double e = st.fft_max_distance;
    ++total_fftmuls;
    if (e > 0.125) ++danger_fftmuls;
    if (e > 0.25) ++danger_fftmuls_1_4;
    if (e > 0.375) ++danger_fftmuls_3_8;
    if (e > max_fft_rounding_error) max_fft_rounding_error = e;
#else
    (void)st;
#endif
}

// One product through the C ABI.  Both operands are the same object for a
// square (operator* passes &a == &b to precn_sqr, mul_basic.cpp:244-246):
// the library sees equal pointers and takes its square route.
precn_t gpu_product(const precn_t& a, const precn_t& b, gpu_mul_fn fn, const char* who) {
    precn_t r;
    if (a.rsiz == 0 || b.rsiz == 0) return r;
    const size_t n = a.rsiz + b.rsiz;
    uint64_t* limbs = static_cast<uint64_t*>(std::realloc(r.a, n * sizeof(uint64_t)));
    if (!limbs) fail(who, PREC_GPU_E_NOMEM);
    r.a = limbs;
    r.asiz = n;
    const int rc = fn(a.a, a.rsiz, b.a, b.rsiz, r.a);
    if (rc != PREC_GPU_OK) fail(who, rc);
    prec_gpu_stats_t st;
    if (prec_gpu_last_stats(&st) == PREC_GPU_OK) count_fft(st);
    r.rsiz = n;
    while (r.rsiz > 0 && r.a[r.rsiz - 1] == 0) --r.rsiz;
    if (r.rsiz == 0) r.a[0] = 0;
    return r;
}

}  // namespace

// src/mul_ntt.cpp:494 -- the NTT band
precn_t mul_ntt(const precn_t& a, const precn_t& b) { return gpu_product(a, b, prec_gpu_mul_ntt, "mul_ntt"); }

// src/mul_fft.cpp:386 -- the FP64 band up to 6144 limbs; larger operands
// (squares that precn_sqr sends here at any size, mul_basic.cpp:203) run
// on the NTT band, which gives the same exact product
precn_t mul_fft(const precn_t& a, const precn_t& b) { return gpu_product(a, b, prec_gpu_mul, "mul_fft"); }
