// Test driver of prec_gpu_precn.cpp over the stand-in precn_t: C entry
// points that wrap host limb arrays in precn_t values, call mul_ntt /
// mul_fft exactly as preclib's dispatcher does, and copy the normalised
// result out (loaded with ctypes by tests/test_precn_gpu.py).
#include <cstdlib>
#include <cstring>

#include "prec.hpp"

precn_t::precn_t() : asiz(1), rsiz(0), a(static_cast<uint64_t*>(std::malloc(sizeof(uint64_t)))) { a[0] = 0; }
precn_t::precn_t(precn_t&& o) : asiz(o.asiz), rsiz(o.rsiz), a(o.a) {
    o.a = static_cast<uint64_t*>(std::malloc(sizeof(uint64_t)));
    o.a[0] = 0;
    o.asiz = 1;
    o.rsiz = 0;
}
precn_t::~precn_t() { std::free(a); }

static void load(precn_t& x, const uint64_t* v, size_t n) {
    x.a = static_cast<uint64_t*>(std::realloc(x.a, (n ? n : 1) * sizeof(uint64_t)));
    x.asiz = n ? n : 1;
    if (n) std::memcpy(x.a, v, n * sizeof(uint64_t));
    x.rsiz = n;
    while (x.rsiz && x.a[x.rsiz - 1] == 0) --x.rsiz;
    if (!x.rsiz) x.a[0] = 0;
}

// which: 0 = mul_ntt, 1 = mul_fft; square != 0 passes the same object twice.
// Writes rsiz limbs to out (capacity an + bn) and returns rsiz; *zero_ok is
// set when a zero result has a[0] == 0 and asiz >= 1.
extern "C" size_t shim_mul(int which, int square, const uint64_t* a, size_t an, const uint64_t* b, size_t bn,
                           uint64_t* out, int* zero_ok) {
    precn_t x, y;
    load(x, a, an);
    if (!square) load(y, b, bn);
    const precn_t& rhs = square ? x : y;
    precn_t r = which ? mul_fft(x, rhs) : mul_ntt(x, rhs);
    if (r.rsiz) std::memcpy(out, r.a, r.rsiz * sizeof(uint64_t));
    *zero_ok = r.rsiz == 0 ? (r.asiz >= 1 && r.a[0] == 0) : (r.a[r.rsiz - 1] != 0);
    return r.rsiz;
}

extern "C" void shim_fft_counters(uint64_t* counts, double* max_err) {
    counts[0] = total_fftmuls;
    counts[1] = danger_fftmuls;
    counts[2] = danger_fftmuls_1_4;
    counts[3] = danger_fftmuls_3_8;
    *max_err = max_fft_rounding_error;
}
