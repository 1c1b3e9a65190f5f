// ref_shim.cpp -- C entry points over the reference's own multiply.
//
// TEST INFRASTRUCTURE ONLY.  Compiled together with the reference's
// src/*.cpp by oracle/build_ref.sh into oracle/_ref/libprecref.so, so the
// restatement in oracle_mul.c can be checked against the reference itself
// and golden vectors can be generated from it.  It exists only where the
// reference sources are present (never on a machine without them).
#include "prec.hpp"

#include <cstdint>
#include <cstring>

static precn_t ref_make(const uint64_t *a, size_t n) {
    precn_t r;  // default ctor: asiz 1, rsiz 0 (src/init_basic.cpp)
    if (n) {
        r.a = (uint64_t *)realloc(r.a, n * sizeof(uint64_t));
        r.asiz = n;
        memcpy(r.a, a, n * sizeof(uint64_t));
    }
    r.rsiz = n;
    while (r.rsiz > 0 && r.a[r.rsiz - 1] == 0) --r.rsiz;
    if (r.rsiz == 0) r.a[0] = 0;
    return r;
}

static size_t ref_out(const precn_t &p, uint64_t *out, size_t cap) {
    memset(out, 0, cap * sizeof(uint64_t));
    size_t n = p.rsiz < cap ? p.rsiz : cap;
    if (n) memcpy(out, p.a, n * sizeof(uint64_t));
    return p.rsiz;
}

extern "C" {

size_t ref_mul_ntt(const uint64_t *a, size_t an, const uint64_t *b, size_t bn, uint64_t *out) {
    precn_t x = ref_make(a, an), y = ref_make(b, bn);
    return ref_out(mul_ntt(x, y), out, an + bn);
}

size_t ref_mul_fft(const uint64_t *a, size_t an, const uint64_t *b, size_t bn, uint64_t *out,
                   double *max_err) {
    precn_t x = ref_make(a, an), y = ref_make(b, bn);
    double before = max_fft_rounding_error;
    max_fft_rounding_error = 0.0;
    size_t r = ref_out(mul_fft(x, y), out, an + bn);
    if (max_err) *max_err = max_fft_rounding_error;
    if (before > max_fft_rounding_error) max_fft_rounding_error = before;
    return r;
}

size_t ref_mul_basic(const uint64_t *a, size_t an, const uint64_t *b, size_t bn, uint64_t *out) {
    precn_t x = ref_make(a, an), y = ref_make(b, bn);
    return ref_out(mul_basic(x, y), out, an + bn);
}

// operator* through the reference dispatcher (src/mul_basic.cpp:278-284)
size_t ref_mul(const uint64_t *a, size_t an, const uint64_t *b, size_t bn, uint64_t *out) {
    precn_t x = ref_make(a, an), y = ref_make(b, bn);
    return ref_out(x * y, out, an + bn);
}

// precn_sqr (src/mul_basic.cpp:193-205)
size_t ref_sqr(const uint64_t *a, size_t an, uint64_t *out) {
    precn_t x = ref_make(a, an);
    return ref_out(precn_sqr(x), out, 2 * an);
}

}  // extern "C"
