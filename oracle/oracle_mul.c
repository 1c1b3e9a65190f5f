/*
 * oracle_mul.c -- CPU restatement of preclib's large-operand multiply.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU library:
 * only the tests, the smoke check and the CPU-baseline leg of bench.py load
 * it.  Nothing in the shipped library calls into it.
 *
 * It restates, in plain C, the algorithms of the reference (preclib):
 *   - src/mul_ntt.cpp  : 16-bit digits, 2 (or 3) 31-bit primes, 32-bit
 *                        Montgomery arithmetic, forward DIF / inverse DIT
 *                        radix-2 NTT, Garner CRT, serial carry.
 *   - src/mul_fft.cpp  : 16/8-bit digits packed as re/im of one complex
 *                        FP64 FFT, recurrence twiddles, pair separation,
 *                        rounding with distance statistics, serial carry.
 *   - src/mul_basic.cpp: schoolbook product (mul_basic).
 * The scalar code paths of the reference are followed operation for
 * operation, so the FFT rounding distances reproduce the reference's.
 *
 * Parity of this restatement is pinned two ways: against the reference
 * compiled from its own sources (oracle/build_ref.sh -> oracle/_ref/) and
 * against golden vectors generated from that build (tests/golden/).
 *
 * Limb convention (prec.hpp:49-52): little-endian uint64 limbs,
 * value = a[0] + a[1]*2^64 + ...  Every entry point writes an+bn limbs to
 * `out` (zero padded) and returns the normalised length (no top zero limb).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;

/* ------------------------------------------------------------------ */
/* helpers                                                              */
/* ------------------------------------------------------------------ */

static size_t norm_len(const uint64_t *a, size_t n) {
    while (n > 0 && a[n - 1] == 0) --n;
    return n;
}

static void *xcalloc(size_t n, size_t sz) {
    void *p = calloc(n ? n : 1, sz);
    if (!p) abort();
    return p;
}

/* ------------------------------------------------------------------ */
/* schoolbook: mul_basic (src/mul_basic.cpp:131-185, 286-288)           */
/* ------------------------------------------------------------------ */

size_t oracle_mul_basic(const uint64_t *a, size_t an, const uint64_t *b,
                        size_t bn, uint64_t *out) {
    size_t total = an + bn;
    memset(out, 0, total * sizeof(uint64_t));
    an = norm_len(a, an);
    bn = norm_len(b, bn);
    if (an == 0 || bn == 0) return 0;
    for (size_t i = 0; i < an; ++i) {
        uint64_t carry = 0;
        for (size_t j = 0; j < bn; ++j) {
            u128 t = (u128)a[i] * b[j] + out[i + j] + carry;
            out[i + j] = (uint64_t)t;
            carry = (uint64_t)(t >> 64);
        }
        size_t k = i + bn;
        while (carry) {
            u128 t = (u128)out[k] + carry;
            out[k] = (uint64_t)t;
            carry = (uint64_t)(t >> 64);
            ++k;
        }
    }
    return norm_len(out, total);
}

/* ------------------------------------------------------------------ */
/* NTT band: mul_ntt (src/mul_ntt.cpp)                                  */
/* ------------------------------------------------------------------ */

/* The three NTT primes and generators of the reference
 * (src/mul_ntt.cpp:29-34).  Montgomery constants are derived here rather
 * than tabulated (the reference tabulates them at mul_ntt.cpp:37-41 from
 * tools/ntt_montgomery_constants.py). */
static const uint32_t ORC_MOD[3] = {469762049u, 1811939329u, 2013265921u};
static const uint32_t ORC_ROOT[3] = {3u, 13u, 31u};
#define ORC_MAX_LIMBS ((size_t)1 << 24)     /* mul_ntt.cpp:27 */
#define ORC_MAX_TRANSFORM ((size_t)1 << 26) /* mul_ntt.cpp:28 */

typedef struct {
    uint32_t mod, root, ninv, r2, one;
} orc_mont_t;

/* -mod^{-1} mod 2^32 by Newton iteration on the 2-adic inverse. */
static uint32_t orc_neg_inv32(uint32_t m) {
    uint32_t x = 1;
    for (int i = 0; i < 5; ++i) x = x * (2u - m * x);
    return (uint32_t)(0u - x);
}

static orc_mont_t orc_mont_make(int idx) {
    orc_mont_t c;
    c.mod = ORC_MOD[idx];
    c.root = ORC_ROOT[idx];
    c.ninv = orc_neg_inv32(c.mod);
    c.r2 = (uint32_t)(((u128)1 << 64) % c.mod);
    c.one = (uint32_t)(((uint64_t)1 << 32) % c.mod);
    return c;
}

/* REDC (mul_ntt.cpp:43-48) */
static inline uint32_t orc_redc(const orc_mont_t *c, uint64_t x) {
    uint32_t m = (uint32_t)x * c->ninv;
    uint64_t t = (x + (uint64_t)m * c->mod) >> 32;
    if (t >= c->mod) t -= c->mod;
    return (uint32_t)t;
}
/* mul_ntt.cpp:50-59 */
static inline uint32_t orc_to_mont(const orc_mont_t *c, uint32_t x) {
    return orc_redc(c, (uint64_t)x * c->r2);
}
static inline uint32_t orc_mmul(const orc_mont_t *c, uint32_t a, uint32_t b) {
    return orc_redc(c, (uint64_t)a * b);
}
/* mul_ntt.cpp:139-148 */
static uint32_t orc_mpow(const orc_mont_t *c, uint32_t a, uint64_t e) {
    uint32_t r = c->one;
    uint32_t x = orc_to_mont(c, a);
    while (e) {
        if (e & 1) r = orc_mmul(c, r, x);
        e >>= 1;
        if (e) x = orc_mmul(c, x, x);
    }
    return r;
}

typedef struct {
    orc_mont_t c;
    uint32_t inv_n;
    uint32_t *fw; /* fw[half + j] = w_len^j (Montgomery), len = 2*half */
    uint32_t *iv; /* iv[half + j] = inverse roots, mul_ntt.cpp:167-170 */
} orc_plan_t;

/* ntt_build_roots / ntt_make_mod_plan (mul_ntt.cpp:150-180) */
static void orc_plan_init(orc_plan_t *p, int idx, size_t n) {
    p->c = orc_mont_make(idx);
    const orc_mont_t *c = &p->c;
    p->inv_n = orc_mpow(c, (uint32_t)(n % c->mod), c->mod - 2);
    p->fw = (uint32_t *)xcalloc(n, sizeof(uint32_t));
    p->iv = (uint32_t *)xcalloc(n, sizeof(uint32_t));
    if (n) {
        p->fw[0] = c->one;
        p->iv[0] = c->one;
    }
    for (size_t len = 2; len <= n; len <<= 1) {
        size_t half = len >> 1;
        uint32_t step = orc_mpow(c, c->root, (uint64_t)(c->mod - 1) / len);
        uint32_t w = c->one;
        for (size_t j = 0; j < half; ++j) {
            p->fw[half + j] = w;
            w = orc_mmul(c, w, step);
        }
        p->iv[half] = c->one;
        for (size_t j = 1; j < half; ++j)
            p->iv[half + j] = c->mod - p->fw[half + half - j];
    }
}

static void orc_plan_free(orc_plan_t *p) {
    free(p->fw);
    free(p->iv);
}

/* ntt_get_mod_plan (mul_ntt.cpp:182-191): one cached plan per prime and
 * thread, rebuilt when the transform length changes */
static const orc_plan_t *orc_get_plan(int idx, size_t n) {
    static _Thread_local orc_plan_t plans[3];
    static _Thread_local size_t sizes[3];
    if (sizes[idx] != n) {
        if (sizes[idx]) orc_plan_free(&plans[idx]);
        orc_plan_init(&plans[idx], idx, n);
        sizes[idx] = n;
    }
    return &plans[idx];
}

/* forward Gentleman-Sande DIF, natural in, bit-reversed out
 * (scalar path of mul_ntt.cpp:193-255) */
static void orc_ntt_fwd(uint32_t *restrict a, size_t n, const orc_plan_t *p) {
    /* local copies: stores to a[] cannot alias them, so they stay in registers */
    const orc_mont_t c = p->c;
    const uint32_t *restrict fw = p->fw;
    const uint32_t mod = c.mod;
    for (size_t len = n; len >= 2; len >>= 1) {
        size_t half = len >> 1;
        for (size_t i = 0; i < n; i += len) {
            for (size_t j = 0; j < half; ++j) {
                uint32_t u = a[i + j], v = a[i + j + half];
                uint32_t s = u + v;
                if (s >= mod) s -= mod;
                uint32_t d = u >= v ? u - v : u + mod - v;
                a[i + j] = s;
                a[i + j + half] = orc_mmul(&c, d, fw[half + j]);
            }
        }
    }
}

/* inverse Cooley-Tukey DIT, bit-reversed in, natural out, times n^{-1}
 * (scalar path of mul_ntt.cpp:257-329) */
static void orc_ntt_inv(uint32_t *restrict a, size_t n, const orc_plan_t *p) {
    const orc_mont_t c = p->c;
    const uint32_t *restrict iv = p->iv;
    const uint32_t mod = c.mod;
    for (size_t len = 2; len <= n; len <<= 1) {
        size_t half = len >> 1;
        for (size_t i = 0; i < n; i += len) {
            for (size_t j = 0; j < half; ++j) {
                uint32_t u = a[i + j];
                uint32_t v = orc_mmul(&c, a[i + j + half], iv[half + j]);
                uint32_t s = u + v;
                if (s >= mod) s -= mod;
                uint32_t d = u >= v ? u - v : u + mod - v;
                a[i + j] = s;
                a[i + j + half] = d;
            }
        }
    }
    const uint32_t inv_n = p->inv_n;
    for (size_t i = 0; i < n; ++i) a[i] = orc_mmul(&c, a[i], inv_n);
}

/* ntt_digits (mul_ntt.cpp:331-342): limbs -> 16-bit digits, LSB first,
 * trailing zero digits trimmed.  Returns the digit count. */
static size_t orc_digits16(const uint64_t *a, size_t an, uint32_t *d) {
    size_t k = 0;
    for (size_t i = 0; i < an; ++i) {
        d[k++] = (uint32_t)(a[i] & 0xFFFFu);
        d[k++] = (uint32_t)((a[i] >> 16) & 0xFFFFu);
        d[k++] = (uint32_t)((a[i] >> 32) & 0xFFFFu);
        d[k++] = (uint32_t)(a[i] >> 48);
    }
    while (k > 0 && d[k - 1] == 0) --k;
    return k;
}

/* ntt_convolve_mod (mul_ntt.cpp:349-387): residues of the cyclic
 * convolution modulo one prime, written to out[0..n). */
static void orc_convolve(const uint32_t *da, size_t na, const uint32_t *db,
                         size_t nb, size_t n, int idx, uint32_t *out,
                         uint32_t *scratch) {
    const orc_plan_t *p = orc_get_plan(idx, n);
    const orc_mont_t c = p->c;
    memset(out, 0, n * sizeof(uint32_t));
    memset(scratch, 0, n * sizeof(uint32_t));
    for (size_t i = 0; i < na; ++i) out[i] = orc_to_mont(&c, da[i]);
    for (size_t i = 0; i < nb; ++i) scratch[i] = orc_to_mont(&c, db[i]);
    orc_ntt_fwd(out, n, p);
    orc_ntt_fwd(scratch, n, p);
    for (size_t i = 0; i < n; ++i) out[i] = orc_mmul(&c, out[i], scratch[i]);
    orc_ntt_inv(out, n, p);
    for (size_t i = 0; i < n; ++i) out[i] = orc_redc(&c, out[i]);
}

/* mod_inv_u32 (mul_ntt.cpp:389-403): extended Euclid */
static uint32_t orc_inv_mod(uint64_t a, uint32_t m) {
    int64_t t = 0, nt = 1, r = m, nr = (int64_t)(a % m);
    while (nr) {
        int64_t q = r / nr, tmp;
        tmp = t - q * nt; t = nt; nt = tmp;
        tmp = r - q * nr; r = nr; nr = tmp;
    }
    if (t < 0) t += m;
    return (uint32_t)t;
}

/* The CRT inverses, computed once (the reference keeps them in
 * function-local statics, mul_ntt.cpp:406, 416); set when the library is
 * loaded, before any thread calls in. */
static uint64_t orc_inv12, orc_inv123;
__attribute__((constructor)) static void orc_crt_init(void) {
    orc_inv12 = orc_inv_mod(ORC_MOD[0], ORC_MOD[1]);
    orc_inv123 = orc_inv_mod(((uint64_t)ORC_MOD[0] * ORC_MOD[1]) % ORC_MOD[2], ORC_MOD[2]);
}

/* Garner CRT for two primes (mul_ntt.cpp:405-412) */
static uint64_t orc_crt2(uint32_t r1, uint32_t r2) {
    const uint64_t m1 = ORC_MOD[0], m2 = ORC_MOD[1];
    const uint64_t inv = orc_inv12;
    uint64_t d = r2 >= r1 ? (uint64_t)r2 - r1 : (uint64_t)r2 + m2 - r1;
    return r1 + m1 * (d * inv % m2);
}

/* Garner CRT for three primes (mul_ntt.cpp:414-424); the result may exceed
 * 64 bits in general, so it is returned as 128 bits. */
static u128 orc_crt3(uint32_t r1, uint32_t r2, uint32_t r3) {
    const uint64_t m1 = ORC_MOD[0], m2 = ORC_MOD[1], m3 = ORC_MOD[2];
    uint64_t x12 = orc_crt2(r1, r2);
    const uint64_t inv = orc_inv123;
    uint64_t x12_m3 = x12 % m3;
    uint64_t d = r3 >= x12_m3 ? r3 - x12_m3 : r3 + m3 - x12_m3;
    return (u128)x12 + (u128)(m1 * m2) * (d * inv % m3);
}

/* ntt_from_residues2/3 (mul_ntt.cpp:426-487): CRT per digit, running carry
 * in base 2^16, packed into limbs.  `out` holds `cap` limbs. */
static void orc_from_residues(const uint32_t *r1, const uint32_t *r2,
                              const uint32_t *r3, size_t n, uint64_t *out,
                              size_t cap) {
    memset(out, 0, cap * sizeof(uint64_t));
    size_t id = 0;
    if (!r3) {
        /* two primes: a coefficient plus the carry stays below 2^64, as in
         * the reference's 64-bit loop (mul_ntt.cpp:438-445) */
        uint64_t c64 = 0;
        for (size_t i = 0; i < n; ++i, ++id) {
            uint64_t cur = orc_crt2(r1[i], r2[i]) + c64;
            if ((id >> 2) < cap) out[id >> 2] |= (cur & 0xFFFFu) << ((id & 3) * 16);
            c64 = cur >> 16;
        }
        for (; c64; c64 >>= 16, ++id)
            if ((id >> 2) < cap) out[id >> 2] |= (c64 & 0xFFFFu) << ((id & 3) * 16);
        return;
    }
    u128 carry = 0;
    for (size_t i = 0; i < n; ++i, ++id) {
        u128 cur = (r3 ? orc_crt3(r1[i], r2[i], r3[i]) : (u128)orc_crt2(r1[i], r2[i])) + carry;
        uint64_t digit = (uint64_t)(cur & 0xFFFFu);
        if ((id >> 2) < cap) out[id >> 2] |= digit << ((id & 3) * 16);
        carry = cur >> 16;
    }
    while (carry) {
        uint64_t digit = (uint64_t)(carry & 0xFFFFu);
        if ((id >> 2) < cap) out[id >> 2] |= digit << ((id & 3) * 16);
        carry >>= 16;
        ++id;
    }
}

size_t oracle_mul_fft(const uint64_t *a, size_t an, const uint64_t *b,
                      size_t bn, uint64_t *out, double *max_err);

/* mul_ntt (mul_ntt.cpp:494-518) including its guards. */
size_t oracle_mul_ntt(const uint64_t *a, size_t an, const uint64_t *b,
                      size_t bn, uint64_t *out) {
    size_t total = an + bn;
    size_t la = norm_len(a, an), lb = norm_len(b, bn);
    if (la == 0 || lb == 0) {
        memset(out, 0, total * sizeof(uint64_t));
        return 0;
    }
    size_t hi = la > lb ? la : lb;
    if (hi <= 192 || hi > ORC_MAX_LIMBS) {
        /* both fallbacks write la+lb limbs; clear the caller's tail first */
        memset(out, 0, total * sizeof(uint64_t));
        if (hi <= 192) oracle_mul_basic(a, la, b, lb, out);
        else oracle_mul_fft(a, la, b, lb, out, NULL);
        return norm_len(out, total);
    }

    uint32_t *da = (uint32_t *)xcalloc(4 * la, sizeof(uint32_t));
    uint32_t *db = (uint32_t *)xcalloc(4 * lb, sizeof(uint32_t));
    size_t na = orc_digits16(a, la, da), nb = orc_digits16(b, lb, db);
    size_t n = 1;
    while (n < na + nb) n <<= 1;
    if (n > ORC_MAX_TRANSFORM) {
        free(da);
        free(db);
        memset(out, 0, total * sizeof(uint64_t));
        oracle_mul_fft(a, la, b, lb, out, NULL);
        return norm_len(out, total);
    }
    uint32_t *r1 = (uint32_t *)xcalloc(n, 4), *r2 = (uint32_t *)xcalloc(n, 4);
    uint32_t *sc = (uint32_t *)xcalloc(n, 4);
    orc_convolve(da, na, db, nb, n, 0, r1, sc);
    orc_convolve(da, na, db, nb, n, 1, r2, sc);
    /* ntt_two_mod_ok (mul_ntt.cpp:489-492) */
    uint64_t m12 = (uint64_t)ORC_MOD[0] * ORC_MOD[1];
    size_t terms = na < nb ? na : nb;
    uint32_t *r3 = NULL;
    if (!(terms <= (m12 - 1) / (0xFFFFull * 0xFFFFull))) {
        r3 = (uint32_t *)xcalloc(n, 4);
        orc_convolve(da, na, db, nb, n, 2, r3, sc);
    }
    orc_from_residues(r1, r2, r3, n, out, total);
    free(da); free(db); free(r1); free(r2); free(r3); free(sc);
    return norm_len(out, total);
}

/* ------------------------------------------------------------------ */
/* FFT band: mul_fft (src/mul_fft.cpp)                                  */
/* ------------------------------------------------------------------ */

/* COUNT_FFTS statistics of the last oracle_mul_fft call
 * (mul_fft.cpp:32-38, 359-382). */
static double orc_last_fft_err = 0.0;
static int orc_last_fft_zone = 0; /* bit0 >1/8, bit1 >1/4, bit2 >3/8 */

double oracle_last_fft_error(void) { return orc_last_fft_err; }
int oracle_last_fft_zones(void) { return orc_last_fft_zone; }

/* fft_fill_roots (mul_fft.cpp:57-76): recurrence, re-anchored every 1024 */
static void orc_fill_roots(double *wr, double *wi, size_t half, double ang) {
    if (half == 0) return;
    double cr = cos(ang), ci = sin(ang);
    wr[0] = 1.0;
    wi[0] = 0.0;
    for (size_t i = 1; i < half; ++i) {
        if ((i & 1023) == 0) {
            wr[i] = cos(ang * (double)i);
            wi[i] = sin(ang * (double)i);
        } else {
            double r = wr[i - 1] * cr - wi[i - 1] * ci;
            double m = wr[i - 1] * ci + wi[i - 1] * cr;
            wr[i] = r;
            wi[i] = m;
        }
    }
}

/* fft (mul_fft.cpp:200-220) with fft_stage's scalar path (155-170) and
 * fft_scale (174-198).  Twiddles are generated per stage exactly as
 * fft_plan does (mul_fft.cpp:87-97). */
static void orc_fft(double *re, double *im, size_t n, int inv) {
    size_t bits = 0;
    while (((size_t)1 << bits) < n) ++bits;
    /* fft_build_rev (mul_fft.cpp:47-55) and the permutation (205-211) */
    size_t *rev = (size_t *)xcalloc(n, sizeof(size_t));
    for (size_t i = 1; i < n; ++i)
        rev[i] = (rev[i >> 1] >> 1) | ((i & 1) << (bits - 1));
    for (size_t i = 1; i < n; ++i) {
        size_t j = rev[i];
        if (i < j) {
            double t = re[i]; re[i] = re[j]; re[j] = t;
            t = im[i]; im[i] = im[j]; im[j] = t;
        }
    }
    free(rev);
    const double pi = acos(-1.0);
    double *wr = (double *)xcalloc(n, sizeof(double));
    double *wi = (double *)xcalloc(n, sizeof(double));
    for (size_t len = 2; len <= n; len <<= 1) {
        size_t half = len >> 1;
        orc_fill_roots(wr, wi, half, (inv ? -2.0 : 2.0) * pi / (double)len);
        for (size_t i = 0; i < n; i += len) {
            for (size_t j = 0; j < half; ++j) {
                size_t p = i + j, q = p + half;
                double br = re[q], bi = im[q];
                double vr = br * wr[j] - bi * wi[j];
                double vi = br * wi[j] + bi * wr[j];
                double ur = re[p], ui = im[p];
                re[p] = ur + vr;
                im[p] = ui + vi;
                re[q] = ur - vr;
                im[q] = ui - vi;
            }
        }
    }
    free(wr);
    free(wi);
    if (inv) {
        double s = 1.0 / (double)n;
        for (size_t i = 0; i < n; ++i) {
            re[i] *= s;
            im[i] *= s;
        }
    }
}

/* fft_digit_count (mul_fft.cpp:222-232) */
static size_t orc_fft_digit_count(const uint64_t *a, size_t an, int bits) {
    if (an == 0) return 0;
    size_t per = 64 / bits;
    size_t n = (an - 1) * per;
    uint64_t top = a[an - 1];
    do {
        ++n;
        top >>= bits;
    } while (top);
    return n;
}

/* fft_load_digits (mul_fft.cpp:234-246) */
static void orc_fft_load(double *dst, const uint64_t *a, size_t an, int bits) {
    uint64_t mask = ((uint64_t)1 << bits) - 1;
    size_t per = 64 / bits, k = 0;
    for (size_t i = 0; i < an; ++i) {
        uint64_t x = a[i];
        for (size_t j = 0; j < per; ++j) {
            dst[k++] = (double)(x & mask);
            x >>= bits;
        }
    }
}

/* mul_fft_bits (mul_fft.cpp:340-384) with fft_pair_convolution's scalar
 * path (290-304), fft_round (307-309) and fft_from_digits (311-338). */
static size_t orc_mul_fft_bits(const uint64_t *a, size_t an, const uint64_t *b,
                               size_t bn, int bits, uint64_t *out,
                               size_t cap) {
    memset(out, 0, cap * sizeof(uint64_t));
    size_t da = orc_fft_digit_count(a, an, bits);
    size_t db = orc_fft_digit_count(b, bn, bits);
    if (da == 0 || db == 0) return 0;
    size_t n = 1;
    while (n < da + db) n <<= 1;
    size_t per = 64 / bits;
    size_t alloc = n > an * per ? n : an * per;
    if (alloc < bn * per) alloc = bn * per;
    double *re = (double *)xcalloc(alloc, sizeof(double));
    double *im = (double *)xcalloc(alloc, sizeof(double));
    orc_fft_load(re, a, an, bits);
    orc_fft_load(im, b, bn, bits);
    orc_fft(re, im, n, 0);
    double *pr = (double *)xcalloc(n, sizeof(double));
    double *pi = (double *)xcalloc(n, sizeof(double));
    for (size_t k = 0; k < n; ++k) {
        size_t j = (n - k) & (n - 1);
        double xr = re[k], xi = im[k], yr = re[j], yi = im[j];
        double ar = (xr + yr) * 0.5;
        double ai = (xi - yi) * 0.5;
        double br = (xi + yi) * 0.5;
        double bi = (yr - xr) * 0.5;
        pr[k] = ar * br - ai * bi;
        pi[k] = ar * bi + ai * br;
    }
    orc_fft(pr, pi, n, 1);
    long long *d = (long long *)xcalloc(n + 8, sizeof(long long));
    double max_err = 0.0;
    int zones = 0;
    for (size_t i = 0; i < n; ++i) {
        double v = pr[i];
        double e = fabs(v - nearbyint(v));
        if (!isfinite(v)) e = INFINITY;
        if (e > max_err) max_err = e;
        if (e > 0.125) zones |= 1;
        if (e > 0.25) zones |= 2;
        if (e > 0.375) zones |= 4;
        d[i] = (long long)(v >= 0.0 ? v + 0.5 : v - 0.5);
    }
    orc_last_fft_err = max_err;
    orc_last_fft_zone = zones;
    /* signed carry in base 2^bits, then repack */
    long long mask = ((long long)1 << bits) - 1;
    long long carry = 0;
    size_t nd = n;
    for (size_t i = 0; i < nd; ++i) {
        long long cur = d[i] + carry;
        d[i] = cur & mask;
        carry = cur >> bits;
    }
    for (size_t i = 0; i < nd; ++i) {
        size_t limb = i / per;
        if (limb < cap) out[limb] |= (uint64_t)d[i] << ((i % per) * bits);
    }
    /* leftover carry digits beyond n (mul_fft.cpp:320-323) */
    size_t i = nd;
    while (carry) {
        size_t limb = i / per;
        if (limb < cap) out[limb] |= (uint64_t)(carry & mask) << ((i % per) * bits);
        carry >>= bits;
        ++i;
    }
    free(re); free(im); free(pr); free(pi); free(d);
    return norm_len(out, cap);
}

/* mul_fft (mul_fft.cpp:386-394): <=192 limbs schoolbook, <=1024 limbs
 * 16-bit digits, else 8-bit digits. */
size_t oracle_mul_fft(const uint64_t *a, size_t an, const uint64_t *b,
                      size_t bn, uint64_t *out, double *max_err) {
    size_t total = an + bn;
    size_t la = norm_len(a, an), lb = norm_len(b, bn);
    orc_last_fft_err = 0.0;
    orc_last_fft_zone = 0;
    size_t r;
    if (la == 0 || lb == 0) {
        memset(out, 0, total * sizeof(uint64_t));
        r = 0;
    } else {
        size_t hi = la > lb ? la : lb;
        if (hi <= 192) {
            oracle_mul_basic(a, la, b, lb, out);
            r = norm_len(out, total);
        } else {
            memset(out, 0, total * sizeof(uint64_t));
            r = orc_mul_fft_bits(a, la, b, lb, hi <= 1024 ? 16 : 8, out, total);
        }
    }
    if (max_err) *max_err = orc_last_fft_err;
    return r;
}

/* operator* dispatch for the two bands this library replaces
 * (src/mul_basic.cpp:238-276): squares (a == b by address) go to mul_fft
 * through precn_sqr (193-205); >6144 limbs -> NTT; >192 -> FFT. */
size_t oracle_mul(const uint64_t *a, size_t an, const uint64_t *b, size_t bn,
                  uint64_t *out) {
    size_t la = norm_len(a, an), lb = norm_len(b, bn);
    size_t hi = la > lb ? la : lb;
    if (hi > 6144) return oracle_mul_ntt(a, an, b, bn, out);
    if (hi > 192) return oracle_mul_fft(a, an, b, bn, out, NULL);
    return oracle_mul_basic(a, an, b, bn, out);
}

/* ------------------------------------------------------------------ */
/* spot checks and generators                                           */
/* ------------------------------------------------------------------ */

/* value of a limb vector modulo q (q < 2^63) */
uint64_t oracle_mod_u64(const uint64_t *a, size_t an, uint64_t q) {
    u128 r = 0;
    u128 base = ((u128)1 << 64) % q;
    for (size_t i = an; i > 0; --i) r = (r * base + a[i - 1] % q) % q;
    return (uint64_t)r;
}

/* SplitMix64 stream: out[i] = mix(seed + (i+1)*golden) */
void oracle_splitmix64(uint64_t seed, size_t n, uint64_t *out) {
    uint64_t s = seed;
    for (size_t i = 0; i < n; ++i) {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        out[i] = z ^ (z >> 31);
    }
}

/* 64-bit LCG pattern of test/bench_ntt.cpp:6-17 and
 * test/test_opt_smoke.cpp:8-19 (limb = x | 1). */
void oracle_lcg64_pattern(uint64_t seed, size_t n, uint64_t *out) {
    uint64_t x = seed;
    for (size_t i = 0; i < n; ++i) {
        x = x * 6364136223846793005ull + 1442695040888963407ull;
        out[i] = x | 1;
    }
}

/* 32-bit LCG pattern of test/test_prec.cpp:63-76 (limb = x | 1). */
void oracle_lcg32_pattern(uint32_t seed, size_t n, uint64_t *out) {
    uint32_t x = seed;
    for (size_t i = 0; i < n; ++i) {
        x = x * 1664525u + 1013904223u;
        out[i] = (uint64_t)(x | 1u);
    }
}
