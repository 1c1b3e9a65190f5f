// bignum.cpp -- see bignum.hpp.
//
// Newton methods follow the textbook fixed-point forms (R. Brent and
// P. Zimmermann, "Modern Computer Arithmetic", 2010, sections 3.4 and
// 3.5): each step doubles the precision of the previous approximation and
// works on operands truncated to the precision it needs, so the cost of a
// reciprocal or inverse square root is a small multiple of one product of
// the final size.  Exact results come from a final correction against the
// definition (q*D <= N < (q+1)*D, s^2 <= n < (s+1)^2).  Division by the
// fixed 10^19 in the decimal conversion uses a precomputed inverse
// (N. Moeller and T. Granlund, "Improved division by invariant integers",
// IEEE Trans. Computers 60, 2011).
#include "bignum.hpp"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <new>
#include <mutex>
#include <thread>

namespace precpi {

namespace {

MulBackend* g_be = nullptr;

[[noreturn]] void fail(const char* what) {
    std::fprintf(stderr, "pi: internal error: %s\n", what);
    std::abort();
}

}  // namespace

// Free big blocks by capacity.  A block starts with a 64-byte header that
// holds its capacity; a request takes the smallest free block of at least
// its size and at most half again as large.
namespace {
constexpr size_t kBigHeader = 64;
constexpr size_t kBigKeep = (size_t)8 << 30;  // free bytes kept at most
std::mutex g_big_mu;
std::multimap<size_t, char*> g_big_free;
size_t g_big_held = 0;
}  // namespace

void* big_alloc(size_t bytes) {
    {
        std::lock_guard<std::mutex> lk(g_big_mu);
        auto it = g_big_free.lower_bound(bytes);
        if (it != g_big_free.end() && it->first <= bytes + bytes / 2) {
            char* b = it->second;
            g_big_held -= it->first;
            g_big_free.erase(it);
            return b + kBigHeader;
        }
    }
    char* b = static_cast<char*>(std::malloc(bytes + kBigHeader));
    if (!b) throw std::bad_alloc();
    std::memcpy(b, &bytes, sizeof(bytes));
    return b + kBigHeader;
}

void big_free(void* p) noexcept {
    if (!p) return;
    char* b = static_cast<char*>(p) - kBigHeader;
    size_t cap;
    std::memcpy(&cap, b, sizeof(cap));
    {
        std::lock_guard<std::mutex> lk(g_big_mu);
        if (g_big_held + cap <= kBigKeep) {
            g_big_free.emplace(cap, b);
            g_big_held += cap;
            return;
        }
    }
    std::free(b);
}

void set_backend(MulBackend* be) { g_be = be; }

MulBackend& backend() {
    if (!g_be) fail("no multiply backend");
    return *g_be;
}

void parallel_for(size_t n, const std::function<void(size_t)>& fn) {
    unsigned T = std::max(1u, std::thread::hardware_concurrency());
    if (n < 2 || T == 1) {
        for (size_t i = 0; i < n; ++i) fn(i);
        return;
    }
    T = (unsigned)std::min<size_t>(T, n);
    std::atomic<size_t> next{0};
    std::vector<std::thread> th;
    th.reserve(T);
    for (unsigned t = 0; t < T; ++t)
        th.emplace_back([&] {
            for (size_t i; (i = next.fetch_add(1)) < n;) fn(i);
        });
    for (auto& x : th) x.join();
}

void normalize(Nat& x) {
    while (!x.d.empty() && x.d.back() == 0) x.d.pop_back();
}

int cmp(const Nat& a, const Nat& b) {
    if (a.size() != b.size()) return a.size() < b.size() ? -1 : 1;
    for (size_t i = a.size(); i-- > 0;)
        if (a.d[i] != b.d[i]) return a.d[i] < b.d[i] ? -1 : 1;
    return 0;
}

size_t bitlen(const Nat& a) {
    if (a.zero()) return 0;
    return 64 * (a.size() - 1) + (64 - (size_t)__builtin_clzll(a.d.back()));
}

void add_in(Nat& a, const Nat& b) {
    if (a.size() < b.size()) a.d.resize(b.size(), 0);
    u64 c = 0;
    size_t i = 0;
    for (; i < b.size(); ++i) {
        const u128 s = (u128)a.d[i] + b.d[i] + c;
        a.d[i] = (u64)s;
        c = (u64)(s >> 64);
    }
    for (; c && i < a.size(); ++i) {
        a.d[i] += 1;
        c = a.d[i] == 0;
    }
    if (c) a.d.push_back(1);
}

void sub_in(Nat& a, const Nat& b) {
    if (cmp(a, b) < 0) fail("subtraction below zero");
    u64 br = 0;
    size_t i = 0;
    for (; i < b.size(); ++i) {
        const u64 x = a.d[i], y = b.d[i];
        const u64 t = x - y - br;
        br = (x < y) || (x == y && br) ? 1 : 0;
        a.d[i] = t;
    }
    for (; br && i < a.size(); ++i) {
        br = a.d[i] == 0;
        a.d[i] -= 1;
    }
    normalize(a);
}

Nat add(const Nat& a, const Nat& b) {
    Nat r = a.size() >= b.size() ? a : b;
    add_in(r, a.size() >= b.size() ? b : a);
    return r;
}

Nat sub(const Nat& a, const Nat& b) {
    Nat r = a;
    sub_in(r, b);
    return r;
}

Nat shl(const Nat& a, size_t bits) {
    if (a.zero()) return a;
    const size_t w = bits / 64, s = bits % 64;
    Nat r;
    r.d.assign(a.size() + w + 1, 0);
    for (size_t i = 0; i < a.size(); ++i) {
        r.d[i + w] |= a.d[i] << s;
        if (s) r.d[i + w + 1] |= a.d[i] >> (64 - s);
    }
    normalize(r);
    return r;
}

Nat shr(const Nat& a, size_t bits) {
    const size_t w = bits / 64, s = bits % 64;
    if (w >= a.size()) return Nat();
    Nat r;
    r.d.resize(a.size() - w);
    for (size_t i = 0; i < r.size(); ++i) {
        u64 v = a.d[i + w] >> s;
        if (s && i + w + 1 < a.size()) v |= a.d[i + w + 1] << (64 - s);
        r.d[i] = v;
    }
    normalize(r);
    return r;
}

Nat pow2(size_t bits) {
    Nat r;
    r.d.assign(bits / 64 + 1, 0);
    r.d.back() = (u64)1 << (bits % 64);
    return r;
}

Nat mul_u64(const Nat& a, u64 b) {
    Nat r;
    if (a.zero() || b == 0) return r;
    r.d.resize(a.size() + 1);
    u64 c = 0;
    for (size_t i = 0; i < a.size(); ++i) {
        const u128 t = (u128)a.d[i] * b + c;
        r.d[i] = (u64)t;
        c = (u64)(t >> 64);
    }
    r.d[a.size()] = c;
    normalize(r);
    return r;
}

u64 divmod_u64(Nat& a, u64 b) {
    u128 rem = 0;
    for (size_t i = a.size(); i-- > 0;) {
        const u128 cur = (rem << 64) | a.d[i];
        a.d[i] = (u64)(cur / b);
        rem = cur % b;
    }
    normalize(a);
    return (u64)rem;
}

void mul_school(const u64* a, size_t an, const u64* b, size_t bn, u64* out) {
    std::memset(out, 0, (an + bn) * sizeof(u64));
    for (size_t i = 0; i < an; ++i) {
        u64 c = 0;
        const u64 ai = a[i];
        for (size_t j = 0; j < bn; ++j) {
            const u128 t = (u128)ai * b[j] + out[i + j] + c;
            out[i + j] = (u64)t;
            c = (u64)(t >> 64);
        }
        out[i + bn] = c;
    }
}

Nat mul(const Nat& a, const Nat& b) {
    Nat r;
    if (a.zero() || b.zero()) return r;
    backend().mul(a, b, r);
    return r;
}

Nat sqr(const Nat& a) { return mul(a, a); }

Nat pow_u64(u64 base, size_t e) {
    Nat r(1);
    if (e == 0) return r;
    int top = 63 - __builtin_clzll((unsigned long long)e);
    for (int i = top; i >= 0; --i) {
        r = sqr(r);
        if ((e >> i) & 1) r = mul_u64(r, base);
    }
    return r;
}

// ---------------------------------------------------------------------------
// Newton reciprocal and exact division
// ---------------------------------------------------------------------------

// top `bits` (<= 64) bits of a as an integer
static u64 top_bits(const Nat& a, size_t bits) {
    const size_t n = bitlen(a);
    const Nat t = shr(a, n - bits);
    return t.zero() ? 0 : t.d[0];
}

Nat recip(const Nat& D, size_t p) {
    if (D.zero()) fail("reciprocal of zero");
    const size_t n = bitlen(D);
    if (p <= 62) {
        const size_t tb = std::min<size_t>(n, 64);
        const u64 dt = top_bits(D, tb);
        const u128 x = ((u128)1 << (tb + p)) / dt;
        Nat r;
        r.d.push_back((u64)x);
        if (x >> 64) r.d.push_back((u64)(x >> 64));
        normalize(r);
        return r;
    }
    const size_t h = (p + 1) / 2 + 16;
    const Nat xh = recip(D, h);
    const size_t s = n > p + 64 ? n - (p + 64) : 0;  // D truncated to p + 64 bits
    const Nat dt = shr(D, s);
    const size_t np = n - s;
    const Nat x0 = shl(xh, p - h);
    const Nat t = mul(dt, x0);
    const Nat one = pow2(np + p);
    const bool over = cmp(t, one) > 0;
    const Nat e = over ? sub(t, one) : sub(one, t);
    const size_t keep = p - h + 64, eb = bitlen(e);
    const size_t te = eb > keep ? eb - keep : 0;
    const Nat corr = shr(mul(x0, shr(e, te)), np + p - te);
    return over ? sub(x0, corr) : add(x0, corr);
}

void divmod(const Nat& N, const Nat& D, Nat& q, Nat& r) {
    if (D.zero()) fail("division by zero");
    if (cmp(N, D) < 0) {
        q = Nat();
        r = N;
        return;
    }
    const size_t P = bitlen(N) - bitlen(D) + 2 + 32;
    divmod_recip(N, D, recip(D, P), P, q, r);
}

void divmod_recip(const Nat& N, const Nat& D, const Nat& X, size_t P, Nat& q, Nat& r) {
    if (D.zero()) fail("division by zero");
    if (cmp(N, D) < 0) {
        q = Nat();
        r = N;
        return;
    }
    const size_t nn = bitlen(N), nd = bitlen(D);
    if (P < nn - nd + 2 + 32) fail("reciprocal precision below the quotient's size");
    // X ~ 2^(nd + P) / D; N truncated to P + 64 bits
    const size_t s = nn > P + 64 ? nn - (P + 64) : 0;
    q = shr(mul(shr(N, s), X), nd + P - s);
    Nat qd = mul(q, D);
    int steps = 0;
    while (cmp(qd, N) > 0) {
        sub_in(q, Nat(1));
        sub_in(qd, D);
        if (++steps > 8) fail("division estimate too large");
    }
    r = sub(N, qd);
    while (cmp(r, D) >= 0) {
        add_in(q, Nat(1));
        sub_in(r, D);
        if (++steps > 8) fail("division estimate too small");
    }
}

// ---------------------------------------------------------------------------
// Newton inverse square root and integer square root
// ---------------------------------------------------------------------------

// Y with |Y - 2^(e/2 + p) / sqrt(n)| <= 4, for even e >= bitlen(n)
Nat invsqrt(const Nat& n, size_t e, size_t p) {
    const size_t L = bitlen(n);
    if (p <= 40) {
        const size_t sh = L > 56 ? ((L - 56 + 1) & ~(size_t)1) : 0;  // even shift
        const Nat m = shr(n, sh);
        const double md = (double)(m.zero() ? 0 : m.d[0]);
        const double y = std::ldexp(1.0 / std::sqrt(md), (int)(e / 2 + p - sh / 2));
        return Nat((u64)std::llround(y));
    }
    const size_t h = (p + 1) / 2 + 16;
    const Nat yh = invsqrt(n, e, h);
    const Nat y0 = shl(yh, p - h);
    // Y1 = Y0 + Y0 (2^(e+2p) - n Y0^2) / 2^(e+2p+1), n and Y0^2 truncated
    const size_t t = L > p + 64 ? L - (p + 64) : 0;
    const Nat y2 = sqr(y0);
    const size_t b2 = bitlen(y2);
    const size_t t2 = b2 > p + 64 ? b2 - (p + 64) : 0;
    const Nat w = mul(shr(n, t), shr(y2, t2));
    const Nat one = pow2(e + 2 * p - t - t2);
    const bool over = cmp(w, one) > 0;
    const Nat E = over ? sub(w, one) : sub(one, w);
    const size_t keep = p - h + 64, eb = bitlen(E);
    const size_t te = eb > keep ? eb - keep : 0;
    const Nat corr = shr(mul(y0, shr(E, te)), e + 2 * p + 1 - t - t2 - te);
    return over ? sub(y0, corr) : add(y0, corr);
}

Nat isqrt(const Nat& n) {
    if (n.zero()) return n;
    const size_t L = bitlen(n);
    const size_t e = L + (L & 1);
    const size_t p = L / 2 + 64;
    const Nat y = invsqrt(n, e, p);
    const size_t t = L > p + 64 ? L - (p + 64) : 0;
    Nat s = shr(mul(shr(n, t), y), e / 2 + p - t);
    Nat S = sqr(s);
    int steps = 0;
    while (cmp(S, n) > 0) {  // (s-1)^2 = s^2 - 2s + 1
        sub_in(S, shl(s, 1));
        add_in(S, Nat(1));
        sub_in(s, Nat(1));
        if (++steps > 8) fail("square root estimate too large");
    }
    for (;;) {
        Nat T = add(S, shl(s, 1));
        add_in(T, Nat(1));  // (s+1)^2
        if (cmp(T, n) > 0) break;
        S = std::move(T);
        add_in(s, Nat(1));
        if (++steps > 8) fail("square root estimate too small");
    }
    return s;
}

// ---------------------------------------------------------------------------
// Decimal conversion
// ---------------------------------------------------------------------------

namespace {

constexpr u64 kTen19 = 10000000000000000000ull;  // 10^19 >= 2^63: a normalized divisor
constexpr size_t kLeafDigits = kDecimalLeafDigits;  // digits converted per leaf

// a /= 10^19 in place, returns the remainder (2-by-1 division with the
// precomputed inverse v = floor((2^128 - 1) / d) - 2^64)
u64 divmod_ten19(Nat& a) {
    static const u64 v = (u64)(~(u128)0 / kTen19 - ((u128)1 << 64));
    u64 r = 0;
    for (size_t i = a.size(); i-- > 0;) {
        const u64 u0 = a.d[i];
        const u128 qq = (u128)v * r + (((u128)r << 64) | u0);
        u64 q1 = (u64)(qq >> 64) + 1;
        const u64 q0 = (u64)qq;
        u64 rr = u0 - q1 * kTen19;
        if (rr > q0) {
            q1 -= 1;
            rr += kTen19;
        }
        if (rr >= kTen19) {
            q1 += 1;
            rr -= kTen19;
        }
        a.d[i] = q1;
        r = rr;
    }
    normalize(a);
    return r;
}

// exactly kLeafDigits digits of v < 10^kLeafDigits into out
void leaf_digits(Nat v, char* out) {
    std::memset(out, '0', kLeafDigits);
    long pos = (long)kLeafDigits;
    while (!v.zero()) {
        u64 r = divmod_ten19(v);
        for (int k = 0; k < 19 && pos > 0; ++k) {
            out[--pos] = (char)('0' + r % 10);
            r /= 10;
        }
    }
}

}  // namespace

static double tnow() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int decimal_levels(size_t digits) {
    int J = 0;
    while ((kLeafDigits << J) < digits) ++J;
    return J;
}

DecimalPowers decimal_powers(int levels) {
    DecimalPowers d;
    for (int j = 0; j < levels; ++j) {
        d.pw.push_back(j == 0 ? pow_u64(10, kLeafDigits) : sqr(d.pw[j - 1]));
        d.P.push_back(bitlen(d.pw[j]) + 2 + 32);
        d.rx.push_back(recip(d.pw[j], d.P[j]));
    }
    return d;
}

std::string to_decimal(const Nat& x, size_t width, const DecimalPowers* pre) {
    static const bool trace = std::getenv("PI_GB300_TRACE") != nullptr;
    double t0 = tnow();
    // digits of x are at most floor(bitlen * log10(2)) + 1
    const size_t need = std::max<size_t>(width, (size_t)((double)bitlen(x) * 0.30102999566398120) + 2);
    const int J = decimal_levels(need);
    // powers 10^(kLeafDigits * 2^j), j < J, and their reciprocals
    DecimalPowers own;
    if (!pre || (int)pre->pw.size() < J) {
        own = decimal_powers(J);
        pre = &own;
    }
    if (trace) std::fprintf(stderr, "  to_decimal: %d powers %.3f s\n", J, tnow() - t0);
    std::vector<Nat> pieces{x};
    for (int j = J - 1; j >= 0; --j) {
        const double tl = tnow();
        const Nat& D = pre->pw[j];
        const size_t nd = bitlen(D), P = pre->P[j];
        const Nat& X = pre->rx[j];
        const double tr = tnow();
        const size_t m = pieces.size();
        std::vector<Nat> qs(m), rs(m);
        // quotient estimates of every piece in one batch
        std::vector<Nat> nts(m);
        std::vector<size_t> sh(m, 0);
        std::vector<const Nat*> A, B;
        std::vector<size_t> idx;
        for (size_t i = 0; i < m; ++i) {
            if (cmp(pieces[i], D) < 0) continue;
            const size_t nn = bitlen(pieces[i]);
            sh[i] = nn > P + 64 ? nn - (P + 64) : 0;
            nts[i] = shr(pieces[i], sh[i]);
        }
        for (size_t i = 0; i < m; ++i) {
            if (cmp(pieces[i], D) < 0) continue;
            A.push_back(&nts[i]);
            B.push_back(&X);
            idx.push_back(i);
        }
        std::vector<Nat> prod;
        backend().mul_many(A, B, prod);
        for (size_t u = 0; u < idx.size(); ++u) qs[idx[u]] = shr(prod[u], nd + P - sh[idx[u]]);
        // q * D in one batch, then the exact corrections
        A.clear();
        B.clear();
        for (size_t u = 0; u < idx.size(); ++u) {
            A.push_back(&qs[idx[u]]);
            B.push_back(&D);
        }
        backend().mul_many(A, B, prod);
        std::vector<Nat> qd(m);
        for (size_t u = 0; u < idx.size(); ++u) qd[idx[u]] = std::move(prod[u]);
        parallel_for(m, [&](size_t i) {
            if (cmp(pieces[i], D) < 0) {
                rs[i] = pieces[i];
                return;
            }
            Nat& q = qs[i];
            Nat& t = qd[i];
            int steps = 0;
            while (cmp(t, pieces[i]) > 0) {
                sub_in(q, Nat(1));
                sub_in(t, D);
                if (++steps > 8) fail("decimal split estimate too large");
            }
            rs[i] = sub(pieces[i], t);
            while (cmp(rs[i], D) >= 0) {
                add_in(q, Nat(1));
                sub_in(rs[i], D);
                if (++steps > 8) fail("decimal split estimate too small");
            }
        });
        std::vector<Nat> next(2 * m);
        for (size_t i = 0; i < m; ++i) {
            next[2 * i] = std::move(qs[i]);
            next[2 * i + 1] = std::move(rs[i]);
        }
        pieces.swap(next);
        if (trace)
            std::fprintf(stderr, "  to_decimal level %d: %zu pieces, reciprocal %.3f s, splits %.3f s\n", j, m, tr - tl,
                         tnow() - tr);
    }
    const double tleaf = tnow();
    std::string s(pieces.size() * kLeafDigits, '0');
    parallel_for(pieces.size(), [&](size_t i) { leaf_digits(pieces[i], &s[i * kLeafDigits]); });
    if (trace) std::fprintf(stderr, "  to_decimal leaves: %.3f s\n", tnow() - tleaf);
    size_t first = s.find_first_not_of('0');
    if (first == std::string::npos) first = s.size() - 1;  // x == 0: "0"
    const size_t keep = std::max(width, s.size() - first);
    return s.substr(s.size() - keep);
}

}  // namespace precpi
