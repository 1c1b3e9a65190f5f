// dnat.cu -- device-resident natural numbers and the Newton operations on
// them (see dnat.hpp).  The shifts are one kernel each; additions and
// subtractions run the chunked signed-add kernels of pi_kernels.cu on one
// pair; products go through prec_gpu_mul_device on the object's stream.
// Low precisions (a few thousand limbs) run bignum.cpp's host versions on a
// downloaded truncation of the operand and upload the result.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>

#include "../../include/prec_gpu.h"
#include "dnat.hpp"
#include "pi_device.hpp"

namespace precpi {

namespace {

// below this precision (bits) the Newton recursions run on the host
constexpr size_t kHostNewtonBits = (size_t)1 << 16;

[[noreturn]] void die_cuda(const char* what, cudaError_t e) {
    std::fprintf(stderr, "pi_gb300: device math: %s: %s\n", what, cudaGetErrorString(e));
    std::exit(3);
}
[[noreturn]] void die_lib(const char* what, int rc) {
    std::fprintf(stderr, "pi_gb300: device math: %s: %s\n", what, prec_gpu_strerror(rc));
    std::exit(3);
}
void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) die_cuda(what, e);
}

size_t limbs_for(size_t bits) { return (bits + 63) / 64; }

size_t bitlen64(u64 x) { return x ? 64 - (size_t)__builtin_clzll(x) : 0; }

__global__ void k_shr(u64* __restrict__ out, const u64* __restrict__ a, size_t na, size_t w, unsigned b,
                      size_t nout) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nout; i += (size_t)gridDim.x * blockDim.x) {
        const size_t j = i + w;
        u64 v = j < na ? a[j] >> b : 0;
        if (b && j + 1 < na) v |= a[j + 1] << (64 - b);
        out[i] = v;
    }
}

__global__ void k_shl(u64* __restrict__ out, const u64* __restrict__ a, size_t na, size_t w, unsigned b,
                      size_t nout) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nout; i += (size_t)gridDim.x * blockDim.x) {
        u64 v = 0;
        if (i >= w && i - w < na) v = a[i - w] << b;
        if (b && i >= w + 1 && i - w - 1 < na) v |= a[i - w - 1] >> (64 - b);
        out[i] = v;
    }
}

__global__ void k_set(u64* p, size_t n, size_t idx, u64 v) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        p[i] = i == idx ? v : 0;
}

// the highest limb index where a and b differ (a and b both n limbs); *top
// starts at -1
__global__ void k_top_differ(const u64* __restrict__ a, const u64* __restrict__ b, size_t n, long long* top) {
    long long best = -1;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        if (a[i] != b[i]) best = (long long)i;
    for (int o = 16; o > 0; o >>= 1) {
        const long long t = __shfl_xor_sync(0xffffffffu, best, o);
        best = t > best ? t : best;
    }
    if ((threadIdx.x & 31) == 0 && best >= 0) atomicMax(top, best);
}

// the highest nonzero limb index of p[0 .. n) (*top starts at -1)
__global__ void k_top_nonzero(const u64* __restrict__ p, size_t n, long long* top) {
    long long best = -1;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        if (p[i]) best = (long long)i;
    for (int o = 16; o > 0; o >>= 1) {
        const long long t = __shfl_xor_sync(0xffffffffu, best, o);
        best = t > best ? t : best;
    }
    if ((threadIdx.x & 31) == 0 && best >= 0) atomicMax(top, best);
}

// *out = {index, limb} of the highest nonzero limb (index -1: zero)
__global__ void k_top_limb(const u64* p, const long long* top, long long* out) {
    const long long t = *top;
    out[0] = t;
    out[1] = t < 0 ? 0 : (long long)p[t];
}

__global__ void k_cmp_sign(const u64* a, const u64* b, const long long* top, long long* sign) {
    const long long t = *top;
    *sign = t < 0 ? 0 : (a[t] > b[t] ? 1 : -1);
}

int grid_for(size_t n) { return (int)std::max<size_t>(1, std::min<size_t>((n + 255) / 256, 4096)); }

std::atomic<uint64_t> g_launches{0};

// device block of the math object: the pair descriptor, its three signs,
// the compare words
struct DevBlock {
    AddPair pair;
    int8_t sx, sy, sz, pad;
    long long top, sign;
    long long found[2];  // k_top_limb's result
};

}  // namespace

uint64_t dnat_launches() { return g_launches.load(std::memory_order_relaxed); }

DNat& DNat::operator=(DNat&& o) noexcept {
    if (this != &o) {
        if (d) cudaFreeAsync(d, st);
        d = o.d;
        n = o.n;
        bits = o.bits;
        st = o.st;
        o.d = nullptr;
        o.n = o.bits = 0;
    }
    return *this;
}

DNat::~DNat() {
    if (d) cudaFreeAsync(d, st);
}

DevMath::DevMath(cudaStream_t st) : st_(st) {
    // stream-ordered allocations come from the device's default pool; keep
    // freed memory in it (the Newton steps free and allocate numbers of the
    // same sizes over and over)
    int dev = 0;
    cudaMemPool_t pool = nullptr;
    ck(cudaGetDevice(&dev), "device");
    ck(cudaDeviceGetDefaultMemPool(&pool, dev), "memory pool");
    uint64_t keep = ~0ull;
    ck(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep), "memory pool");
    ck(cudaMallocHost(&h_top_, 4 * sizeof(u64)), "pinned read-back");
    ck(cudaMalloc(&dev_, sizeof(DevBlock)), "descriptor block");
}

DevMath::~DevMath() {
    cudaStreamSynchronize(st_);
    cudaFreeHost(h_top_);
    cudaFree(dev_);
    if (scratch_) cudaFree(scratch_);
}

DNat DevMath::alloc(size_t limbs) {
    DNat x;
    x.st = st_;
    x.n = limbs;
    ck(cudaMallocAsync(reinterpret_cast<void**>(&x.d), std::max<size_t>(limbs, 1) * sizeof(u64), st_), "alloc");
    return x;
}

void DevMath::fix_size(DNat& x, size_t limbs) {
    // the top two limbs of the first `limbs`; callers guarantee the number
    // is 0 or has one of its two highest limbs nonzero (a product)
    h_top_[0] = h_top_[1] = 0;
    const size_t lo = limbs >= 2 ? limbs - 2 : 0;
    if (limbs) ck(cudaMemcpyAsync(h_top_, x.d + lo, (limbs - lo) * sizeof(u64), cudaMemcpyDeviceToHost, st_), "top");
    ck(cudaStreamSynchronize(st_), "sync");
    ++syncs;
    const u64 t1 = limbs >= 2 ? h_top_[1] : h_top_[0];
    const u64 t0 = limbs >= 2 ? h_top_[0] : 0;
    if (t1) {
        x.n = limbs;
        x.bits = 64 * (limbs - 1) + bitlen64(t1);
    } else if (t0 && limbs >= 2) {
        x.n = limbs - 1;
        x.bits = 64 * (limbs - 2) + bitlen64(t0);
    } else {
        x.n = 0;
        x.bits = 0;
        if (limbs > 2) {
            std::fprintf(stderr, "pi_gb300: device math: result shorter than its two top limbs\n");
            std::exit(3);
        }
    }
}

DNat DevMath::upload(const Nat& x) {
    DNat r = alloc(x.size());
    if (x.size()) ck(cudaMemcpyAsync(r.d, x.d.data(), x.size() * sizeof(u64), cudaMemcpyHostToDevice, st_), "H2D");
    r.bits = bitlen(x);
    return r;
}

Nat DevMath::download(const DNat& x) {
    Nat r;
    r.d.resize(x.n);
    if (x.n) ck(cudaMemcpyAsync(r.d.data(), x.d, x.n * sizeof(u64), cudaMemcpyDeviceToHost, st_), "D2H");
    ck(cudaStreamSynchronize(st_), "sync");
    ++syncs;
    return r;
}

DNat DevMath::copy(const DNat& a) {
    DNat r = alloc(a.n);
    if (a.n) ck(cudaMemcpyAsync(r.d, a.d, a.n * sizeof(u64), cudaMemcpyDeviceToDevice, st_), "D2D");
    r.bits = a.bits;
    return r;
}

DNat DevMath::pow2(size_t bits) {
    DNat r = alloc(bits / 64 + 1);
    k_set<<<grid_for(r.n), 256, 0, st_>>>(r.d, r.n, bits / 64, 1ull << (bits % 64));
    g_launches.fetch_add(1, std::memory_order_relaxed);
    ck(cudaGetLastError(), "pow2");
    r.bits = bits + 1;
    return r;
}

DNat DevMath::shr(const DNat& a, size_t bits) {
    if (bits >= a.bits) return alloc(0);
    DNat r = alloc(limbs_for(a.bits - bits));
    k_shr<<<grid_for(r.n), 256, 0, st_>>>(r.d, a.d, a.n, bits / 64, (unsigned)(bits % 64), r.n);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    ck(cudaGetLastError(), "shr");
    r.bits = a.bits - bits;
    return r;
}

DNat DevMath::shl(const DNat& a, size_t bits) {
    if (a.zero()) return alloc(0);
    DNat r = alloc(limbs_for(a.bits + bits));
    k_shl<<<grid_for(r.n), 256, 0, st_>>>(r.d, a.d, a.n, bits / 64, (unsigned)(bits % 64), r.n);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    ck(cudaGetLastError(), "shl");
    r.bits = a.bits + bits;
    return r;
}

DNat DevMath::mul(const DNat& a, const DNat& b) {
    if (a.zero() || b.zero()) return alloc(0);
    DNat r = alloc(a.n + b.n);
    const int rc = prec_gpu_mul_device(a.d, a.n, b.d, b.n, r.d, st_);
    if (rc) die_lib("product", rc);
    ++products;
    fix_size(r, a.n + b.n);
    return r;
}

DNat DevMath::mul_u64(const DNat& a, u64 v) {
    Nat s(v);
    const DNat d = upload(s);
    return mul(a, d);
}

DNat DevMath::pow_u64(u64 base, size_t e) {
    if (e == 0) return upload(Nat(1));
    int top = 63;
    while (!((e >> top) & 1)) --top;
    DNat r = upload(Nat(base));
    for (int i = top - 1; i >= 0; --i) {
        r = sqr(r);
        if ((e >> i) & 1) r = mul_u64(r, base);
    }
    return r;
}

// (-1)^sa a + (-1)^sb b through the chunked signed-add kernels (sa, sb:
// 0 = +, 1 = -); the result's sign in *sign
DNat DevMath::signed_sum(const DNat& a, int sa, const DNat& b, int sb, int* sign) {
    const size_t nz = std::max(a.n, b.n) + 1;
    DNat z = alloc(nz);
    const size_t nch = add_chunks((uint32_t)nz);
    const size_t need = signed_add_scratch_bytes(1, nch) + 256 + nch * sizeof(uint32_t);
    if (need > scratch_cap_) {
        if (scratch_) {
            ck(cudaStreamSynchronize(st_), "sync");
            cudaFree(scratch_);
        }
        scratch_cap_ = need + need / 2;
        ck(cudaMalloc(&scratch_, scratch_cap_), "add scratch");
    }
    uint32_t* chunk_pair = reinterpret_cast<uint32_t*>(static_cast<char*>(scratch_) +
                                                       ((signed_add_scratch_bytes(1, nch) + 255) & ~(size_t)255));
    ck(cudaMemsetAsync(chunk_pair, 0, nch * sizeof(uint32_t), st_), "chunk table");
    DevBlock* blk = static_cast<DevBlock*>(dev_);
    DevBlock h{};
    h.pair.x = a.d;
    h.pair.y = b.d;
    h.pair.z = z.d;
    h.pair.sx = &blk->sx;
    h.pair.sy = &blk->sy;
    h.pair.sz = &blk->sz;
    h.pair.nx = (uint32_t)a.n;
    h.pair.ny = (uint32_t)b.n;
    h.pair.nz = (uint32_t)nz;
    h.pair.chunk0 = 0;
    h.sx = (int8_t)(sa ? -1 : 1);
    h.sy = (int8_t)(sb ? -1 : 1);
    // pageable source: the copy is staged before the call returns
    ck(cudaMemcpyAsync(blk, &h, sizeof(DevBlock), cudaMemcpyHostToDevice, st_), "pair");
    ck(signed_add_many(&blk->pair, 1, chunk_pair, nch, scratch_, st_), "signed add");
    // a difference may cancel any number of top limbs: scan for the length
    ck(cudaMemsetAsync(&blk->top, 0xFF, sizeof(long long), st_), "scan init");
    k_top_nonzero<<<grid_for(nz), 256, 0, st_>>>(z.d, nz, &blk->top);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    k_top_limb<<<1, 1, 0, st_>>>(z.d, &blk->top, blk->found);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    ck(cudaGetLastError(), "scan");
    ck(cudaMemcpyAsync(h_top_, blk->found, 2 * sizeof(long long), cudaMemcpyDeviceToHost, st_), "top");
    ck(cudaMemcpyAsync(reinterpret_cast<char*>(h_top_) + 2 * sizeof(u64), &blk->sz, 1, cudaMemcpyDeviceToHost, st_),
       "sign");
    ck(cudaStreamSynchronize(st_), "sync");
    ++syncs;
    const long long ti = (long long)h_top_[0];
    z.n = ti < 0 ? 0 : (size_t)ti + 1;
    z.bits = ti < 0 ? 0 : 64 * (size_t)ti + bitlen64(h_top_[1]);
    const int8_t s = *reinterpret_cast<const int8_t*>(reinterpret_cast<const char*>(h_top_) + 2 * sizeof(u64));
    if (sign) *sign = z.zero() ? 0 : (s < 0 ? -1 : 1);
    return z;
}

DNat DevMath::add(const DNat& a, const DNat& b) { return signed_sum(a, 0, b, 0, nullptr); }

DNat DevMath::sub(const DNat& a, const DNat& b) {
    int s = 0;
    DNat z = signed_sum(a, 0, b, 1, &s);
    if (s < 0) {
        std::fprintf(stderr, "pi_gb300: device math: negative difference\n");
        std::exit(3);
    }
    return z;
}

DNat DevMath::absdiff(const DNat& a, const DNat& b, int* sign) { return signed_sum(a, 0, b, 1, sign); }

int DevMath::cmp(const DNat& a, const DNat& b) {
    if (a.n != b.n) return a.n < b.n ? -1 : 1;
    if (a.n == 0) return 0;
    DevBlock* blk = static_cast<DevBlock*>(dev_);
    ck(cudaMemsetAsync(&blk->top, 0xFF, sizeof(long long), st_), "cmp init");
    k_top_differ<<<grid_for(a.n), 256, 0, st_>>>(a.d, b.d, a.n, &blk->top);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    k_cmp_sign<<<1, 1, 0, st_>>>(a.d, b.d, &blk->top, &blk->sign);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    ck(cudaGetLastError(), "cmp");
    ck(cudaMemcpyAsync(h_top_ + 3, &blk->sign, sizeof(long long), cudaMemcpyDeviceToHost, st_), "cmp sign");
    ck(cudaStreamSynchronize(st_), "sync");
    ++syncs;
    return (int)(long long)h_top_[3];
}

// bignum.cpp's recip: X with |X - 2^(bitlen(D) + p) / D| <= 4.  The result
// depends only on the top p + 64 bits of D, so the low precisions run on
// the host on that truncation.
DNat DevMath::recip(const DNat& D, size_t p) {
    const size_t n = D.bits;
    if (p <= kHostNewtonBits) {
        const size_t s = n > p + 64 ? n - (p + 64) : 0;
        const DNat dt = shr(D, s);
        const Nat x = precpi::recip(download(dt), p);
        return upload(x);
    }
    const size_t h = (p + 1) / 2 + 16;
    const DNat xh = recip(D, h);
    const size_t s = n > p + 64 ? n - (p + 64) : 0;  // D truncated to p + 64 bits
    const DNat dt = shr(D, s);
    const size_t np = n - s;
    DNat x0 = shl(xh, p - h);
    const DNat t = mul(dt, x0);
    const DNat one = pow2(np + p);
    int sg = 0;
    const DNat e = absdiff(t, one, &sg);
    const bool over = sg > 0;
    const size_t keep = p - h + 64, eb = e.bits;
    const size_t te = eb > keep ? eb - keep : 0;
    const DNat corr = shr(mul(x0, shr(e, te)), np + p - te);
    return over ? sub(x0, corr) : add(x0, corr);
}

void DevMath::divmod_recip(const DNat& N, const DNat& D, const DNat& X, size_t P, DNat* q, DNat* r) {
    if (cmp(N, D) < 0) {
        *q = alloc(0);
        *r = copy(N);
        return;
    }
    const size_t nn = N.bits, nd = D.bits;
    if (P < nn - nd + 2 + 32) {
        std::fprintf(stderr, "pi_gb300: device math: reciprocal precision below the quotient's size\n");
        std::exit(3);
    }
    const size_t s = nn > P + 64 ? nn - (P + 64) : 0;
    DNat qq = shr(mul(shr(N, s), X), nd + P - s);
    DNat qd = mul(qq, D);
    const DNat one = upload(Nat(1));
    int steps = 0;
    while (cmp(qd, N) > 0) {
        qq = sub(qq, one);
        qd = sub(qd, D);
        if (++steps > 8) {
            std::fprintf(stderr, "pi_gb300: device math: division estimate too large\n");
            std::exit(3);
        }
    }
    DNat rr = sub(N, qd);
    while (cmp(rr, D) >= 0) {
        qq = add(qq, one);
        rr = sub(rr, D);
        if (++steps > 8) {
            std::fprintf(stderr, "pi_gb300: device math: division estimate too small\n");
            std::exit(3);
        }
    }
    *q = std::move(qq);
    *r = std::move(rr);
}

// bignum.cpp's invsqrt: Y with |Y - 2^(e/2 + p) / sqrt(n)| <= 4 for even
// e >= bitlen(n).  Low precisions run on the host on n truncated by an even
// number of bits t to about p + 64 bits, with e - t (the same quotient up to
// a relative 2^-(p+63)).
DNat DevMath::invsqrt(const DNat& n, size_t e, size_t p) {
    const size_t L = n.bits;
    if (p <= kHostNewtonBits) {
        const size_t t = L > p + 64 ? (L - (p + 64)) & ~(size_t)1 : 0;
        const Nat nt = download(shr(n, t));
        return upload(precpi::invsqrt(nt, e - t, p));
    }
    const size_t h = (p + 1) / 2 + 16;
    const DNat yh = invsqrt(n, e, h);
    DNat y0 = shl(yh, p - h);
    // Y1 = Y0 + Y0 (2^(e+2p) - n Y0^2) / 2^(e+2p+1), n and Y0^2 truncated
    const size_t t = L > p + 64 ? L - (p + 64) : 0;
    const DNat y2 = sqr(y0);
    const size_t b2 = y2.bits;
    const size_t t2 = b2 > p + 64 ? b2 - (p + 64) : 0;
    const DNat w = mul(shr(n, t), shr(y2, t2));
    const DNat one = pow2(e + 2 * p - t - t2);
    int sg = 0;
    const DNat E = absdiff(w, one, &sg);
    const bool over = sg > 0;
    const size_t keep = p - h + 64, eb = E.bits;
    const size_t te = eb > keep ? eb - keep : 0;
    const DNat corr = shr(mul(y0, shr(E, te)), e + 2 * p + 1 - t - t2 - te);
    return over ? sub(y0, corr) : add(y0, corr);
}

DNat DevMath::isqrt(const DNat& n) {
    if (n.zero()) return alloc(0);
    const size_t L = n.bits;
    const size_t e = L + (L & 1);
    const size_t p = L / 2 + 64;
    const DNat y = invsqrt(n, e, p);
    const size_t t = L > p + 64 ? L - (p + 64) : 0;
    DNat s = shr(mul(shr(n, t), y), e / 2 + p - t);
    DNat S = sqr(s);
    const DNat one = upload(Nat(1));
    int steps = 0;
    while (cmp(S, n) > 0) {  // (s-1)^2 = s^2 - 2s + 1
        S = add(sub(S, shl(s, 1)), one);
        s = sub(s, one);
        if (++steps > 8) {
            std::fprintf(stderr, "pi_gb300: device math: square root estimate too large\n");
            std::exit(3);
        }
    }
    for (;;) {
        DNat T = add(add(S, shl(s, 1)), one);  // (s+1)^2
        if (cmp(T, n) > 0) break;
        S = std::move(T);
        s = add(s, one);
        if (++steps > 8) {
            std::fprintf(stderr, "pi_gb300: device math: square root estimate too small\n");
            std::exit(3);
        }
    }
    return s;
}

}  // namespace precpi
