// ddec.cu -- decimal conversion of a device-resident number (DevMath::
// to_decimal) and its powers of ten (DevMath::decimal_powers).
//
// The algorithm is bignum.cpp's: divide and conquer on D_j = 10^(L 2^j)
// down to leaves below 10^L, each split a quotient estimate from the
// reciprocal X_j followed by an exact correction.  Here every piece of a
// level lives in one device buffer at a fixed stride, and the level runs as
// a fixed sequence on the object's stream:
//   1. nt = x >> sh for every piece (one kernel; sh = 2 nd - (P + 64) for all
//      pieces, nd = bitlen(D), P = nd + 34);
//   2. nt * X for every piece (one prec_gpu_mul_batch);
//   3. q = (nt X) >> (nd + P - sh) (one kernel);
//   4. q * D (one batch);
//   5. r0 = x - q D, then u = r0 - D (r0 >= 0) or u = r0 + D (r0 < 0), both
//      by signed_add_many over all pieces, the second pass's sign of D
//      chosen on the device from the first pass's sign;
//   6. one kernel writes (q - 1, u) where r0 < 0, (q + 1, u) where u >= 0,
//      else (q, r0) into the next level's pieces.
// Pieces below D_j^2 give |q_est - x / D| < 2^-31 (|X - 2^(nd+P)/D| <= 4, and
// the shift drops below 2^-97 of x / D), so q_est is within one of the
// quotient and step 6 is the whole correction.  The leaves are converted by
// one kernel (a thread per leaf, repeated 2-by-1 division by 10^19 with a
// precomputed inverse, Moeller and Granlund 2011), and the digit text is the
// only thing that comes back.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/prec_gpu.h"
#include "dnat.hpp"
#include "pi_device.hpp"

namespace precpi {

namespace {

constexpr u64 kTen19 = 10000000000000000000ull;
// limbs that hold any number below 10^L (bitlen <= ceil(L log2 10))
constexpr size_t kLeafLimbs = (size_t)((double)kDecimalLeafDigits * 3.3219280948873623 / 64.0) + 2;
static_assert(kDecimalLeafDigits % 8 == 0, "leaves are written in 8-byte words");

[[noreturn]] void dec_die(const char* what, const char* detail) {
    std::fprintf(stderr, "pi_gb300: device decimal conversion: %s%s%s\n", what, detail ? ": " : "", detail ? detail : "");
    std::exit(3);
}
void dec_ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) dec_die(what, cudaGetErrorString(e));
}

size_t lim(size_t bits) { return (bits + 63) / 64; }

unsigned grid_of(size_t n) { return (unsigned)std::max<size_t>(1, std::min<size_t>((n + 255) / 256, 8192)); }

// out[i * os + t] = bits of piece i (in[i * is ..], in_n limbs) from bit
// 64 w + b up, t < on, for i < m
__global__ void k_shr_many(u64* __restrict__ out, size_t os, size_t on, const u64* __restrict__ in, size_t is,
                           size_t in_n, size_t m, size_t w, unsigned b) {
    const size_t total = m * on;
    for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < total; g += (size_t)gridDim.x * blockDim.x) {
        const size_t i = g / on, t = g - i * on;
        const u64* a = in + i * is;
        const size_t j = t + w;
        u64 v = j < in_n ? a[j] >> b : 0;
        if (b && j + 1 < in_n) v |= a[j + 1] << (64 - b);
        out[i * os + t] = v;
    }
}

// the second pass subtracts D where r0 >= 0 and adds it where r0 < 0
__global__ void k_flip(int8_t* __restrict__ s2, const int8_t* __restrict__ sz, size_t m) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < m; i += (size_t)gridDim.x * blockDim.x)
        s2[i] = sz[i] < 0 ? 1 : -1;
}

// next-level pieces 2i (quotient) and 2i+1 (remainder), stride so:
// remainder u where r0 < 0 or u >= 0, else r0; the quotient copied here and
// moved by one in k_qfix
__global__ void k_select(u64* __restrict__ out, size_t so, const u64* __restrict__ q, size_t nq,
                         const u64* __restrict__ r0, size_t nr, const u64* __restrict__ u, size_t nu,
                         const int8_t* __restrict__ sz, const int8_t* __restrict__ su, size_t m, size_t nD) {
    const size_t total = m * so;
    for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < total; g += (size_t)gridDim.x * blockDim.x) {
        const size_t i = g / so, t = g - i * so;
        const bool use_u = sz[i] < 0 || su[i] >= 0;
        out[2 * i * so + t] = t < nq ? q[i * nq + t] : 0;
        out[(2 * i + 1) * so + t] = t < nD ? (use_u ? u[i * nu + t] : r0[i * nr + t]) : 0;
    }
}

// quotient i: -1 where r0 < 0, +1 where u >= 0 (the borrow or carry runs
// through the piece's limbs; almost always one)
__global__ void k_qfix(u64* __restrict__ out, size_t so, const int8_t* __restrict__ sz,
                       const int8_t* __restrict__ su, size_t m) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < m; i += (size_t)gridDim.x * blockDim.x) {
        const int d = sz[i] < 0 ? -1 : (su[i] >= 0 ? 1 : 0);
        if (!d) continue;
        u64* q = out + 2 * i * so;
        for (size_t t = 0; t < so; ++t) {
            const u64 old = q[t];
            q[t] = d > 0 ? old + 1 : old - 1;
            if (d > 0 ? old != ~0ull : old != 0) break;
        }
    }
}

// a /= 10^19 over a[0 .. n), returns the remainder (2-by-1 division with the
// precomputed inverse v = floor((2^128 - 1) / 10^19) - 2^64)
__device__ __forceinline__ u64 div_ten19(u64* a, int n) {
    const u64 v = (u64)(~(unsigned __int128)0 / kTen19 - ((unsigned __int128)1 << 64));
    u64 r = 0;
    for (int i = n - 1; i >= 0; --i) {
        const u64 u0 = a[i];
        const unsigned __int128 qq = (unsigned __int128)v * r + (((unsigned __int128)r << 64) | u0);
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
        a[i] = q1;
        r = rr;
    }
    return r;
}

// leaf i (kLeafLimbs limbs, below 10^L) as exactly L digits at out + i L
__global__ void __launch_bounds__(128) k_leaves(char* __restrict__ out, const u64* __restrict__ pieces,
                                                size_t nleaves) {
    constexpr int L = (int)kDecimalLeafDigits;
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= nleaves) return;
    u64 v[kLeafLimbs];
    int n = 0;
    for (int t = 0; t < (int)kLeafLimbs; ++t) {
        v[t] = pieces[i * kLeafLimbs + t];
        if (v[t]) n = t + 1;
    }
    alignas(16) char buf[L];
    int pos = L;
    while (n > 0 && pos > 0) {
        u64 r = div_ten19(v, n);
        while (n > 0 && v[n - 1] == 0) --n;
        for (int k = 0; k < 19 && pos > 0; ++k) {
            buf[--pos] = (char)('0' + r % 10);
            r /= 10;
        }
    }
    while (pos > 0) buf[--pos] = '0';
    u64* o = reinterpret_cast<u64*>(out + i * (size_t)L);
    const u64* b = reinterpret_cast<const u64*>(buf);
    for (int k = 0; k < L / 8; ++k) o[k] = b[k];
}

}  // namespace

DevDecimalPowers DevMath::decimal_powers(int levels) {
    DevDecimalPowers d;
    for (int j = 0; j < levels; ++j) {
        d.pw.push_back(j == 0 ? pow_u64(10, kDecimalLeafDigits) : sqr(d.pw[j - 1]));
        d.P.push_back(d.pw[j].bits + 2 + 32);
        d.rx.push_back(recip(d.pw[j], d.P[j]));
    }
    return d;
}

void DevMath::adopt(DevDecimalPowers& p) {
    for (DNat& x : p.pw) adopt(x);
    for (DNat& x : p.rx) adopt(x);
}

std::string DevMath::to_decimal(const DNat& x, const DevDecimalPowers& pw) {
    if (x.zero()) return "0";
    // digits of x are at most floor(bitlen log10 2) + 1
    const size_t need = (size_t)((double)x.bits * 0.30102999566398120) + 2;
    const int J = decimal_levels(need);
    if ((int)pw.pw.size() < J) dec_die("too few powers of ten", nullptr);
    // the top level's one piece: x, zero-extended to the level's stride
    size_t sin = J ? std::max(2 * pw.pw[J - 1].n, x.n) : kLeafLimbs;
    if (!J && x.n > kLeafLimbs) dec_die("number above its leaf", nullptr);
    DNat cur = alloc(sin);
    dec_ck(cudaMemsetAsync(cur.d, 0, sin * sizeof(u64), st_), "piece");
    dec_ck(cudaMemcpyAsync(cur.d, x.d, x.n * sizeof(u64), cudaMemcpyDeviceToDevice, st_), "piece");
    for (int j = J - 1; j >= 0; --j) {
        const size_t m = (size_t)1 << (J - 1 - j);
        const DNat& D = pw.pw[j];
        const DNat& X = pw.rx[j];
        const size_t nD = D.n, nd = D.bits, P = pw.P[j], nX = X.n;
        const size_t so = j ? 2 * pw.pw[j - 1].n : kLeafLimbs;  // the next level's stride
        if (so < nD || 2 * nd < P + 64) dec_die("level layout", nullptr);
        const size_t sh = 2 * nd - (P + 64);
        // 1-2: quotient estimates
        const size_t nnt = lim(P + 64), nprod = nnt + nX;
        DNat nt = alloc(m * nnt), prod = alloc(m * nprod);
        k_shr_many<<<grid_of(m * nnt), 256, 0, st_>>>(nt.d, nnt, nnt, cur.d, sin, sin, m, sh / 64, (unsigned)(sh % 64));
        std::vector<prec_gpu_product_t> items(m);
        for (size_t i = 0; i < m; ++i) items[i] = {nt.d + i * nnt, nnt, X.d, nX, prod.d + i * nprod};
        int rc = prec_gpu_mul_batch(items.data(), m, st_);
        if (rc) dec_die("quotient estimates", prec_gpu_strerror(rc));
        products += m;
        // 3-4: q and q D
        const size_t s2 = nd + P - sh, nq = nD + 1, nqd = nq + nD;
        DNat qb = alloc(m * nq), qd = alloc(m * nqd);
        k_shr_many<<<grid_of(m * nq), 256, 0, st_>>>(qb.d, nq, nq, prod.d, nprod, nprod, m, s2 / 64, (unsigned)(s2 % 64));
        for (size_t i = 0; i < m; ++i) items[i] = {qb.d + i * nq, nq, D.d, nD, qd.d + i * nqd};
        rc = prec_gpu_mul_batch(items.data(), m, st_);
        if (rc) dec_die("quotient times divisor", prec_gpu_strerror(rc));
        products += m;
        nt = DNat();
        prod = DNat();
        // 5: r0 = x - q D and u = r0 -/+ D, as two passes over all pieces
        const size_t nr = std::max(sin, nqd) + 1, nu = nr + 1;
        DNat r0 = alloc(m * nr), u = alloc(m * nu);
        // signs: [0] +1, [1] -1, then sz[m], s2[m], su[m]
        DNat signs = alloc((2 + 3 * m + 7) / 8);
        int8_t* sg = reinterpret_cast<int8_t*>(signs.d);
        int8_t* sz = sg + 2;
        int8_t* s2v = sz + m;
        int8_t* su = s2v + m;
        const int8_t pm[2] = {1, -1};
        dec_ck(cudaMemcpyAsync(sg, pm, 2, cudaMemcpyHostToDevice, st_), "signs");
        for (int pass = 0; pass < 2; ++pass) {
            const size_t nz = pass ? nu : nr;
            const size_t per = add_chunks((uint32_t)nz), nch = m * per;
            std::vector<AddPair> pairs(m);
            std::vector<uint32_t> chunk_pair(nch);
            for (size_t i = 0; i < m; ++i) {
                AddPair& a = pairs[i];
                if (!pass) {
                    a.x = cur.d + i * sin, a.nx = (uint32_t)sin, a.sx = sg;
                    a.y = qd.d + i * nqd, a.ny = (uint32_t)nqd, a.sy = sg + 1;
                    a.z = r0.d + i * nr, a.sz = sz + i;
                } else {
                    a.x = r0.d + i * nr, a.nx = (uint32_t)nr, a.sx = sz + i;
                    a.y = D.d, a.ny = (uint32_t)nD, a.sy = s2v + i;
                    a.z = u.d + i * nu, a.sz = su + i;
                }
                a.nz = (uint32_t)nz;
                a.chunk0 = (uint32_t)(i * per);
                for (size_t c = 0; c < per; ++c) chunk_pair[i * per + c] = (uint32_t)i;
            }
            const size_t sb = (signed_add_scratch_bytes(m, nch) + 255) & ~(size_t)255;
            const size_t pb = (m * sizeof(AddPair) + 255) & ~(size_t)255;
            DNat work = alloc((sb + pb + nch * sizeof(uint32_t) + 7) / 8);
            char* base = reinterpret_cast<char*>(work.d);
            AddPair* d_pairs = reinterpret_cast<AddPair*>(base + sb);
            uint32_t* d_chunks = reinterpret_cast<uint32_t*>(base + sb + pb);
            // pageable sources: staged before each call returns
            dec_ck(cudaMemcpyAsync(d_pairs, pairs.data(), m * sizeof(AddPair), cudaMemcpyHostToDevice, st_), "pairs");
            dec_ck(cudaMemcpyAsync(d_chunks, chunk_pair.data(), nch * sizeof(uint32_t), cudaMemcpyHostToDevice, st_),
                   "chunk table");
            if (pass) {
                k_flip<<<grid_of(m), 256, 0, st_>>>(s2v, sz, m);
                dec_ck(cudaGetLastError(), "signs");
            }
            dec_ck(signed_add_many(d_pairs, m, d_chunks, nch, base, st_), "signed sums");
            // the work block is freed in stream order after the kernels
        }
        // 6: the next level's pieces
        DNat next = alloc(2 * m * so);
        k_select<<<grid_of(m * so), 256, 0, st_>>>(next.d, so, qb.d, nq, r0.d, nr, u.d, nu, sz, su, m, nD);
        k_qfix<<<grid_of(m), 256, 0, st_>>>(next.d, so, sz, su, m);
        dec_ck(cudaGetLastError(), "level");
        cur = std::move(next);
        sin = so;
    }
    // leaves: 2^J pieces of kLeafLimbs limbs, L digits each
    const size_t nleaves = (size_t)1 << J;
    const size_t total = nleaves * kDecimalLeafDigits;
    DNat text = alloc((total + 7) / 8);
    k_leaves<<<(unsigned)((nleaves + 127) / 128), 128, 0, st_>>>(reinterpret_cast<char*>(text.d), cur.d, nleaves);
    dec_ck(cudaGetLastError(), "leaves");
    const size_t keep = std::min(total, need);
    std::string s(keep, '0');
    dec_ck(cudaMemcpyAsync(&s[0], reinterpret_cast<const char*>(text.d) + (total - keep), keep, cudaMemcpyDeviceToHost,
                           st_),
           "digits");
    dec_ck(cudaStreamSynchronize(st_), "digits");
    ++syncs;
    const size_t first = s.find_first_not_of('0');
    return first == std::string::npos ? std::string("0") : s.substr(first);
}

}  // namespace precpi
