// pi_chudnovsky.cpp -- pi by the Chudnovsky series on the GB300 multiply.
//
//   pi_gb300 DIGITS [--phases] [--full] [--file PATH]
//   pi_gb300 --self-check
//
// Same computation and output as preclib's pi/pi_chudnovsky.cpp (same
// guard digits, term count, scaled square root, floor divisions, decimal
// text and file format: "3.<DIGITS digits>\n"), so the digits are
// byte-identical.  What differs is the order of work:
//   * binary splitting runs level by level over the whole term range
//     instead of depth first (pi_chudnovsky.cpp:117-148): every level's
//     products (Q = Ql*Qr, T terms Tl*Qr and Tr*Pl, P = Pl*Pr where a later
//     level needs it) are independent and go to the GPU as one batch
//     (prec_gpu_mul_batch); the node values are shape independent
//     (T(a,b) = sum_k t_k P(a,k) Q(k+1,b)), so any tree gives the same Q, T;
//   * the square root and the final division run their Newton iterations
//     on numbers resident in device memory (dnat.cu): products through
//     prec_gpu_mul_device, shifts, additions and comparisons as device
//     kernels, only the operands in and the quotient out crossing the link
//     (PI_GB300_HOST_NEWTON=1: the host-resident iterations of bignum.cpp,
//     every product staged through host memory, for comparison);
//   * the decimal conversion runs Newton divisions whose products go to the
//     GPU (bignum.cpp), its splits as one batch per level;
//   * the square root and the conversion's powers of ten (with their
//     reciprocals) depend only on the digit count, so a second host thread
//     computes them while the binary splitting and the division run.
// The tree's five lowest levels (blocks of 32 terms, products of at most
// about 66 limbs) and any other product of at most kHostMaxLimbs limbs run
// on the host threads, as the reference multiplies such sizes with its
// schoolbook and Karatsuba code; everything larger is computed by
// libprecgpu.  There is no CPU path for those: without a device the
// program stops.  PI_GB300_TRACE=1 prints the time of every level.  The
// reported `time` runs from the start of main's work to the finished digits:
// the library's start-up (on its own thread, beside the tree's bottom blocks
// on the host threads) is inside it.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#ifdef __GLIBC__
#include <malloc.h>
#endif
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <future>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/prec_gpu.h"
#include "bignum.hpp"
#include "dnat.hpp"
#include "pi_device.hpp"

using namespace precpi;

#ifndef PI_HOST_MAX_LIMBS
#define PI_HOST_MAX_LIMBS 48
#endif

namespace {

constexpr u64 kC3Over24 = 10939058860032000ull;  // 640320^3 / 24
constexpr u64 kA = 13591409ull;
constexpr u64 kB = 545140134ull;
constexpr size_t kHostMaxLimbs = PI_HOST_MAX_LIMBS;  // products up to this size stay on the host

double now_sec() {
    static const auto t0 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

[[noreturn]] void die(const char* what, int rc) {
    std::fprintf(stderr, "pi_gb300: %s: %s\n", what, prec_gpu_strerror(rc));
    std::exit(1);
}

void check_cuda(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        std::fprintf(stderr, "pi_gb300: %s: %s\n", what, cudaGetErrorString(e));
        std::exit(1);
    }
}

// ---------------------------------------------------------------------------
// multiply backend on libprecgpu
// ---------------------------------------------------------------------------

// device-math work of the Newton steps (summary line of --phases)
static std::mutex g_dm_mu;
static size_t g_dm_products = 0, g_dm_syncs = 0;
static void dm_stats_add(const DevMath& dm) {
    std::lock_guard<std::mutex> lk(g_dm_mu);
    g_dm_products += dm.products;
    g_dm_syncs += dm.syncs;
}

static cudaStream_t g_stream = nullptr;  // the main thread's stream (the backend's)

// the device's default memory pool keeps freed memory for reuse (stream-
// ordered allocations of the tree levels and the device-resident numbers)
static void keep_pool_memory() {
    int dev = 0;
    cudaMemPool_t pool = nullptr;
    check_cuda(cudaGetDevice(&dev), "device");
    check_cuda(cudaDeviceGetDefaultMemPool(&pool, dev), "memory pool");
    uint64_t keep = ~0ull;
    check_cuda(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep), "memory pool");
}
static cudaStream_t gpu_stream() { return g_stream; }

struct GpuBackend : MulBackend {
    cudaStream_t st = nullptr;
    u64* h_buf = nullptr;  // pinned staging of a batch (operands, then results)
    size_t h_cap = 0;
    u64* d_buf = nullptr;  // device copy of the same layout
    size_t d_cap = 0;
    // the square root and the decimal powers run on a second host thread:
    // single products may come from both threads at once, batches from one
    // at a time (the staging buffers are shared)
    std::mutex stats_mu, batch_mu;
    size_t gpu_products = 0, host_products = 0, batches = 0;
    double mul_seconds = 0.0;  // wall time inside single products (host API), summed over threads

    GpuBackend() {
        check_cuda(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream");
        g_stream = st;
    }
    ~GpuBackend() override {
        if (h_buf) cudaFreeHost(h_buf);
        if (d_buf) cudaFree(d_buf);
        if (st) cudaStreamDestroy(st);
    }

    static bool small(const Nat& a, const Nat& b) { return std::max(a.size(), b.size()) <= kHostMaxLimbs; }

    void mul(const Nat& a, const Nat& b, Nat& out) override {
        const double t0 = now_sec();
        out.d.assign(a.size() + b.size(), 0);
        const bool host = small(a, b);
        if (host) {
            mul_school(a.d.data(), a.size(), b.d.data(), b.size(), out.d.data());
        } else {
            const int rc = prec_gpu_mul(a.d.data(), a.size(), b.d.data(), b.size(), out.d.data());
            if (rc) die("prec_gpu_mul", rc);
        }
        normalize(out);
        std::lock_guard<std::mutex> lk(stats_mu);
        ++(host ? host_products : gpu_products);
        mul_seconds += now_sec() - t0;
    }

    void reserve(size_t limbs) {
        if (limbs > h_cap) {
            if (h_buf) cudaFreeHost(h_buf);
            h_cap = limbs + limbs / 4;
            check_cuda(cudaHostAlloc(reinterpret_cast<void**>(&h_buf), h_cap * sizeof(u64), 0), "pinned buffer");
        }
        if (limbs > d_cap) {
            if (d_buf) cudaFree(d_buf);
            d_cap = limbs + limbs / 4;
            check_cuda(cudaMalloc(reinterpret_cast<void**>(&d_buf), d_cap * sizeof(u64)), "device buffer");
        }
    }

    static size_t up32(size_t x) { return (x + 31) & ~(size_t)31; }  // 256-byte aligned operands

    void mul_many(const std::vector<const Nat*>& A, const std::vector<const Nat*>& B,
                  std::vector<Nat>& out) override {
        std::lock_guard<std::mutex> blk(batch_mu);
        const size_t n = A.size();
        out.assign(n, Nat());
        std::vector<size_t> host, gpu;
        for (size_t i = 0; i < n; ++i) {
            if (A[i]->zero() || B[i]->zero()) continue;
            (small(*A[i], *B[i]) ? host : gpu).push_back(i);
        }
        parallel_for(host.size(), [&](size_t u) {
            const size_t i = host[u];
            out[i].d.assign(A[i]->size() + B[i]->size(), 0);
            mul_school(A[i]->d.data(), A[i]->size(), B[i]->d.data(), B[i]->size(), out[i].d.data());
            normalize(out[i]);
        });
        {
            std::lock_guard<std::mutex> lk(stats_mu);
            host_products += host.size();
        }
        if (gpu.empty()) return;
        // layout: the operands (one copy of an operand repeated within the
        // last few products, e.g. a shared divisor or a node used twice),
        // then the results
        std::vector<size_t> aoff(gpu.size()), boff(gpu.size());
        std::vector<std::pair<const Nat*, size_t>> uniq;  // operand, offset
        size_t in = 0;
        auto place = [&](const Nat* x) {
            const size_t lo = uniq.size() > 8 ? uniq.size() - 8 : 0;
            for (size_t j = uniq.size(); j-- > lo;)
                if (uniq[j].first == x) return uniq[j].second;
            uniq.emplace_back(x, in);
            in += up32(x->size());
            return uniq.back().second;
        };
        for (size_t u = 0; u < gpu.size(); ++u) {
            aoff[u] = place(A[gpu[u]]);
            boff[u] = place(B[gpu[u]]);
        }
        std::vector<size_t> ooff(gpu.size());
        size_t total = in;
        for (size_t u = 0; u < gpu.size(); ++u) {
            ooff[u] = total;
            total += up32(A[gpu[u]]->size() + B[gpu[u]]->size());
        }
        reserve(total);
        parallel_for(uniq.size(), [&](size_t u) {
            std::memcpy(h_buf + uniq[u].second, uniq[u].first->d.data(), uniq[u].first->size() * sizeof(u64));
        });
        check_cuda(cudaMemcpyAsync(d_buf, h_buf, in * sizeof(u64), cudaMemcpyHostToDevice, st), "H2D");
        std::vector<prec_gpu_product_t> items(gpu.size());
        for (size_t u = 0; u < gpu.size(); ++u) {
            const size_t i = gpu[u];
            items[u].a = d_buf + aoff[u];
            items[u].an = A[i]->size();
            items[u].b = d_buf + boff[u];
            items[u].bn = B[i]->size();
            items[u].out = d_buf + ooff[u];
        }
        const int rc = prec_gpu_mul_batch(items.data(), items.size(), st);
        if (rc) die("prec_gpu_mul_batch", rc);
        check_cuda(cudaMemcpyAsync(h_buf + in, d_buf + in, (total - in) * sizeof(u64), cudaMemcpyDeviceToHost, st),
                   "D2H");
        check_cuda(cudaStreamSynchronize(st), "batch");
        parallel_for(gpu.size(), [&](size_t u) {
            const size_t i = gpu[u];
            const size_t len = A[i]->size() + B[i]->size();
            out[i].d.assign(h_buf + ooff[u], h_buf + ooff[u] + len);
            normalize(out[i]);
        });
        std::lock_guard<std::mutex> lk(stats_mu);
        gpu_products += gpu.size();
        ++batches;
    }
};

// ---------------------------------------------------------------------------
// binary splitting, one level at a time
// ---------------------------------------------------------------------------

struct Node {
    Nat p, q, t;
    bool neg = false;  // sign of t
};

Nat from_u128(u128 v) {
    Nat r;
    r.d.push_back((u64)v);
    r.d.push_back((u64)(v >> 64));
    normalize(r);
    return r;
}

// term k of the series (pi_chudnovsky.cpp:119-136)
Node leaf(u64 k) {
    Node n;
    if (k == 0) {
        n.p = Nat(1);
        n.q = Nat(1);
        n.t = Nat(kA);
        return n;
    }
    const u128 p = (u128)(6 * k - 5) * (2 * k - 1) * (6 * k - 1);
    const u128 q = (u128)k * k * k * kC3Over24;
    const u128 t = p * (u128)(kB * k + kA);
    n.p = from_u128(p);
    n.q = from_u128(q);
    n.t = from_u128(t);
    n.neg = (k & 1) != 0;
    return n;
}

// signed sum of two magnitudes
void signed_add(Nat a, bool an, Nat b, bool bn, Nat& r, bool& rn) {
    if (an == bn) {
        add_in(a, b);
        r = std::move(a);
        rn = an && !r.zero();
        return;
    }
    if (cmp(a, b) >= 0) {
        sub_in(a, b);
        r = std::move(a);
        rn = an && !r.zero();
    } else {
        sub_in(b, a);
        r = std::move(b);
        rn = bn && !r.zero();
    }
}

// the node of terms [a, b) by recursive halving on the host (small operands)
Node host_split(u64 a, u64 b) {
    if (b - a == 1) return leaf(a);
    const u64 m = a + (b - a) / 2;
    Node l = host_split(a, m), r = host_split(m, b);
    auto hmul = [](const Nat& x, const Nat& y, Nat& out) {
        out.d.assign(x.size() + y.size(), 0);
        mul_school(x.d.data(), x.size(), y.d.data(), y.size(), out.d.data());
        normalize(out);
    };
    Node u;
    Nat t1, t2;
    hmul(l.q, r.q, u.q);
    hmul(l.t, r.q, t1);
    hmul(r.t, l.p, t2);
    hmul(l.p, r.p, u.p);
    signed_add(std::move(t1), l.neg, std::move(t2), r.neg, u.t, u.neg);
    return u;
}

bool trace_on() {
    static const bool on = std::getenv("PI_GB300_TRACE") != nullptr;
    return on;
}

// ---------------------------------------------------------------------------
// binary splitting with the levels resident in device memory
// ---------------------------------------------------------------------------

// One level of the tree on the device: P, Q and |T| of every node in one
// buffer (offsets in limbs, 4-limb aligned), T's signs in another.
struct DevLevel {
    std::vector<uint64_t> op, oq, ot;
    std::vector<uint32_t> np, nq, nt;
    uint64_t* buf = nullptr;
    int8_t* sign = nullptr;
    size_t nodes() const { return nq.size(); }
    void release(cudaStream_t st) {
        if (buf) cudaFreeAsync(buf, st);
        if (sign) cudaFreeAsync(sign, st);
        buf = nullptr;
        sign = nullptr;
    }
};

size_t up4(size_t x) { return (x + 3) & ~(size_t)3; }

// stream-ordered, from the device's default pool (its release threshold
// raised at start-up, so freed levels are reused without device-wide
// synchronisation)
template <class T>
T* dev_alloc(size_t n, cudaStream_t st) {
    void* p = nullptr;
    check_cuda(cudaMallocAsync(&p, std::max<size_t>(n, 1) * sizeof(T), st), "device level buffer");
    return static_cast<T*>(p);
}

// A block of kHostBlock terms on the stack: the node of terms [a, b) with
// fixed-size magnitudes (no heap allocation), by the same recursive
// halving.  For terms k < 3.1e7 (the program's limit of 4.3e8 digits) a
// term's q_k has at most 128 bits, p_k 81 and |t_k| 135, so a block of b
// terms has Q, P and |T| below 2^(128 (b - 1) + 140): 65 limbs for 32
// terms, and nothing inside it (Tl * Qr of two 16-term halves, plus the
// sum) above 66.
constexpr int kSmallLimbs = 72;

struct SmallNat {
    uint32_t n = 0;
    u64 d[kSmallLimbs];
};
struct SmallNode {
    SmallNat p, q, t;
    bool neg = false;
};

void small_set(SmallNat& x, u128 v) {
    x.d[0] = (u64)v;
    x.d[1] = (u64)(v >> 64);
    x.n = x.d[1] ? 2 : (x.d[0] ? 1 : 0);
}

void small_mul(const SmallNat& a, const SmallNat& b, SmallNat& r) {
    if (!a.n || !b.n) {
        r.n = 0;
        return;
    }
    if (a.n + b.n > (uint32_t)kSmallLimbs) std::abort();
    mul_school(a.d, a.n, b.d, b.n, r.d);
    r.n = a.n + b.n;
    while (r.n && r.d[r.n - 1] == 0) --r.n;
}

int small_cmp(const SmallNat& a, const SmallNat& b) {
    if (a.n != b.n) return a.n < b.n ? -1 : 1;
    for (uint32_t i = a.n; i-- > 0;)
        if (a.d[i] != b.d[i]) return a.d[i] < b.d[i] ? -1 : 1;
    return 0;
}

// r = a + b or |a - b| with its sign, as signed_add
void small_signed_add(const SmallNat& a, bool an, const SmallNat& b, bool bn, SmallNat& r, bool& rn) {
    if (an == bn) {
        const SmallNat& x = a.n >= b.n ? a : b;
        const SmallNat& y = a.n >= b.n ? b : a;
        u64 c = 0;
        for (uint32_t i = 0; i < x.n; ++i) {
            const u128 s = (u128)x.d[i] + (i < y.n ? y.d[i] : 0) + c;
            r.d[i] = (u64)s;
            c = (u64)(s >> 64);
        }
        r.n = x.n;
        if (c) {
            if (r.n >= (uint32_t)kSmallLimbs) std::abort();
            r.d[r.n++] = c;
        }
        rn = an && r.n;
        return;
    }
    const bool a_big = small_cmp(a, b) >= 0;
    const SmallNat& x = a_big ? a : b;
    const SmallNat& y = a_big ? b : a;
    u64 br = 0;
    for (uint32_t i = 0; i < x.n; ++i) {
        const u64 yi = i < y.n ? y.d[i] : 0;
        const u64 t = x.d[i] - yi - br;
        br = (x.d[i] < yi) || (x.d[i] == yi && br) ? 1 : 0;
        r.d[i] = t;
    }
    r.n = x.n;
    while (r.n && r.d[r.n - 1] == 0) --r.n;
    rn = (a_big ? an : bn) && r.n;
}

void small_leaf(u64 k, SmallNode& n) {
    if (k == 0) {
        small_set(n.p, 1);
        small_set(n.q, 1);
        small_set(n.t, kA);
        n.neg = false;
        return;
    }
    const u128 p = (u128)(6 * k - 5) * (2 * k - 1) * (6 * k - 1);
    small_set(n.p, p);
    small_set(n.q, (u128)k * k * k * kC3Over24);
    small_set(n.t, p * (u128)(kB * k + kA));
    n.neg = (k & 1) != 0;
}

void small_split(u64 a, u64 b, SmallNode& out) {
    if (b - a == 1) {
        small_leaf(a, out);
        return;
    }
    const u64 m = a + (b - a) / 2;
    SmallNode l, r;
    small_split(a, m, l);
    small_split(m, b, r);
    SmallNat t1, t2;
    small_mul(l.q, r.q, out.q);
    small_mul(l.t, r.q, t1);
    small_mul(r.t, l.p, t2);
    small_mul(l.p, r.p, out.p);
    small_signed_add(t1, l.neg, t2, r.neg, out.t, out.neg);
}

// The bottom level (blocks of `block` terms) computed on the host threads
// straight into fixed slots of the upload buffer; needs no device, so it
// runs while the device comes up.
struct HostBlocks {
    DevLevel L;  // offsets and sizes (no device buffers yet)
    // limbs in fixed slots; the tails past each number's size are never read
    // (not zero-filled: that took longer than the blocks' arithmetic)
    std::unique_ptr<u64[]> hv;
    size_t hv_n = 0;
    std::vector<int8_t> hs;
};

HostBlocks host_blocks(size_t terms, size_t block) {
    HostBlocks B;
    DevLevel& L = B.L;
    std::vector<int8_t>& hs = B.hs;
    const size_t m = (terms + block - 1) / block;
    constexpr size_t slot = 3 * kSmallLimbs;
    L.op.resize(m), L.oq.resize(m), L.ot.resize(m), L.np.resize(m), L.nq.resize(m), L.nt.resize(m);
    B.hv_n = m * slot;
    B.hv.reset(new u64[B.hv_n]);
    hs.resize(m);
    parallel_for(m, [&](size_t i) {
        SmallNode nd;
        small_split(i * block, std::min<size_t>(terms, (i + 1) * block), nd);
        u64* h = B.hv.get() + i * slot;
        std::copy(nd.p.d, nd.p.d + nd.p.n, h);
        std::copy(nd.q.d, nd.q.d + nd.q.n, h + kSmallLimbs);
        std::copy(nd.t.d, nd.t.d + nd.t.n, h + 2 * kSmallLimbs);
        L.op[i] = i * slot, L.oq[i] = i * slot + kSmallLimbs, L.ot[i] = i * slot + 2 * kSmallLimbs;
        L.np[i] = nd.p.n, L.nq[i] = nd.q.n, L.nt[i] = nd.t.n;
        hs[i] = nd.neg ? 1 : 0;
    });
    return B;
}

void upload_blocks(HostBlocks& B, DevLevel& L, cudaStream_t st) {
    L = std::move(B.L);
    L.buf = dev_alloc<u64>(B.hv_n, st);
    L.sign = dev_alloc<int8_t>(B.hs.size(), st);
    check_cuda(cudaMemcpyAsync(L.buf, B.hv.get(), B.hv_n * sizeof(u64), cudaMemcpyHostToDevice, st),
               "level upload");
    check_cuda(cudaMemcpyAsync(L.sign, B.hs.data(), B.hs.size(), cudaMemcpyHostToDevice, st), "sign upload");
    check_cuda(cudaStreamSynchronize(st), "level upload");
}

Nat download(const uint64_t* d, size_t n, cudaStream_t st) {
    Nat r;
    r.d.resize(n);
    check_cuda(cudaMemcpyAsync(r.d.data(), d, n * sizeof(u64), cudaMemcpyDeviceToHost, st), "download");
    check_cuda(cudaStreamSynchronize(st), "download");
    normalize(r);
    return r;
}

bool trace_on();
Node host_split(u64 a, u64 b);

// 32 terms: the host threads compute the tree's five lowest levels while the
// device comes up (its context takes ~0.2 s); at 10^8 digits the device had
// spent 0.076 s on the fifth level (9e5 products of ~30 limbs), mostly in
// planning and descriptor traffic.  (64-term blocks measured no faster: the
// host blocks took 0.145 s instead of 0.09.)
constexpr size_t kHostBlock = 32;

// Q(0, terms) and T(0, terms) from the host blocks of kHostBlock terms: every level
// on the device (products through one batch per level, T's signed sums by
// signed_add_many); only the root comes back.
void binary_split_device(HostBlocks& blocks, Nat& Q, Nat& T, bool& tneg) {
    cudaStream_t st;
    check_cuda(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream");
    double t0 = now_sec();
    DevLevel cur;
    upload_blocks(blocks, cur, st);
    if (trace_on()) std::fprintf(stderr, "  %zu blocks of %zu terms uploaded %.3f s\n", cur.nodes(), kHostBlock,
                                 now_sec() - t0);
    std::vector<prec_gpu_product_t> items;
    std::vector<AddPair> pairs;
    std::vector<uint32_t> chunk_pair;
    while (cur.nodes() > 1) {
        t0 = now_sec();
        const size_t m = cur.nodes(), npair = m / 2;
        const bool last_pair_is_last = (m % 2) == 0;
        DevLevel nx;
        const size_t mn = (m + 1) / 2;
        nx.op.resize(mn), nx.oq.resize(mn), nx.ot.resize(mn), nx.np.resize(mn), nx.nq.resize(mn), nx.nt.resize(mn);
        std::vector<uint64_t> o1(npair), o2(npair);
        std::vector<uint32_t> n1(npair), n2(npair);
        size_t total = 0, tmp = 0;
        for (size_t i = 0; i < npair; ++i) {
            const size_t l = 2 * i, r = 2 * i + 1;
            const bool need_p = !(last_pair_is_last && i == npair - 1);
            n1[i] = cur.nt[l] + cur.nq[r];
            n2[i] = cur.nt[r] + cur.np[l];
            nx.np[i] = need_p ? cur.np[l] + cur.np[r] : 0;
            nx.nq[i] = cur.nq[l] + cur.nq[r];
            nx.nt[i] = std::max(n1[i], n2[i]) + 1;
            nx.op[i] = total, total += up4(nx.np[i]);
            nx.oq[i] = total, total += up4(nx.nq[i]);
            nx.ot[i] = total, total += up4(nx.nt[i]);
            o1[i] = tmp, tmp += up4(n1[i]);
            o2[i] = tmp, tmp += up4(n2[i]);
        }
        if (m % 2) {  // the last node moves up unchanged
            const size_t s = m - 1, d = mn - 1;
            nx.np[d] = cur.np[s], nx.nq[d] = cur.nq[s], nx.nt[d] = cur.nt[s];
            nx.op[d] = total, total += up4(nx.np[d]);
            nx.oq[d] = total, total += up4(nx.nq[d]);
            nx.ot[d] = total, total += up4(nx.nt[d]);
        }
        nx.buf = dev_alloc<u64>(total, st);
        nx.sign = dev_alloc<int8_t>(mn, st);
        uint64_t* tbuf = dev_alloc<u64>(tmp, st);
        items.clear();
        for (size_t i = 0; i < npair; ++i) {
            const size_t l = 2 * i, r = 2 * i + 1;
            auto P = [&](uint64_t off) { return cur.buf + off; };
            items.push_back({P(cur.oq[l]), cur.nq[l], P(cur.oq[r]), cur.nq[r], nx.buf + nx.oq[i]});
            items.push_back({P(cur.ot[l]), cur.nt[l], P(cur.oq[r]), cur.nq[r], tbuf + o1[i]});
            items.push_back({P(cur.ot[r]), cur.nt[r], P(cur.op[l]), cur.np[l], tbuf + o2[i]});
            if (nx.np[i]) items.push_back({P(cur.op[l]), cur.np[l], P(cur.op[r]), cur.np[r], nx.buf + nx.op[i]});
        }
        int rc = prec_gpu_mul_batch(items.data(), items.size(), st);
        if (rc) die("prec_gpu_mul_batch", rc);
        pairs.resize(npair);
        chunk_pair.clear();
        for (size_t i = 0; i < npair; ++i) {
            AddPair& a = pairs[i];
            a.x = tbuf + o1[i];
            a.y = tbuf + o2[i];
            a.z = nx.buf + nx.ot[i];
            a.sx = cur.sign + 2 * i;
            a.sy = cur.sign + 2 * i + 1;
            a.sz = nx.sign + i;
            a.nx = n1[i], a.ny = n2[i], a.nz = nx.nt[i];
            a.chunk0 = (uint32_t)chunk_pair.size();
            chunk_pair.insert(chunk_pair.end(), add_chunks(a.nz), (uint32_t)i);
        }
        AddPair* d_pairs = dev_alloc<AddPair>(npair, st);
        uint32_t* d_chunks = dev_alloc<uint32_t>(chunk_pair.size(), st);
        void* scratch = dev_alloc<uint8_t>(signed_add_scratch_bytes(npair, chunk_pair.size()), st);
        check_cuda(cudaMemcpyAsync(d_pairs, pairs.data(), npair * sizeof(AddPair), cudaMemcpyHostToDevice, st), "pairs");
        check_cuda(cudaMemcpyAsync(d_chunks, chunk_pair.data(), chunk_pair.size() * sizeof(uint32_t),
                                   cudaMemcpyHostToDevice, st), "chunks");
        check_cuda(signed_add_many(d_pairs, npair, d_chunks, chunk_pair.size(), scratch, st), "signed sums");
        if (m % 2) {
            const size_t s = m - 1, d = mn - 1;
            if (cur.np[s])
                cudaMemcpyAsync(nx.buf + nx.op[d], cur.buf + cur.op[s], cur.np[s] * sizeof(u64), cudaMemcpyDeviceToDevice, st);
            cudaMemcpyAsync(nx.buf + nx.oq[d], cur.buf + cur.oq[s], cur.nq[s] * sizeof(u64), cudaMemcpyDeviceToDevice, st);
            cudaMemcpyAsync(nx.buf + nx.ot[d], cur.buf + cur.ot[s], cur.nt[s] * sizeof(u64), cudaMemcpyDeviceToDevice, st);
            cudaMemcpyAsync(nx.sign + d, cur.sign + s, 1, cudaMemcpyDeviceToDevice, st);
        }
        check_cuda(cudaStreamSynchronize(st), "level");
        cudaFreeAsync(d_pairs, st);
        cudaFreeAsync(d_chunks, st);
        cudaFreeAsync(scratch, st);
        cudaFreeAsync(tbuf, st);
        cur.release(st);
        cur = std::move(nx);
        if (trace_on())
            std::fprintf(stderr, "  level of %zu nodes on the device: %zu products, Q of the first node %u limbs, %.3f s\n",
                         m, items.size(), cur.nq[0], now_sec() - t0);
    }
    Q = download(cur.buf + cur.oq[0], cur.nq[0], st);
    T = download(cur.buf + cur.ot[0], cur.nt[0], st);
    int8_t sg = 0;
    check_cuda(cudaMemcpy(&sg, cur.sign, 1, cudaMemcpyDeviceToHost), "sign");
    tneg = sg != 0;
    cur.release(st);
    check_cuda(cudaStreamSynchronize(st), "levels freed");
    cudaStreamDestroy(st);
}

// Q(0, terms) and T(0, terms)
void binary_split(size_t terms, Nat& Q, Nat& T, bool& tneg) {
    // the lowest levels in blocks of kHostBlock terms on the host threads:
    // their products have at most about 66 limbs
    double t0 = now_sec();
    std::vector<Node> lv((terms + kHostBlock - 1) / kHostBlock);
    parallel_for(lv.size(), [&](size_t i) {
        lv[i] = host_split(i * kHostBlock, std::min<size_t>(terms, (i + 1) * kHostBlock));
    });
    if (trace_on()) std::fprintf(stderr, "  blocks of %zu terms: %zu nodes %.3f s\n", kHostBlock, lv.size(), now_sec() - t0);
    while (lv.size() > 1) {
        t0 = now_sec();
        const size_t m = lv.size(), pairs = m / 2;
        // the last node of a level (the range ending at `terms`) never needs P
        const bool last_pair_is_last = (m % 2) == 0;
        std::vector<const Nat*> A, B;
        A.reserve(4 * pairs);
        B.reserve(4 * pairs);
        for (size_t i = 0; i < pairs; ++i) {
            const Node& l = lv[2 * i];
            const Node& r = lv[2 * i + 1];
            A.push_back(&l.q), B.push_back(&r.q);  // Q
            A.push_back(&l.t), B.push_back(&r.q);  // Tl * Qr
            A.push_back(&r.t), B.push_back(&l.p);  // Tr * Pl
            const bool need_p = !(last_pair_is_last && i == pairs - 1);
            if (need_p) A.push_back(&l.p), B.push_back(&r.p);
        }
        std::vector<Nat> prod;
        backend().mul_many(A, B, prod);
        std::vector<size_t> base(pairs + 1, 0);
        for (size_t i = 0; i < pairs; ++i) base[i + 1] = base[i] + (last_pair_is_last && i == pairs - 1 ? 3 : 4);
        std::vector<Node> up((m + 1) / 2);
        parallel_for(pairs, [&](size_t i) {
            const size_t b = base[i];
            Node& u = up[i];
            u.q = std::move(prod[b]);
            signed_add(std::move(prod[b + 1]), lv[2 * i].neg, std::move(prod[b + 2]), lv[2 * i + 1].neg, u.t,
                       u.neg);
            if (base[i + 1] - b == 4) u.p = std::move(prod[b + 3]);
        });
        if (m % 2) up.back() = std::move(lv.back());
        lv.swap(up);
        if (trace_on())
            std::fprintf(stderr, "  level of %zu nodes: Q of the first node %zu limbs, %.3f s\n", m, lv[0].q.size(),
                         now_sec() - t0);
    }
    Q = std::move(lv[0].q);
    T = std::move(lv[0].t);
    tneg = lv[0].neg;
}

struct Phases {
    double init = 0;    // the library's start-up (its own thread, beside the host blocks)
    double blocks = 0;  // the bottom blocks of the tree on the host threads
    double split = 0, sqrt = 0, div = 0, dec = 0;
    double powers = 0;     // decimal powers and reciprocals (second thread)
    double root_wait = 0;  // time the main thread waited for the square root
};

// pi_chudnovsky.cpp:162-194.  `device_ready` waits for the library's
// start-up and installs the multiply backend; nothing before it touches the
// device.
std::string pi_digits(size_t digits, Phases& ph, const std::function<void()>& device_ready) {
    const size_t guard = 10, work = digits + guard, terms = work / 14 + 2;
    const bool host_levels = std::getenv("PI_GB300_HOST_LEVELS") != nullptr;
    const double tb = now_sec();
    HostBlocks blocks;
    if (!host_levels) blocks = host_blocks(terms, kHostBlock);
    ph.blocks = now_sec() - tb;
    device_ready();
    double t0 = now_sec();
    // isqrt(10005 * 10^(2 work)) and the powers of ten of the decimal
    // conversion do not depend on the series: a second thread computes them
    // while this one runs the binary splitting and the division (the
    // reference program computes the same values in sequence)
    const char* hn = std::getenv("PI_GB300_HOST_NEWTON");
    const bool host_newton = hn && hn[0] == '1';
    Nat root;     // host-resident form
    DNat root_d;  // device-resident form
    DecimalPowers pows;     // host-resident form
    DevDecimalPowers dpows; // device-resident form
    std::promise<void> root_set;
    std::future<void> root_ready = root_set.get_future();
    // pi * 10^digits < 4 * 10^digits: at most digits + 1 decimal digits (the
    // host form converts it); the device form converts pi * 10^(digits+10)
    // before the division by 10^10 and drops the last 10 digits: at most
    // digits + 12 by the conversion's bound on the digit count
    const int levels = decimal_levels(digits + 2);
    const int dlevels = decimal_levels(digits + 12);
    std::thread side([&] {
        const double s0 = now_sec();
        if (host_newton) {
            root = isqrt(mul_u64(pow_u64(10, 2 * work), 10005));
        } else {
            // 10005 * 10^(2 work) and its square root without leaving the device
            cudaStream_t sst = nullptr;
            check_cuda(cudaStreamCreateWithFlags(&sst, cudaStreamNonBlocking), "stream");
            double s1 = 0;
            {
                DevMath dm(sst);
                const DNat n = dm.mul_u64(dm.pow_u64(10, 2 * work), 10005);
                root_d = dm.isqrt(n);
                check_cuda(cudaStreamSynchronize(sst), "square root");
                root_d.st = nullptr;  // handed to the main thread (its stream adopts it)
                s1 = now_sec();
                root_set.set_value();
                dpows = dm.decimal_powers(dlevels);
                check_cuda(cudaStreamSynchronize(sst), "decimal powers");
                for (DNat& x : dpows.pw) x.st = nullptr;
                for (DNat& x : dpows.rx) x.st = nullptr;
                dm_stats_add(dm);
            }
            check_cuda(cudaStreamSynchronize(sst), "side stream");
            cudaStreamDestroy(sst);
            ph.sqrt = s1 - s0;
            ph.powers = now_sec() - s1;
            return;
        }
        const double s1 = now_sec();
        root_set.set_value();
        pows = decimal_powers(levels);
        ph.sqrt = s1 - s0;
        ph.powers = now_sec() - s1;
    });
    Nat Q, T;
    bool tneg = false;
    // PI_GB300_HOST_LEVELS=1: the tree's levels on the host, products staged
    // through host memory per level (the slower form, for comparison)
    if (host_levels) binary_split(terms, Q, T, tneg);
    else binary_split_device(blocks, Q, T, tneg);
    double t1 = now_sec();
    if (tneg || T.zero()) {
        side.join();
        return "error";
    }
    // T's reciprocal needs no root: its precision comes from a bound on
    // bitlen(Q * 426880 * root), with bitlen(root) <= log2(sqrt(10005) * 10^work) + 1
    const Nat q426880 = mul_u64(Q, 426880);
    const size_t root_bits = (size_t)(std::log2(std::sqrt(10005.0)) + (double)work * std::log2(10.0)) + 2;
    const size_t P = bitlen(q426880) + root_bits - bitlen(T) + 2 + 32;
    Nat pi, rem;
    std::string s;
    double t2r = 0, t2 = 0, t3 = 0;
    if (host_newton) {
        const Nat X = recip(T, P);
        t2r = now_sec();
        root_ready.wait();
        t2 = now_sec();
        const Nat num = mul(q426880, root);
        divmod_recip(num, T, X, P, pi, rem);
        divmod_u64(pi, 10000000000ull);
        t3 = now_sec();
        side.join();
        s = to_decimal(pi, 0, &pows);
    } else {
        // T, Q * 426880 up, the quotient down; everything between on the device
        DevMath dm(gpu_stream());
        const DNat Td = dm.upload(T);
        const DNat X = dm.recip(Td, P);
        const DNat qd = dm.upload(q426880);
        t2r = now_sec();
        root_ready.wait();
        t2 = now_sec();
        dm.adopt(root_d);
        const DNat num = dm.mul(qd, root_d);
        root_d = DNat();
        DNat pid, remd;
        dm.divmod_recip(num, Td, X, P, &pid, &remd);
        t3 = now_sec();
        // the digits of pi * 10^(digits + 10) on the device; dropping the
        // last 10 is the floor division by 10^10
        side.join();
        dm.adopt(dpows);
        s = dm.to_decimal(pid, dpows);
        s = s.size() > 10 ? s.substr(0, s.size() - 10) : std::string("0");
        dpows = DevDecimalPowers();
        dm_stats_add(dm);
    }
    double t4 = now_sec();
    ph.split = t1 - t0;
    ph.root_wait = t2 - t2r;
    ph.div = (t2r - t1) + (t3 - t2);
    ph.dec = t4 - t3;
    if (digits == 0) return s;
    if (s.size() <= digits) s.insert(0, digits + 1 - s.size(), '0');
    s.insert(s.end() - (long long)digits, '.');
    return s;
}

std::string short_form(const std::string& s, bool full) {
    if (full || s.size() <= 24) return s;
    return s.substr(0, 11) + "..." + s.substr(s.size() - 10);
}

// --self-check: the device-resident forms of the decimal conversion, the
// square root and the exact division (ddec.cu, dnat.cu) against bignum.cpp's
// host-resident forms, on the numbers where a divide and conquer or a
// correction step goes wrong first: zero, the powers of ten at the leaf and
// level sizes and their neighbours, long runs of nines and zeros, all-ones
// limbs, perfect squares and their predecessors, random numbers.  Returns the
// number of disagreements.
int self_check() {
    DevMath dm(gpu_stream());
    int bad = 0;
    auto report = [&](const std::string& what, bool ok) {
        if (!ok) {
            ++bad;
            std::fprintf(stderr, "self-check: %s: device and host forms differ\n", what.c_str());
        }
    };
    u64 rs = 0x9E3779B97F4A7C15ull;
    auto random_nat = [&](size_t limbs) {
        Nat x;
        x.d.resize(limbs);
        for (u64& v : x.d) {  // xorshift64
            rs ^= rs << 13, rs ^= rs >> 7, rs ^= rs << 17;
            v = rs;
        }
        normalize(x);
        return x;
    };
    const Nat one(1);
    const Nat t2048 = pow_u64(10, kDecimalLeafDigits), t4096 = sqr(t2048), t8192 = sqr(t4096);
    std::vector<std::pair<std::string, Nat>> xs;
    xs.push_back({"0", Nat()});
    xs.push_back({"1", one});
    xs.push_back({"9", Nat(9)});
    for (const auto& p : {std::make_pair(std::string("10^2048"), &t2048), std::make_pair(std::string("10^4096"), &t4096),
                          std::make_pair(std::string("10^8192"), &t8192)}) {
        xs.push_back({p.first + " - 1", sub(*p.second, one)});
        xs.push_back({p.first, *p.second});
        xs.push_back({p.first + " + 1", add(*p.second, one)});
    }
    const Nat t50000 = pow_u64(10, 50000);
    xs.push_back({"(10^50000 - 1) 10^50000", mul(sub(t50000, one), t50000)});
    xs.push_back({"2^64000 - 1", sub(pow2(64000), one)});
    xs.push_back({"2^(64 * 50000) - 1", sub(pow2(64 * 50000), one)});
    xs.push_back({"random 5190 limbs", random_nat(5190)});
    xs.push_back({"random 51906 limbs", random_nat(51906)});
    int levels = 0;
    for (const auto& x : xs) levels = std::max(levels, decimal_levels((size_t)((double)bitlen(x.second) * 0.30103) + 2));
    DevDecimalPowers pw = dm.decimal_powers(levels);
    for (const auto& x : xs) {
        const std::string h = to_decimal(x.second, 0);
        const std::string d = dm.to_decimal(dm.upload(x.second), pw);
        report("decimal text of " + x.first, h == d);
    }
    // square roots: the pi program's kind, perfect squares and their neighbours, random
    const Nat s = random_nat(40000);
    const Nat s2 = sqr(s);
    std::vector<std::pair<std::string, Nat>> ns;
    ns.push_back({"10005 10^100000", mul_u64(pow_u64(10, 100000), 10005)});
    ns.push_back({"s^2", s2});
    ns.push_back({"s^2 - 1", sub(s2, one)});
    ns.push_back({"s^2 + 2s", add(s2, shl(s, 1))});
    ns.push_back({"random 300000 limbs", random_nat(300000)});
    for (const auto& n : ns) report("square root of " + n.first, cmp(isqrt(n.second), dm.download(dm.isqrt(dm.upload(n.second)))) == 0);
    // exact division: random, and quotients at the correction's edges
    const Nat D = random_nat(150000);
    const Nat q0 = random_nat(250000);
    std::vector<std::pair<std::string, Nat>> nums;
    nums.push_back({"random 400000 limbs", random_nat(400000)});
    nums.push_back({"q D", mul(q0, D)});
    nums.push_back({"q D - 1", sub(mul(q0, D), one)});
    nums.push_back({"q D + D - 1", sub(add(mul(q0, D), D), one)});
    const DNat Dd = dm.upload(D);
    for (const auto& n : nums) {
        const size_t P = bitlen(n.second) - bitlen(D) + 2 + 32;
        Nat hq, hr;
        divmod_recip(n.second, D, recip(D, P), P, hq, hr);
        DNat dq, dr;
        dm.divmod_recip(dm.upload(n.second), Dd, dm.recip(Dd, P), P, &dq, &dr);
        report("division of " + n.first, cmp(hq, dm.download(dq)) == 0 && cmp(hr, dm.download(dr)) == 0);
    }
    std::fprintf(stderr, "self-check: %zu conversions, %zu square roots, %zu divisions, %d disagreements\n",
                 xs.size(), ns.size(), nums.size(), bad);
    return bad;
}

}  // namespace

int main(int argc, char** argv) {
#ifdef __GLIBC__
    // keep freed blocks of up to 32 MiB in the heap for reuse: the Newton
    // steps and conversion levels allocate and free numbers of the same
    // sizes over and over, and fresh pages cost a fault each
    mallopt(M_MMAP_THRESHOLD, 32 << 20);
    mallopt(M_TRIM_THRESHOLD, 1 << 30);
#endif
    size_t digits = 100;
    bool phases = false, full = false;
    std::string file;
    if (argc > 1 && std::string(argv[1]) == "--self-check") {
        const int rc = prec_gpu_init(-1);
        if (rc) die("prec_gpu_init", rc);
        GpuBackend be;
        set_backend(&be);
        const int bad = self_check();
        set_backend(nullptr);
        return bad ? 1 : 0;
    }
    if (argc > 1) digits = (size_t)std::strtoull(argv[1], nullptr, 10);
    for (int i = 2; i < argc; ++i) {
        const std::string a = argv[i];
        if (a == "--phases") phases = true;
        if (a == "--full") full = true;
        if (a == "--file" && i + 1 < argc) file = argv[++i];
    }
    // k^3 * 640320^3/24 must fit 128 bits: k < 3.1e7, about 4.3e8 digits
    if (digits > 400000000ull) {
        std::fprintf(stderr, "pi_gb300: at most 400000000 digits\n");
        return 1;
    }
    // the device comes up on its own thread while the host threads compute
    // the bottom blocks of the tree
    const double start = now_sec();
    Phases ph;
    int init_rc = 0;
    std::thread init_thread([&] {
        init_rc = prec_gpu_init(-1);
        ph.init = now_sec() - start;
    });
    std::unique_ptr<GpuBackend> be;
    auto device_ready = [&] {
        init_thread.join();
        if (init_rc) die("prec_gpu_init", init_rc);
        keep_pool_memory();
        be.reset(new GpuBackend());
        set_backend(be.get());
    };
    const std::string out = pi_digits(digits, ph, device_ready);
    const double sec = now_sec() - start;
    if (!file.empty()) {
        std::ofstream f(file.c_str(), std::ios::out | std::ios::binary);
        if (!f) {
            std::fprintf(stderr, "pi_gb300: cannot open %s\n", file.c_str());
            return 1;
        }
        f << out << "\n";
        f.flush();
        if (!f) {
            std::fprintf(stderr, "pi_gb300: writing %s failed\n", file.c_str());
            return 1;
        }
    }
    const double written = now_sec();
    std::printf("%s\n", short_form(out, full).c_str());
    if (phases) {
        std::fprintf(stderr, "init %.6f sec (its own thread)\n", ph.init);
        std::fprintf(stderr, "host_blocks %.6f sec\n", ph.blocks);
        std::fprintf(stderr, "write %.6f sec\n", written - start - sec);
        std::fprintf(stderr, "binary_split %.6f sec\n", ph.split);
        std::fprintf(stderr, "sqrt_scale %.6f sec (second thread)\n", ph.sqrt);
        std::fprintf(stderr, "decimal_powers %.6f sec (second thread)\n", ph.powers);
        std::fprintf(stderr, "root_wait %.6f sec\n", ph.root_wait);
        std::fprintf(stderr, "final_div %.6f sec\n", ph.div);
        std::fprintf(stderr, "to_decimal %.6f sec\n", ph.dec);
        std::fprintf(stderr, "gpu_products %zu host_products %zu gpu_batches %zu single-product time %.3f s\n",
                     be->gpu_products, be->host_products, be->batches, be->mul_seconds);
        std::fprintf(stderr, "device_newton_products %zu device_newton_syncs %zu\n", g_dm_products, g_dm_syncs);
    }
    std::fprintf(stderr, "gpu_launches %llu\n",
                 (unsigned long long)(prec_gpu_launch_count() + signed_add_launches() + dnat_launches()));
    if (!file.empty()) std::fprintf(stderr, "wrote %s\n", file.c_str());
    std::fprintf(stderr, "time %.6f sec\n", sec);
    return 0;
}
