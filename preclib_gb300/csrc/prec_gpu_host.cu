// prec_gpu_host.cu -- device context, transform plans and the C ABI.
//
// Host side of the multiply (C++17).  It owns, per process:
//   * the prime constants and twiddle tables, derived here from the primes
//     and generators (the reference tabulates Montgomery constants in
//     src/mul_ntt.cpp:37-41 and rebuilds root tables per size in
//     ntt_build_roots, mul_ntt.cpp:150-191; here one 2^13-entry table per
//     prime and direction serves every transform length);
//   * per calling thread, a lane (Lane): a stream for the host-pointer
//     entry points, a workspace and staging buffers that grow to the
//     largest product the thread has made, and its graphs, so
//     products from different threads overlap on the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

#include "../../include/prec_gpu.h"
#include "fft_kernels.cuh"
#include "ntt_kernels.cuh"
#include "prec_gpu_internal.h"

namespace precgpu {

typedef unsigned __int128 u128;

// Prime sets (see ntt_field.cuh): set 0 for transforms up to 2^23 points,
// set 1 -- the reference's primes and generators, src/mul_ntt.cpp:29-34 --
// for 2^24 .. 2^26 points; sets 2 and 3 (five primes, 64-bit digits) up to
// 2^22 and for 2^23 .. 2^25 points.
static const uint32_t kP[kSets][kMaxPrimes] = {
    {998244353u, 897581057u, 880803841u},
    {469762049u, 1811939329u, 2013265921u},
    {998244353u, 985661441u, 943718401u, 935329793u, 918552577u},
    {2113929217u, 2013265921u, 1811939329u, 1711276033u, 1107296257u}};
static const uint32_t kG[kSets][kMaxPrimes] = {
    {3u, 3u, 26u}, {3u, 13u, 31u}, {3u, 3u, 7u, 3u, 5u}, {5u, 31u, 13u, 29u, 10u}};
// a five-prime set recovers every coefficient exactly while min(la, lb)
// stays below p1..p5 / (2^64 - 1)^2: 2344425.6 (set 2), 42941745.4 (set 3)
static uint64_t wide_max_min_limbs(int set) { return set == kWideSet ? 2344425ull : 42941745ull; }

static uint32_t powmod(uint64_t b, uint64_t e, uint32_t m) {
    uint64_t r = 1 % m;
    b %= m;
    while (e) {
        if (e & 1) r = (uint64_t)((u128)r * b % m);
        b = (uint64_t)((u128)b * b % m);
        e >>= 1;
    }
    return (uint32_t)r;
}

static uint32_t invmod(uint32_t a, uint32_t m) { return powmod(a, m - 2, m); }  // m prime

static uint32_t mulmod(uint32_t a, uint32_t b, uint32_t m) { return (uint32_t)((uint64_t)a * b % m); }

static ShoupC shoup(uint32_t w, uint32_t p) {
    ShoupC c;
    c.w = w;
    c.wp = (uint32_t)(((uint64_t)w << 32) / p);
    return c;
}

static uint32_t neg_inv32(uint32_t m) {  // -m^{-1} mod 2^32 (Newton on 2-adic inverse)
    uint32_t x = 1;
    for (int i = 0; i < 5; ++i) x = x * (2u - m * x);
    return 0u - x;
}

int device_sm_count() {
    constexpr int kFallbackSms = 152;  // GB300
    static std::atomic<int> cached[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return kFallbackSms;
    }
    int v = cached[dev].load(std::memory_order_relaxed);
    if (v > 0) return v;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) {
        cudaGetLastError();
        return kFallbackSms;
    }
    cached[dev].store(v, std::memory_order_relaxed);
    return v;
}

const uint32_t* set_primes(int set) { return kP[set]; }
const uint32_t* set_generators(int set) { return kG[set]; }

PrimeC prime_constants(uint32_t p) {
    PrimeC pc;
    pc.p = p;
    pc.pinv = neg_inv32(p);
    pc.one_wp = (uint32_t)((1ull << 32) / p);
    pc.p2 = 2 * p;
    pc.r32 = (uint32_t)((1ull << 32) % p);
    pc.r32p = (uint32_t)(((uint64_t)pc.r32 << 32) / p);
    return pc;
}

constexpr int kMaxStages = 8;

// kernel names of each path, in launch order
static const char* const kStageNames[3][kMaxStages] = {
    {"k_small"},
    {"k_fwd_cols", "k_rows", "k_inv_cols", "k_crt_carry"},
    {"k_fft_fwd_cols", "k_fft_rows", "k_fft_inv_cols", "k_fft_carry"},
};
static const int kStageCount[3] = {1, 4, 4};

constexpr size_t kStatBytes = 16;       // device status block (error bits, FFT distance)
constexpr size_t kFftBandMin = 192;     // src/mul_basic.cpp:4 (FFT above 192 limbs)
constexpr size_t kFftBandMax = 6144;    // src/mul_basic.cpp:5 (NTT above 6144 limbs)

static CrtConst crt_compute(int set, int k) {
    const uint32_t* P = kP[set];
    const uint32_t p1 = P[0], p2 = P[1], p3 = P[2];
    uint32_t s[kPrimes];
    for (int j = 0; j < kPrimes; ++j) {
        const uint32_t R = (uint32_t)((1ull << 32) % P[j]);
        const uint32_t ninv = invmod((uint32_t)((1ull << k) % P[j]), P[j]);
        s[j] = mulmod(R, ninv, P[j]);
    }
    const uint32_t c12 = invmod(p1 % p2, p2), c13 = invmod(p1 % p3, p3), c23 = invmod(p2 % p3, p3);
    CrtConst c;
    c.s1 = shoup(s[0], p1);
    c.k21 = shoup(c12, p2);
    c.k22 = shoup(mulmod(s[1], c12, p2), p2);
    const uint32_t c1323 = mulmod(c13, c23, p3);
    c.k31 = shoup(c1323, p3);
    c.k32 = shoup(c23, p3);
    c.k33 = shoup(mulmod(s[2], c1323, p3), p3);
    c.fold[0] = mulmod(c.s1.w, (uint32_t)((1ull << 32) % p1), p1);
    c.fold[1] = mulmod(c.k22.w, (uint32_t)((1ull << 32) % p2), p2);
    c.fold[2] = mulmod(c.k33.w, (uint32_t)((1ull << 32) % p3), p3);
    return c;
}

// Garner constants of set 2 for 2^k points (Crt5Const): scale
// s_j = 2^32 N^-1 (the Montgomery factor of the pointwise product and the
// inverse transform's 1/N) folded into a_j.
static Crt5Const crt5_compute(int set, int k) {
    const uint32_t* P = kP[set];
    Crt5Const c;
    for (int j = 0; j < 5; ++j) {
        const uint32_t p = P[j];
        const uint32_t R = (uint32_t)((1ull << 32) % p);
        uint32_t a = mulmod(R, invmod((uint32_t)((1ull << k) % p), p), p);
        for (int i = 0; i < j; ++i) a = mulmod(a, invmod(P[i] % p, p), p);
        c.fold[j] = mulmod(a, R, p);
        for (int i = 0; i < j; ++i) {
            uint32_t b = 1;
            for (int l = i; l < j; ++l) b = mulmod(b, invmod(P[l] % p, p), p);
            c.b[j * (j - 1) / 2 + i] = shoup(b, p);
        }
    }
    return c;
}

// CRT constants of every (set, length), computed once: plan_for runs once
// per product of a batch, and a batch can hold millions of small products
static CrtConst crt_for(int set, int k) {
    static CrtConst table[2][kMaxLog2 + 1];
    static std::once_flag once;
    std::call_once(once, [] {
        for (int s = 0; s < 2; ++s)
            for (int j = kSmallMinLog2; j <= kSetMaxLog2[s]; ++j) table[s][j] = crt_compute(s, j);
    });
    return table[set][k];
}

static Crt5Const crt5_for(int set, int k) {
    static Crt5Const table[2][kMaxLog2 + 1];
    static std::once_flag once;
    std::call_once(once, [] {
        for (int s = kWideSet; s < kSets; ++s)
            for (int j = kSmallMaxLog2 + 1; j <= kSetMaxLog2[s]; ++j) table[s - kWideSet][j] = crt5_compute(s, j);
    });
    return table[set - kWideSet][k];
}

static int ceil_log2(uint64_t n) {
    int k = 0;
    while ((1ull << k) < n) ++k;
    return k;
}

int wide_set(int kw) { return kw <= kSetMaxLog2[kWideSet] ? kWideSet : kWideSetL; }

// Below 2^18 points the 64-bit plan measured no faster (2^13 .. 2^17: 5%
// slower to 4% faster): those products are bound by latency and launches,
// and five primes mean more launches.  From 2^18 it is 7-12% faster.
constexpr int kWideMinLog2 = 18;

int wide_log2(uint64_t la, uint64_t lb, int k32) {
    if (k32 <= kSmallMaxLog2) return 0;
    const int kw = ceil_log2(la + lb - 1);
    if (kw < kWideMinLog2 || kw > kSetMaxLog2[kWideSetL]) return 0;
    const uint64_t hi = la > lb ? la : lb, lo = la > lb ? lb : la;
    if (2 * hi <= (1ull << kw) && lo <= wide_max_min_limbs(wide_set(kw)) &&
        5 * ((uint64_t)kw << kw) < 3 * ((uint64_t)k32 << k32))
        return kw;
    return 0;
}

// da, db: 32-bit digit counts (upper bounds are fine)
int plan_for(uint64_t da, uint64_t db, uint64_t lout, Plan& pl, bool wide) {
    int k = ceil_log2(da + db - 1);
    if (k < kSmallMinLog2) k = kSmallMinLog2;
    if (k > kMaxLog2) return PREC_GPU_E_TOO_LARGE;
    pl.k = k;
    pl.set = k <= kSetMaxLog2[0] ? 0 : 1;
    pl.nprimes = kPrimes;
    pl.crt = crt_for(pl.set, k);
    if (k <= kSmallMaxLog2) {
        pl.path = 0;
        pl.work_bytes = 0;
        return 0;
    }
    pl.path = 1;
    if (wide) {
        const int kw = wide_log2((da + 1) / 2, (db + 1) / 2, k);
        if (kw) {
            k = kw;
            pl.k = k;
            pl.set = wide_set(kw);
            pl.nprimes = kMaxPrimes;
            pl.crt5 = crt5_for(pl.set, k);
        }
    }
    apply_config(pl, config_for(k, pl.set));
    const uint64_t bl = (uint64_t)crt_block_limbs(pl.set);
    pl.nblk = (int)((lout + bl - 1) / bl);
    pl.work_bytes = ((size_t)2 * pl.nprimes << k) * sizeof(uint32_t) + ((size_t)pl.nblk + 1) * sizeof(uint32_t);
    return 0;
}

// A single four-step product up to 2^kGraphMaxLog2 points runs as one CUDA
// graph replay: its kernels are the batch form's with a one-entry
// descriptor array, built once per plan shape; each call uploads the
// descriptor (operands, output, workspace, sizes) and launches the graph.
// Below 2^19 points the four kernels take only a few microseconds each,
// so launching them one by one left the GPU waiting on the host.
constexpr int kGraphMaxLog2 = 18;

struct GraphKey {
    int set, k, k1, cg, cmr, rmr, rows, square;
    bool operator<(const GraphKey& o) const {
        const int a[8] = {set, k, k1, cg, cmr, rmr, rows, square};
        const int b[8] = {o.set, o.k, o.k1, o.cg, o.cmr, o.rmr, o.rows, o.square};
        return std::lexicographical_compare(a, a + 8, b, b + 8);
    }
};

struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    ProdPtrs* d_desc = nullptr;  // the one-entry descriptor array the later kernels read
    uint64_t launches = 0;       // kernels per replay
    cudaGraphNode_t first = nullptr;  // the forward column node: the product's arguments by value
    cudaKernelNodeParams params{};
    cudaGraph_t graph = nullptr;  // kept: a node's parameters are set through its graph's node handle
};

// One calling thread's resources (a "lane"): its streams, the per-product
// workspace and staging buffers, the status block a host product reads
// back, events, per-prime streams and single-product graphs.
// Products on different lanes run concurrently on the GPU; a lane runs one
// product at a time (mu).  A thread takes a lane on its first call and
// keeps it; past kMaxLanes threads, threads share lanes round-robin.  (The
// reference's multiply is per thread the same way: its NTT plans are
// thread_local, src/mul_ntt.cpp:182-191.)
constexpr int kMaxLanes = 16;
struct Lane {
    std::mutex mu;
    cudaStream_t stream = nullptr;  // host-pointer products
    cudaStream_t cap = nullptr;     // the stream handle this lane's graph nodes are recorded for
    // host products with a chunked CRT: each chunk's limbs copy out on
    // `copy` while the next chunks run
    cudaStream_t copy = nullptr;
    uint8_t* ws = nullptr;
    size_t ws_cap = 0;
    uint64_t* io = nullptr;
    size_t io_cap = 0;        // limbs
    uint64_t* blk = nullptr;  // blocked products: a block pair's product, then the add kernel's scratch
    size_t blk_cap = 0;       // limbs
    int* d_err = nullptr;     // host products' device status: error bits at +0, FFT max distance at +8
    int* h_err = nullptr;     // pinned copy of the status
    double* d_maxdist = nullptr;
    double* h_maxdist = nullptr;
    FftArgs* fft_args = nullptr;  // the FP64 band product's arguments, read by its kernels
    cudaEvent_t last_done = nullptr, ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t ev_a = nullptr, ev_b = nullptr;  // each operand on the device
    cudaEvent_t stage_ev[kMaxStages + 1] = {};
    cudaEvent_t chunk_done[kCrtMaxChunks] = {};
    cudaEvent_t copy_done = nullptr;
    uint32_t* chunk_words = nullptr;  // 2 * kCrtMaxChunks words
    PrimeStreams prime_streams = {};
    std::map<GraphKey, GraphEntry> graphs;  // single-product graphs by plan shape
};

struct Ctx {
    std::mutex mu;  // initialisation, the lane list, the shared error word
    std::atomic<bool> ready{false};
    int device = -1;
    void* tables = nullptr;
    // library-wide device error word (device-pointer products, batches, the
    // tuner; read by prec_gpu_stream_check) and its pinned copy
    int* d_err = nullptr;
    int* h_err = nullptr;
    double2* fft_tw = nullptr;  // FP64 band twiddles
    FieldArgs field[kSets] = {};
    cudaMemPool_t pool = nullptr;
    bool split_primes = true;  // PREC_GPU_PRIME_STREAMS=0 runs the primes in one launch per kernel
    std::vector<std::unique_ptr<Lane>> lanes;
    std::atomic<uint64_t> gen{0};  // bumped by shutdown: threads then take new lanes
};

// 64-bit digits (set 2) for single products: on unless PREC_GPU_WIDE_DIGITS=0;
// prec_gpu_set_wide_digits changes it at run time
static std::atomic<int> g_wide{-1};

bool wide_digits() {
    int w = g_wide.load(std::memory_order_relaxed);
    if (w < 0) {
        const char* e = std::getenv("PREC_GPU_WIDE_DIGITS");
        int expect = -1;
        g_wide.compare_exchange_strong(expect, (e && e[0] == '0') ? 0 : 1);
        w = g_wide.load(std::memory_order_relaxed);
    }
    return w != 0;
}

static Ctx g_ctx;

static thread_local GraphRecorder* t_recorder = nullptr;
GraphRecorder*& thread_recorder() { return t_recorder; }

cudaGraphNode_t GraphRecorder::tail(cudaStream_t st) const {
    for (const auto& p : last)
        if (p.first == st) return p.second;
    return nullptr;
}

void GraphRecorder::set_tail(cudaStream_t st, cudaGraphNode_t n) {
    for (auto& p : last)
        if (p.first == st) {
            p.second = n;
            return;
        }
    last.emplace_back(st, n);
}

void GraphRecorder::add_kernel(const void* func, dim3 grid, dim3 block, size_t smem, void** args, cudaStream_t st) {
    if (err != cudaSuccess) return;
    cudaKernelNodeParams kp{};
    kp.func = const_cast<void*>(func);
    kp.gridDim = grid;
    kp.blockDim = block;
    kp.sharedMemBytes = (unsigned)smem;
    kp.kernelParams = args;  // the values are copied into the node
    kp.extra = nullptr;
    cudaGraphNode_t dep = tail(st), node = nullptr;
    err = cudaGraphAddKernelNode(&node, graph, dep ? &dep : nullptr, dep ? 1 : 0, &kp);
    if (err != cudaSuccess) return;
    if (!first) first = node;
    set_tail(st, node);
    ++nodes;
}

void GraphRecorder::add_memset(void* dst, size_t bytes, cudaStream_t st) {
    if (err != cudaSuccess || bytes == 0) return;
    cudaMemsetParams mp{};
    mp.dst = dst;
    mp.value = 0;
    mp.elementSize = 1;
    mp.width = bytes;
    mp.height = 1;
    mp.pitch = 0;
    cudaGraphNode_t dep = tail(st), node = nullptr;
    err = cudaGraphAddMemsetNode(&node, graph, dep ? &dep : nullptr, dep ? 1 : 0, &mp);
    if (err != cudaSuccess) return;
    if (!first) first = node;
    set_tail(st, node);
    ++nodes;
}

static std::atomic<uint64_t> g_launches{0};
static thread_local uint64_t t_launches = 0;

void count_launches(uint64_t n) {
    g_launches.fetch_add(n, std::memory_order_relaxed);
    t_launches += n;
}
uint64_t launches_this_thread() { return t_launches; }
void uncount_launches(uint64_t n) {
    g_launches.fetch_sub(n, std::memory_order_relaxed);
    t_launches -= n;
}
static thread_local prec_gpu_stats_t t_stats;

int cuda_code(cudaError_t e) {
    if (e == cudaSuccess) return 0;
    if (e == cudaErrorMemoryAllocation) return PREC_GPU_E_NOMEM;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return PREC_GPU_E_NODEV;
    return PREC_GPU_E_CUDA;
}

// PREC_GPU_DEBUG=1: every failed CUDA call the library checks is named on
// stderr with its error (file:line), before the code is returned
static int cuda_fail(cudaError_t e, const char* call, const char* file, int line) {
    static const bool debug = [] {
        const char* s = std::getenv("PREC_GPU_DEBUG");
        return s && s[0] == '1';
    }();
    if (debug) std::fprintf(stderr, "prec_gpu: %s:%d: %s: %s\n", file, line, call, cudaGetErrorName(e));
    return cuda_code(e);
}

#define CK(x)                                                                \
    do {                                                                     \
        cudaError_t _e = (x);                                                \
        if (_e != cudaSuccess) return cuda_fail(_e, #x, __FILE__, __LINE__); \
    } while (0)

// Per set and prime: Shoup tables of the sub-transform roots (forward and
// inverse, b < 13) and the two-level four-step table of the set's largest
// root in Montgomery form.
static int build_tables(Ctx& c) {
    const int T = 1 << kMaxSubLog2;   // entries of the Shoup tables
    const int H = 1 << kTwLevelBits;  // entries of each four-step level
    const size_t per_prime = (size_t)2 * T * sizeof(uint2) + (size_t)2 * H * sizeof(uint32_t);
    std::vector<uint8_t> host(per_prime * kMaxPrimes * kSets);
    CK(cudaMalloc(&c.tables, host.size()));
    for (int set = 0; set < kSets; ++set) {
        FieldArgs& fa = c.field[set];
        const int L = kSetMaxLog2[set];
        fa.max_log2 = L;
        fa.nprimes = kSetPrimes[set];
        for (int j = 0; j < kSetPrimes[set]; ++j) {
            const uint32_t p = kP[set][j];
            fa.pc[j] = prime_constants(p);
            // g^((p-1)/2) == -1, so wL = g^((p-1)/2^L) has order exactly 2^L
            if (powmod(kG[set][j], (p - 1) / 2, p) != p - 1) return PREC_GPU_E_INTERNAL;
            if (((p - 1) >> L) << L != p - 1) return PREC_GPU_E_INTERNAL;
            const uint32_t wL = powmod(kG[set][j], (p - 1) >> L, p);
            const size_t off = per_prime * (set * kMaxPrimes + j);
            uint2* tf = reinterpret_cast<uint2*>(host.data() + off);
            uint2* ti = tf + T;
            uint32_t* twhi = reinterpret_cast<uint32_t*>(ti + T);
            uint32_t* twlo = twhi + H;
            tf[0] = make_uint2(1, (uint32_t)((1ull << 32) / p));
            ti[0] = tf[0];
            for (int b = 0; b < kMaxSubLog2; ++b) {
                const uint32_t wb = powmod(wL, 1ull << (L - b - 1), p);  // order 2^(b+1)
                const uint32_t wbi = invmod(wb, p);
                uint32_t x = 1, y = 1;
                for (int i = 0; i < (1 << b); ++i) {
                    const ShoupC f = shoup(x, p), g = shoup(y, p);
                    tf[(1 << b) + i] = make_uint2(f.w, f.wp);
                    ti[(1 << b) + i] = make_uint2(g.w, g.wp);
                    x = mulmod(x, wb, p);
                    y = mulmod(y, wbi, p);
                }
            }
            const uint32_t R = (uint32_t)((1ull << 32) % p);
            const uint32_t step_hi = powmod(wL, (uint64_t)H, p);
            uint32_t x = R, y = R;
            for (int i = 0; i < H; ++i) {
                twhi[i] = x;
                twlo[i] = y;
                x = mulmod(x, step_hi, p);
                y = mulmod(y, wL, p);
            }
            const uint8_t* dbase = static_cast<uint8_t*>(c.tables) + off;
            fa.tf[j] = reinterpret_cast<const uint2*>(dbase);
            fa.ti[j] = fa.tf[j] + T;
            fa.twhi[j] = reinterpret_cast<const uint32_t*>(fa.ti[j] + T);
            fa.twlo[j] = fa.twhi[j] + H;
        }
    }
    CK(cudaMemcpy(c.tables, host.data(), host.size(), cudaMemcpyHostToDevice));
    return 0;
}

static int init_locked(Ctx& c, int device) {
    if (c.ready) return 0;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) return PREC_GPU_E_NODEV;
    if (device < 0) CK(cudaGetDevice(&device));
    if (device >= n) return PREC_GPU_E_ARG;
    CK(cudaSetDevice(device));
    c.device = device;
    {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        CK(cudaMemPoolCreate(&c.pool, &props));
        uint64_t keep = ~0ull;
        CK(cudaMemPoolSetAttribute(c.pool, cudaMemPoolAttrReleaseThreshold, &keep));
    }
    {
        const char* env = std::getenv("PREC_GPU_PRIME_STREAMS");
        c.split_primes = !(env && env[0] == '0');
    }
    CK(cudaMalloc(&c.d_err, kStatBytes));
    CK(cudaMemset(c.d_err, 0, kStatBytes));
    CK(cudaMallocHost(&c.h_err, kStatBytes));
    CK((cudaError_t)ntt_configure_kernels());
    CK((cudaError_t)fft_configure_kernels());
    CK(cudaMalloc(&c.fft_tw, fft_table_bytes()));
    fft_build_table(c.fft_tw, nullptr);
    CK(cudaGetLastError());
    int r = build_tables(c);
    if (r) return r;
    CK(cudaDeviceSynchronize());
    c.ready.store(true, std::memory_order_release);
    // a saved tuning table (an invalid file leaves the defaults in place)
    if (const char* tf = std::getenv("PREC_GPU_TUNE_FILE")) {
        if (prec_gpu_tune_load(tf) != PREC_GPU_OK) std::fprintf(stderr, "prec_gpu: ignoring tuning table %s\n", tf);
    }
    return 0;
}

static void lane_destroy(Lane& L) {
    if (L.stream) cudaStreamSynchronize(L.stream);
    for (auto& kv : L.graphs) {
        cudaGraphExecDestroy(kv.second.exec);
        cudaGraphDestroy(kv.second.graph);
        cudaFree(kv.second.d_desc);
    }
    L.graphs.clear();
    cudaFree(L.ws);
    cudaFree(L.io);
    cudaFree(L.blk);
    cudaFree(L.d_err);
    cudaFreeHost(L.h_err);
    cudaFree(L.fft_args);
    cudaFree(L.chunk_words);
    for (cudaEvent_t e : {L.last_done, L.ev0, L.ev1, L.ev_a, L.ev_b, L.copy_done})
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : L.stage_ev)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : L.chunk_done)
        if (e) cudaEventDestroy(e);
    for (int p = 0; p < kMaxPrimes; ++p) {
        if (L.prime_streams.s[p]) cudaStreamDestroy(L.prime_streams.s[p]);
        if (L.prime_streams.join[p]) cudaEventDestroy(L.prime_streams.join[p]);
    }
    if (L.prime_streams.fork) cudaEventDestroy(L.prime_streams.fork);
    for (cudaStream_t s : {L.stream, L.cap, L.copy})
        if (s) cudaStreamDestroy(s);
    fft_release_graphs(L.fft_args);
}

static int lane_create(Lane& L) {
    CK(cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&L.cap, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&L.copy, cudaStreamNonBlocking));
    for (int i = 0; i < kCrtMaxChunks; ++i) CK(cudaEventCreateWithFlags(&L.chunk_done[i], cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&L.copy_done, cudaEventDisableTiming));
    CK(cudaMalloc(&L.chunk_words, 2 * kCrtMaxChunks * sizeof(uint32_t)));
    CK(cudaEventCreateWithFlags(&L.last_done, cudaEventDisableTiming));
    CK(cudaEventCreate(&L.ev0));
    CK(cudaEventCreate(&L.ev1));
    CK(cudaEventCreateWithFlags(&L.ev_a, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&L.ev_b, cudaEventDisableTiming));
    for (int i = 0; i <= kMaxStages; ++i) CK(cudaEventCreate(&L.stage_ev[i]));
    for (int p = 0; p < kMaxPrimes; ++p) {
        CK(cudaStreamCreateWithFlags(&L.prime_streams.s[p], cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&L.prime_streams.join[p], cudaEventDisableTiming));
    }
    CK(cudaEventCreateWithFlags(&L.prime_streams.fork, cudaEventDisableTiming));
    CK(cudaMalloc(&L.d_err, kStatBytes));
    CK(cudaMemset(L.d_err, 0, kStatBytes));
    CK(cudaMallocHost(&L.h_err, kStatBytes));
    L.d_maxdist = reinterpret_cast<double*>(reinterpret_cast<char*>(L.d_err) + 8);
    L.h_maxdist = reinterpret_cast<double*>(reinterpret_cast<char*>(L.h_err) + 8);
    CK(cudaMalloc(&L.fft_args, sizeof(FftArgs)));
    return 0;
}

static thread_local Lane* t_lane = nullptr;
static thread_local uint64_t t_lane_gen = ~0ull;
static std::atomic<uint64_t> g_lane_rr{0};

// The calling thread's lane, the context initialised first (context lock
// held by the caller).
static int thread_lane_locked(Ctx& c, int device, Lane*& out) {
    int r = init_locked(c, device);
    if (r) return r;
    const uint64_t gen = c.gen.load(std::memory_order_relaxed);
    if (!t_lane || t_lane_gen != gen) {
        Lane* L = nullptr;
        if ((int)c.lanes.size() < kMaxLanes) {
            std::unique_ptr<Lane> p(new Lane());
            if ((r = lane_create(*p))) {
                lane_destroy(*p);
                return r;
            }
            L = p.get();
            c.lanes.push_back(std::move(p));
        } else {
            L = c.lanes[g_lane_rr.fetch_add(1, std::memory_order_relaxed) % kMaxLanes].get();
        }
        t_lane = L;
        t_lane_gen = gen;
    }
    out = t_lane;
    return 0;
}

// The calling thread's lane (takes the context lock only on the thread's
// first call and after a shutdown).
static int thread_lane(Ctx& c, Lane*& out) {
    if (t_lane && c.ready.load(std::memory_order_acquire) && t_lane_gen == c.gen.load(std::memory_order_relaxed)) {
        out = t_lane;
        return 0;
    }
    std::lock_guard<std::mutex> lk(c.mu);
    return thread_lane_locked(c, -1, out);
}

std::mutex& ctx_mutex() { return g_ctx.mu; }
int ctx_init_locked(int device) { return init_locked(g_ctx, device); }
const FieldArgs& ctx_field(int set) { return g_ctx.field[set]; }

// The error bits device work has set since the last read, cleared, as a
// library code (the work must have finished: the caller synchronised).
static int take_device_err_locked(Ctx& c) {
    CK(cudaMemcpy(c.h_err, c.d_err, sizeof(int), cudaMemcpyDeviceToHost));
    const int e = *c.h_err;
    CK(cudaMemset(c.d_err, 0, sizeof(int)));
    if (e & kDevErrTimeout) return PREC_GPU_E_TIMEOUT;
    if (e) return PREC_GPU_E_INTERNAL;
    return 0;
}

int ctx_take_device_err() {
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    if (!g_ctx.ready) return PREC_GPU_E_NODEV;
    return take_device_err_locked(g_ctx);
}
int* ctx_device_err() { return g_ctx.d_err; }
cudaMemPool_t ctx_pool() { return g_ctx.pool; }

// The lane's buffers grow to the largest product it has seen.  (A grown
// buffer is freed after the device is idle: earlier products of this lane
// may have been enqueued on callers' streams.)
static int grow(void** buf, size_t* cap, size_t bytes, bool slack) {
    if (bytes <= *cap) return 0;
    if (*buf) {
        CK(cudaDeviceSynchronize());
        cudaFree(*buf);
        *buf = nullptr;
        *cap = 0;
    }
    size_t want = slack ? std::max(bytes, bytes + bytes / 2) : bytes;
    if (cudaMalloc(buf, want) != cudaSuccess) {
        cudaGetLastError();
        if (want == bytes || cudaMalloc(buf, bytes) != cudaSuccess) {
            cudaGetLastError();
            return PREC_GPU_E_NOMEM;
        }
        want = bytes;
    }
    *cap = want;
    return 0;
}

static int ensure_ws(Lane& L, size_t bytes) { return grow(reinterpret_cast<void**>(&L.ws), &L.ws_cap, bytes, true); }

static int ensure_blk(Lane& L, size_t limbs) {
    size_t cap = L.blk_cap * sizeof(uint64_t);
    const int r = grow(reinterpret_cast<void**>(&L.blk), &cap, limbs * sizeof(uint64_t), false);
    L.blk_cap = cap / sizeof(uint64_t);
    return r;
}

static int ensure_io(Lane& L, size_t limbs) {
    size_t cap = L.io_cap * sizeof(uint64_t);
    const int r = grow(reinterpret_cast<void**>(&L.io), &cap, limbs * sizeof(uint64_t), false);
    L.io_cap = cap / sizeof(uint64_t);
    return r;
}

// Enqueues one NTT-band product on device pointers.
// A square (d_a == d_b, la == lb) transforms its one operand only on the
// four-step path; the single-CTA path reads the operand twice.
// One four-step product as a replay of its shape's graph (built on first
// use).  The forward column kernel takes the product by value -- a replay
// sets that node's parameters -- and stores its descriptor for the row,
// inverse column and carry kernels, which run in batch form on it.  (An
// upload of the descriptor by a copy in the stream measured 8-10 us slower
// per product when the caller's operands were page-locked.)
static int enqueue_graph(Lane& L, const ProdArgs& args, const Plan& pl, cudaStream_t st) {
    const GraphKey key{pl.set, pl.k, pl.k1, pl.cg, pl.cmr, pl.rmr, pl.rows, args.square};
    auto it = L.graphs.find(key);
    if (it == L.graphs.end()) {
        GraphEntry e;
        CK(cudaMalloc(&e.d_desc, sizeof(ProdPtrs)));
        ProdArgs first = args;
        first.publish = e.d_desc;
        ProdArgs cls = args;  // class-wide fields; the product's own come from the descriptor
        cls.a = cls.b = nullptr;
        cls.out = nullptr;
        cls.work = cls.scratch = nullptr;
        const uint64_t lout_max = set_wide(pl.set) ? (1ull << pl.k) + 1 : (1ull << pl.k) / 2 + 1;
        const uint64_t bl = (uint64_t)crt_block_limbs(pl.set);
        const int max_nblk = (int)((lout_max + bl - 1) / bl);
        // the four launches as a chain of kernel nodes (explicit
        // construction: no stream capture)
        GraphRecorder rec;
        cudaError_t err = cudaGraphCreate(&rec.graph, 0);
        if (err != cudaSuccess) {
            cudaFree(e.d_desc);
            return cuda_code(err);
        }
        const uint64_t before = launches_this_thread();
        t_recorder = &rec;
        launch_fwd_cols(pl.set, first, L.cap);
        launch_rows(pl.set, cls, L.cap, e.d_desc, 1);
        launch_inv_cols(pl.set, cls, L.cap, e.d_desc, 1);
        launch_crt_carry(pl.set, cls, L.cap, e.d_desc, 1, max_nblk);
        t_recorder = nullptr;
        e.launches = launches_this_thread() - before;  // recorded, counted at every replay
        uncount_launches(e.launches);
        cudaGraph_t g = rec.graph;
        err = rec.err;
        // the forward column node: the first recorded
        cudaGraphNode_t root = rec.first;
        if (err == cudaSuccess && root) err = cudaGraphKernelNodeGetParams(root, &e.params);
        if (err == cudaSuccess && !root) err = cudaErrorInvalidValue;
        e.first = root;
        if (err == cudaSuccess) err = cudaGraphInstantiate(&e.exec, g, 0);
        if (err != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            cudaFree(e.d_desc);
            return cuda_code(err);
        }
        e.graph = g;
        it = L.graphs.emplace(key, e).first;
    }
    GraphEntry& e = it->second;
    ProdArgs first = args;
    first.publish = e.d_desc;
    const ProdPtrs* no_batch = nullptr;
    void* params[2] = {&first, &no_batch};
    cudaKernelNodeParams kp = e.params;
    kp.kernelParams = params;
    kp.extra = nullptr;
    CK(cudaGraphExecKernelNodeSetParams(e.exec, e.first, &kp));
    CK(cudaGraphLaunch(e.exec, st));
    count_launches(e.launches);
    return 0;
}

// Device error bits go to `err` (the lane's status block for host
// products, the library-wide word otherwise).
static int enqueue_ntt(Ctx& c, Lane& L, const uint64_t* d_a, uint64_t la, const uint64_t* d_b, uint64_t lb,
                       uint64_t* d_out, const Plan& pl, cudaStream_t st, int* err, cudaEvent_t* ev = nullptr,
                       cudaEvent_t a_ready = nullptr, cudaEvent_t b_ready = nullptr,
                       const CrtChunks* chunks = nullptr) {
    const int square = (d_a == d_b && la == lb) ? 1 : 0;
    const uint64_t lout = la + lb;
    if (pl.path == 0) {
        SmallDesc d;
        d.a = d_a;
        d.b = d_b;
        d.out = d_out;
        d.la = la;
        d.lb = lb;
        d.lout = lout;
        d.k = pl.k;
        d.square = square;
        ntt_launch_small(nullptr, &d, 1, pl.k, c.field[0], pl.crt, st, ev);
    } else {
        ProdArgs args{};
        args.a = d_a;
        args.b = d_b;
        args.out = d_out;
        args.work = reinterpret_cast<uint32_t*>(L.ws);
        args.scratch = args.work + ((size_t)2 * pl.nprimes << pl.k);
        args.err = err;
        args.la = la;
        args.lb = lb;
        args.lout = lout;
        args.k = pl.k;
        args.k1 = pl.k1;
        args.k2 = pl.k2;
        args.nblk = pl.nblk;
        args.rows = pl.rows;
        args.cg = pl.cg;
        args.cmr = pl.cmr;
        args.rmr = pl.rmr;
        args.square = square;
        args.crt = pl.crt;
        args.crt5 = pl.crt5;
        args.f = c.field[pl.set];
        const bool split = c.split_primes && pl.split;
        // (a caller capturing `st` into its own graph gets plain launches: the
        // descriptor upload reads host memory that is gone at its replay)
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
        if (!split && !ev && pl.k <= kGraphMaxLog2 && cudaStreamIsCapturing(st, &cap) == cudaSuccess &&
            cap == cudaStreamCaptureStatusNone)
            return enqueue_graph(L, args, pl, st);
        ntt_launch_4step(pl.set, args, st, ev, split ? &L.prime_streams : nullptr, a_ready, b_ready,
                         split ? chunks : nullptr);
    }
    CK(cudaGetLastError());
    return 0;
}

// ---------------------------------------------------------------------------
// Blocked products: operands above the block size B (default 2^24 limbs,
// the size above which the reference's mul_ntt hands a product to mul_fft,
// src/mul_ntt.cpp:494-518) are cut into blocks of at most B limbs; every
// pair of blocks is one NTT-band product into a temporary, added into the
// result at its limb offset by k_add_into (ntt_add.cu).  All on one stream.
// ---------------------------------------------------------------------------

constexpr uint64_t kDefaultBlockLimbs = 1ull << 24;
constexpr uint64_t kMinBlockLimbs = 1024;
static std::atomic<uint64_t> g_block_limbs{kDefaultBlockLimbs};

static uint64_t block_limbs() { return g_block_limbs.load(std::memory_order_relaxed); }

// Device memory of a blocked product (the workspace of every block shape --
// whole blocks and the remainders -- and the temporary); `top` gets the
// plan of a whole block pair.
static int prepare_blocked(Lane& L, uint64_t la, uint64_t lb, uint64_t B, Plan& top) {
    const uint64_t sa[2] = {std::min(B, la), la % B}, sb[2] = {std::min(B, lb), lb % B};
    size_t ws = 0;
    for (int x = 0; x < 2; ++x)
        for (int y = 0; y < 2; ++y) {
            if (!sa[x] || !sb[y]) continue;
            Plan pl;
            int r = plan_for(2 * sa[x], 2 * sb[y], sa[x] + sb[y], pl, wide_digits());
            if (r) return r;
            ws = std::max(ws, pl.work_bytes);
            if (x == 0 && y == 0) top = pl;
        }
    const uint64_t tl = sa[0] + sb[0];
    int r = ensure_ws(L, ws);
    if (!r) r = ensure_blk(L, tl + (add_into_scratch_words(tl) + 1) / 2);
    return r;
}

// Enqueues a blocked product (after prepare_blocked for the same sizes).
static int enqueue_blocked(Ctx& c, Lane& L, const uint64_t* d_a, uint64_t la, const uint64_t* d_b, uint64_t lb,
                           uint64_t* d_out, cudaStream_t st, uint64_t B, int* err) {
    const uint64_t lout = la + lb;
    const uint64_t tl = std::min(B, la) + std::min(B, lb);
    uint64_t* tmp = L.blk;
    uint32_t* scratch = reinterpret_cast<uint32_t*>(L.blk + tl);
    int r = 0;
    CK(cudaMemsetAsync(d_out, 0, lout * sizeof(uint64_t), st));
    for (uint64_t i = 0; i < la; i += B)
        for (uint64_t j = 0; j < lb; j += B) {
            const uint64_t na = std::min(B, la - i), nb = std::min(B, lb - j);
            Plan pl;
            if ((r = plan_for(2 * na, 2 * nb, na + nb, pl, wide_digits()))) return r;
            if ((r = enqueue_ntt(c, L, d_a + i, na, d_b + j, nb, tmp, pl, st, err))) return r;
            launch_add_into(d_out + i + j, lout - i - j, tmp, na + nb, scratch, err, st);
        }
    CK(cudaGetLastError());
    return 0;
}

int ctx_enqueue_ntt_locked(const uint64_t* d_a, uint64_t la, const uint64_t* d_b, uint64_t lb, uint64_t* d_out,
                           const Plan& pl, cudaStream_t st) {
    Lane* L = nullptr;
    int r = thread_lane_locked(g_ctx, -1, L);
    if (r) return r;
    std::lock_guard<std::mutex> lk(L->mu);
    return enqueue_ntt(g_ctx, *L, d_a, la, d_b, lb, d_out, pl, st, g_ctx.d_err);
}

int ctx_ensure_ws_locked(size_t bytes) {
    Lane* L = nullptr;
    int r = thread_lane_locked(g_ctx, -1, L);
    if (r) return r;
    std::lock_guard<std::mutex> lk(L->mu);
    return ensure_ws(*L, bytes);
}

static size_t trim(const uint64_t* a, size_t n) {
    while (n > 0 && a[n - 1] == 0) --n;
    return n;
}

static uint64_t digits32(const uint64_t* a, size_t n) {  // n > 0, a[n-1] != 0
    return 2 * (uint64_t)n - ((a[n - 1] >> 32) == 0 ? 1 : 0);
}

// ---------------------------------------------------------------------------
// FP64 FFT band plan
// ---------------------------------------------------------------------------

// Worst-case rounding error of a 2^k-point FP64 convolution of b-bit
// balanced digits: C. Percival, "Rapid multiplication modulo the sum and
// difference of highly composite numbers", Math. Comp. 72 (2003), Thm 5.1:
// |err| <= |x| |y| ((1+e)^3k (1+e sqrt5)^(3k+1) (1+beta)^3k - 1), with
// |x| |y| <= N 2^(2b-2), e = 2^-53 and beta = 2^-52 for sincospi twiddles;
// doubled because both operands share one complex transform.
static double fft_error_bound(int b, int k) {
    const double e = std::ldexp(1.0, -53), beta = std::ldexp(1.0, -52);
    const double g = std::expm1(3.0 * k * std::log1p(e) + (3.0 * k + 1) * std::log1p(e * std::sqrt(5.0)) +
                                3.0 * k * std::log1p(beta));
    return 2.0 * std::ldexp(1.0, k + 2 * b - 2) * g;
}

struct FftPlan {
    int b = 0, k = 0, k1 = 0, k2 = 0;
    uint64_t da = 0, db = 0;
    size_t work_bytes = 0;
};

// Test knob for the rounding-failure path: PREC_GPU_FFT_DIGIT_BITS=b (8..30)
// forces the digit width regardless of the bound, so a test can make the
// FP64 band exceed 1/4 and check that the product is refused.
static int fft_forced_bits() {
    const char* s = std::getenv("PREC_GPU_FFT_DIGIT_BITS");
    if (!s) return 0;
    const int b = std::atoi(s);
    return b >= 8 && b <= 30 ? b : 0;
}

// widest digit (16 .. 8 bits) whose bound stays below 1/4
static bool fft_plan_for(uint64_t la, uint64_t lb, FftPlan& fp) {
    const int forced = fft_forced_bits();
    for (int b = forced ? forced : 16; b >= 8; --b) {
        const uint64_t da = (64 * la + b - 1) / b + 1, db = (64 * lb + b - 1) / b + 1;
        int k = 6;
        while ((1ull << k) < da + db - 1) ++k;
        if (k > kFftMaxLog2) continue;
        if (!forced && fft_error_bound(b, k) >= 0.25) continue;
        fp.b = b;
        fp.k = k;
        // the longer half along the columns: twice the row-pair CTAs of the
        // FP64-bound row kernel for odd k
        fp.k1 = (k + 1) / 2;
        fp.k2 = k - fp.k1;
        fp.da = da;
        fp.db = db;
        fp.work_bytes = ((size_t)sizeof(double2) + sizeof(long long)) << k;
        return true;
    }
    return false;
}

enum { kModeBands = 0, kModeNtt = 1, kModeFft = 2 };

// A square (a == b, an == bn: the reference's &a == &b test,
// src/mul_basic.cpp:244-246) copies its operand to the device once.
static int host_mul(const uint64_t* a, size_t an, const uint64_t* b, size_t bn, uint64_t* out, int mode) {
    if ((!a && an) || (!b && bn) || (!out && an + bn)) return PREC_GPU_E_ARG;
    const bool square = a == b && an == bn;
    Ctx& c = g_ctx;
    Lane* lp = nullptr;
    int r = thread_lane(c, lp);
    if (r) return r;
    Lane& L = *lp;
    std::lock_guard<std::mutex> lk(L.mu);
    const size_t total = an + bn;
    const size_t la = a ? trim(a, an) : 0, lb = b ? trim(b, bn) : 0;
    memset(&t_stats, 0, sizeof(t_stats));
    t_stats.limbs_a = la;
    t_stats.limbs_b = lb;
    if (la == 0 || lb == 0) {
        if (total) memset(out, 0, total * sizeof(uint64_t));
        return 0;
    }
    const uint64_t lout = la + lb;
    const size_t hi = la > lb ? la : lb;
    // band routing of src/mul_basic.cpp:263-269: 193..6144 limbs -> FP64 FFT;
    // larger products (and squares reaching mul_fft above 6144 limbs) and
    // products below 193 limbs -> NTT
    FftPlan fp;
    const bool use_fft = ((mode == kModeBands && hi > kFftBandMin) || mode == kModeFft) && hi <= kFftBandMax &&
                         fft_plan_for(la, lb, fp);
    // operands above the block size: a blocked product (the reference's
    // mul_ntt passes them to mul_fft, src/mul_ntt.cpp:494-518)
    const uint64_t B = block_limbs();
    const bool blocked = !use_fft && hi > B;
    Plan pl;
    if (blocked) {
        if ((r = prepare_blocked(L, la, lb, B, pl))) return r;
    } else {
        if (!use_fft && (r = plan_for(digits32(a, la), digits32(b, lb), lout, pl, wide_digits()))) return r;
        if ((r = ensure_ws(L, use_fft ? fp.work_bytes : pl.work_bytes))) return r;
    }
    // operands and result each start on a 256-byte boundary (32 limbs)
    const size_t la_pad = (la + 31) & ~(size_t)31, lb_pad = square ? 0 : (lb + 31) & ~(size_t)31;
    if ((r = ensure_io(L, la_pad + lb_pad + lout))) return r;
    uint64_t* d_a = L.io;
    uint64_t* d_b = square ? d_a : L.io + la_pad;
    uint64_t* d_out = L.io + la_pad + lb_pad;
    cudaStream_t st = L.stream;
    NvtxRange range("prec_gpu_mul %zux%zu %s", la, lb, use_fft ? "fft" : (blocked ? "blocked" : "ntt"));
    CK(cudaStreamWaitEvent(st, L.last_done, 0));
    // the per-prime chains start on a's forward columns while b is copied
    CK(cudaMemcpyAsync(d_a, a, la * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
    CK(cudaEventRecord(L.ev_a, st));
    if (!square) CK(cudaMemcpyAsync(d_b, b, lb * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
    CK(cudaEventRecord(L.ev_b, st));
    CK(cudaEventRecord(L.ev0, st));
    bool copied = false;  // the result went out chunk by chunk
    nvtxRangePushA("enqueue product");
    if (use_fft) {
        FftArgs f{};  // pageable: the small upload travels in the command stream
        f.a = d_a;
        f.bp = d_b;
        f.out = d_out;
        f.work = reinterpret_cast<double2*>(L.ws);
        f.coef = reinterpret_cast<long long*>(L.ws + (sizeof(double2) << fp.k));
        f.maxdist = L.d_maxdist;
        f.err = L.d_err;
        f.tw = c.fft_tw;
        f.la = la;
        f.lb = lb;
        f.lout = lout;
        f.da = fp.da;
        f.db = fp.db;
        f.ncoef = 1ull << fp.k;
        f.b = fp.b;
        f.k = fp.k;
        f.k1 = fp.k1;
        f.k2 = fp.k2;
        CK((cudaError_t)fft_launch(f, L.fft_args, st, nullptr, L.cap));
    } else if (blocked) {
        if ((r = enqueue_blocked(c, L, d_a, la, d_b, lb, d_out, st, B, L.d_err))) return r;
    } else {
        // a large product's CRT runs in limb chunks; each chunk's limbs copy
        // out on the copy stream while the next chunks run
        CrtChunks ch{};
        const bool chunked = pl.path == 1 && c.split_primes && pl.split && pl.nblk >= 2 * kCrtMaxChunks;
        if (chunked) {
            const int per = (pl.nblk + kCrtMaxChunks - 1) / kCrtMaxChunks;
            ch.count = (pl.nblk + per - 1) / per;  // every chunk nonempty
            ch.words = L.chunk_words;
            for (int i = 0; i <= ch.count; ++i) ch.blk0[i] = std::min(i * per, pl.nblk);
            for (int i = 0; i < ch.count; ++i) ch.done[i] = L.chunk_done[i];
            CK(cudaMemsetAsync(L.chunk_words, 0, 2 * kCrtMaxChunks * sizeof(uint32_t), st));
        }
        if ((r = enqueue_ntt(c, L, d_a, la, d_b, lb, d_out, pl, st, L.d_err, nullptr, L.ev_a, L.ev_b, chunked ? &ch : nullptr)))
            return r;
        if (chunked) {
            const uint64_t bl = (uint64_t)crt_block_limbs(pl.set);
            for (int i = 0; i < ch.count; ++i) {
                const uint64_t lo = std::min((uint64_t)ch.blk0[i] * bl, lout);
                const uint64_t hi = std::min((uint64_t)ch.blk0[i + 1] * bl, lout);
                CK(cudaStreamWaitEvent(L.copy, ch.done[i], 0));
                if (hi > lo)
                    CK(cudaMemcpyAsync(out + lo, d_out + lo, (hi - lo) * sizeof(uint64_t), cudaMemcpyDeviceToHost,
                                       L.copy));
            }
            CK(cudaEventRecord(L.copy_done, L.copy));
            copied = true;
        }
    }
    nvtxRangePop();
    CK(cudaEventRecord(L.ev1, st));
    // error word and the FFT distance first: a failed product leaves `out` untouched
    CK(cudaMemcpyAsync(L.h_err, L.d_err, kStatBytes, cudaMemcpyDeviceToHost, st));
    CK(cudaMemsetAsync(L.d_err, 0, sizeof(int), st));
    if (use_fft) CK(cudaStreamSynchronize(st));
    const bool fft_failed = use_fft && (*L.h_err & kDevErrFftRound);
    if (copied) CK(cudaStreamWaitEvent(st, L.copy_done, 0));
    else if (!fft_failed) CK(cudaMemcpyAsync(out, d_out, lout * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    CK(cudaEventRecord(L.last_done, st));
    {
        NvtxRange wait("wait for product and result copy");
        CK(cudaStreamSynchronize(st));
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, L.ev0, L.ev1);
    t_stats.path = use_fft ? 2 : (blocked ? 3 : pl.path);
    t_stats.log2_n = use_fft ? fp.k : pl.k;
    t_stats.primes = use_fft ? 0 : pl.nprimes;
    t_stats.digit_bits = use_fft ? fp.b : (set_wide(pl.set) ? 64 : 32);
    t_stats.device_ms = ms;
    t_stats.fft_max_distance = use_fft ? *L.h_maxdist : 0.0;
    if (fft_failed) return PREC_GPU_E_FFT_ROUNDING;
    if (total > lout) memset(out + lout, 0, (total - lout) * sizeof(uint64_t));
    if (*L.h_err & kDevErrTimeout) return PREC_GPU_E_TIMEOUT;
    if (*L.h_err) return PREC_GPU_E_INTERNAL;
    return 0;
}

}  // namespace precgpu

using namespace precgpu;

extern "C" {

int prec_gpu_init(int device) {
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    return init_locked(g_ctx, device);
}

void prec_gpu_shutdown(void) {
    Ctx& c = g_ctx;
    std::lock_guard<std::mutex> lk(c.mu);
    if (!c.ready) return;
    cudaDeviceSynchronize();
    for (auto& L : c.lanes) {
        std::lock_guard<std::mutex> ll(L->mu);
        lane_destroy(*L);
    }
    c.lanes.clear();
    c.gen.fetch_add(1, std::memory_order_relaxed);  // every thread takes a new lane next time
    cudaFree(c.tables);
    cudaFree(c.fft_tw);
    cudaFree(c.d_err);
    cudaFreeHost(c.h_err);
    if (c.pool) cudaMemPoolDestroy(c.pool);
    c.pool = nullptr;
    c.tables = nullptr;
    c.fft_tw = nullptr;
    c.d_err = c.h_err = nullptr;
    c.ready.store(false, std::memory_order_release);
}

int prec_gpu_mul(const uint64_t* a, size_t an, const uint64_t* b, size_t bn, uint64_t* out) {
    return host_mul(a, an, b, bn, out, kModeBands);
}

int prec_gpu_mul_ntt(const uint64_t* a, size_t an, const uint64_t* b, size_t bn, uint64_t* out) {
    return host_mul(a, an, b, bn, out, kModeNtt);
}

int prec_gpu_mul_fft(const uint64_t* a, size_t an, const uint64_t* b, size_t bn, uint64_t* out) {
    return host_mul(a, an, b, bn, out, kModeFft);
}

int prec_gpu_sqr(const uint64_t* a, size_t an, uint64_t* out) { return host_mul(a, an, a, an, out, kModeBands); }

int prec_gpu_fft_digit_bits(size_t an, size_t bn) {
    FftPlan fp;
    if (an == 0 || bn == 0 || (an > bn ? an : bn) > kFftBandMax || !fft_plan_for(an, bn, fp)) return 0;
    return fp.b;
}

int prec_gpu_mul_device(const uint64_t* d_a, size_t an, const uint64_t* d_b, size_t bn, uint64_t* d_out,
                        void* stream) {
    if (!d_a || !d_b || !d_out || an == 0 || bn == 0) return PREC_GPU_E_ARG;
    Ctx& c = g_ctx;
    Lane* lp = nullptr;
    int r = thread_lane(c, lp);
    if (r) return r;
    Lane& L = *lp;
    std::lock_guard<std::mutex> lk(L.mu);
    NvtxRange range("prec_gpu_mul_device %zux%zu", an, bn);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Plan pl;
    const uint64_t B = block_limbs();
    if (an > B || bn > B) {
        if ((r = prepare_blocked(L, an, bn, B, pl))) return r;
        CK(cudaStreamWaitEvent(st, L.last_done, 0));
        if ((r = enqueue_blocked(c, L, d_a, an, d_b, bn, d_out, st, B, c.d_err))) return r;
        CK(cudaEventRecord(L.last_done, st));
        return 0;
    }
    if ((r = plan_for(2 * (uint64_t)an, 2 * (uint64_t)bn, an + bn, pl, wide_digits()))) return r;
    if ((r = ensure_ws(L, pl.work_bytes))) return r;
    CK(cudaStreamWaitEvent(st, L.last_done, 0));
    if ((r = enqueue_ntt(c, L, d_a, an, d_b, bn, d_out, pl, st, c.d_err))) return r;
    CK(cudaEventRecord(L.last_done, st));
    return 0;
}

int prec_gpu_mul_device_profile(const uint64_t* d_a, size_t an, const uint64_t* d_b, size_t bn,
                                uint64_t* d_out, void* stream, float* stage_ms, int* nstages) {
    if (!d_a || !d_b || !d_out || an == 0 || bn == 0 || !stage_ms || !nstages) return PREC_GPU_E_ARG;
    Ctx& c = g_ctx;
    Lane* lp = nullptr;
    int r = thread_lane(c, lp);
    if (r) return r;
    Lane& L = *lp;
    std::lock_guard<std::mutex> lk(L.mu);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Plan pl;
    if ((r = plan_for(2 * (uint64_t)an, 2 * (uint64_t)bn, an + bn, pl, wide_digits()))) return r;
    if ((r = ensure_ws(L, pl.work_bytes))) return r;
    CK(cudaStreamWaitEvent(st, L.last_done, 0));
    if ((r = enqueue_ntt(c, L, d_a, an, d_b, bn, d_out, pl, st, c.d_err, L.stage_ev))) return r;
    CK(cudaEventRecord(L.last_done, st));
    CK(cudaStreamSynchronize(st));
    const int n = kStageCount[pl.path];
    for (int i = 0; i < n; ++i) CK(cudaEventElapsedTime(&stage_ms[i], L.stage_ev[i], L.stage_ev[i + 1]));
    *nstages = n;
    return 0;
}

const char* prec_gpu_stage_name(int path, int stage) {
    if (path < 0 || path > 2 || stage < 0 || stage >= kStageCount[path]) return "";
    return kStageNames[path][stage];
}

int prec_gpu_stream_check(void* stream) {
    Ctx& c = g_ctx;
    std::lock_guard<std::mutex> lk(c.mu);
    // a caller of the no-allocation entry point alone never starts the
    // context; its error word is read without allocating anything
    const bool na = noalloc_ready();
    if (!c.ready && !na) return PREC_GPU_E_NODEV;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CK(cudaStreamSynchronize(st));
    const int r = c.ready ? take_device_err_locked(c) : 0;
    const int rn = na ? noalloc_take_err() : 0;
    if (r) return r;
    if (rn) return rn;
    CK(cudaGetLastError());
    return 0;
}

int prec_gpu_last_stats(prec_gpu_stats_t* st) {
    if (!st) return PREC_GPU_E_ARG;
    *st = t_stats;
    return 0;
}

uint64_t prec_gpu_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

size_t prec_gpu_set_block_limbs(size_t limbs) {
    uint64_t v = limbs == 0 ? kDefaultBlockLimbs : limbs;
    v = std::max(kMinBlockLimbs, std::min(kDefaultBlockLimbs, v));
    return (size_t)g_block_limbs.exchange(v, std::memory_order_relaxed);
}

int prec_gpu_set_wide_digits(int on) {
    const int prev = wide_digits() ? 1 : 0;
    g_wide.store(on ? 1 : 0, std::memory_order_relaxed);
    return prev;
}

int prec_gpu_ntt_log2(size_t an, size_t bn) {
    if (an == 0 || bn == 0 || an > block_limbs() || bn > block_limbs()) return 0;
    Plan pl;
    if (plan_for(2 * (uint64_t)an, 2 * (uint64_t)bn, an + bn, pl, wide_digits())) return 0;
    return pl.k;
}

const char* prec_gpu_strerror(int code) {
    switch (code) {
        case PREC_GPU_OK: return "ok";
        case PREC_GPU_E_ARG: return "invalid argument";
        case PREC_GPU_E_TOO_LARGE: return "product exceeds the 2^26-point transform";
        case PREC_GPU_E_NOMEM: return "device allocation failed";
        case PREC_GPU_E_CUDA: return "CUDA runtime error";
        case PREC_GPU_E_TIMEOUT: return "bounded device-side wait ran out";
        case PREC_GPU_E_FFT_ROUNDING: return "FP64 rounding distance above 0.25";
        case PREC_GPU_E_NODEV: return "no usable CUDA device";
        case PREC_GPU_E_INTERNAL: return "internal consistency check failed";
        default: return "unknown error";
    }
}

}  // extern "C"
