// prec_gpu_noalloc.cu -- a product entry point that allocates no memory.
//
// Some callers cannot call cudaMalloc: an application whose device memory
// is owned by its own pool allocator, a latency-critical loop that cannot
// afford the device-wide synchronisation cudaFree implies, or a plugin host
// that forbids device allocation once it has started.  For them,
// prec_gpu_mul_device_noalloc runs the same kernels as prec_gpu_mul_device
// but takes every byte it needs beyond the caller's inputs and outputs from
// memory that is part of this library image:
//   * g_noalloc_scratch -- the residue work buffer and carry words of one
//     product of up to 2^18 transform points (an + bn <= 131072 limbs),
//     about 6 MiB;
//   * g_noalloc_tables  -- the twiddle tables of the prime set those
//     transforms use, about 576 KiB.
// Every GPU that loads this library holds both arrays until the process
// exits.  Host code never passes the arrays' names to a kernel (in host
// code those names are host-side stand-ins, not device addresses): the
// set-up below asks the runtime for each array's device address once per
// device and passes that address.
//
// The device error word g_noalloc_err collects the error bits the kernels
// raise (a carry out of the product, a plan a kernel does not cover: both
// mean an internal fault).  prec_gpu_stream_check reads and clears it.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/prec_gpu.h"
#include "ntt_engine.cuh"
#include "prec_gpu_internal.h"

namespace precgpu {

constexpr int kNoAllocMaxLog2 = 18;
constexpr size_t kNoAllocWorkWords = (size_t)2 * kPrimes << kNoAllocMaxLog2;
// carry words: one counter plus one aggregate per 1024-limb block
constexpr size_t kNoAllocCarryWords = 1 + ((((size_t)1 << kNoAllocMaxLog2) / 2) / (kCarryThreads * kCarryLimbs) + 1);
constexpr int kTabEntries = 1 << kMaxSubLog2;  // Shoup entries per direction
constexpr int kTwEntries = 1 << kTwLevelBits;  // entries per four-step level
constexpr size_t kTabBytesPerPrime = (size_t)2 * kTabEntries * sizeof(uint2) + (size_t)2 * kTwEntries * sizeof(uint32_t);

static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocWorkWords + kNoAllocCarryWords];
static __device__ __align__(256) uint8_t g_noalloc_tables[kTabBytesPerPrime * kPrimes];
static __device__ __align__(256) int g_noalloc_err;

// prime set 0 (transforms up to 2^23 points; see ntt_field.cuh), the
// library's own primes and generators (set_primes / set_generators)
constexpr int kNaSet = 0;
constexpr int kNaL = kSetMaxLog2[kNaSet];
// largest product: an + bn limbs (2(an + bn) - 1 digits in 2^18 points)
constexpr uint64_t kNoAllocMaxLimbs = (uint64_t)1 << (kNoAllocMaxLog2 - 1);

__device__ uint32_t na_powmod(uint32_t b, uint64_t e, uint32_t p) {
    uint64_t r = 1, x = b % p;
    while (e) {
        if (e & 1) r = r * x % p;
        x = x * x % p;
        e >>= 1;
    }
    return (uint32_t)r;
}

// Fills the tables of one prime (blockIdx.y): Shoup pairs of the
// sub-transform roots in both directions and the two-level four-step
// table in Montgomery form, exactly the layout of the library context.
__global__ void k_noalloc_tables(uint8_t* tables, uint32_t p0, uint32_t p1, uint32_t p2, uint32_t g0, uint32_t g1,
                                 uint32_t g2) {
    const int j = blockIdx.y;
    const uint32_t p = j == 0 ? p0 : (j == 1 ? p1 : p2);
    const uint32_t g = j == 0 ? g0 : (j == 1 ? g1 : g2);
    uint2* tf = reinterpret_cast<uint2*>(tables + kTabBytesPerPrime * j);
    uint2* ti = tf + kTabEntries;
    uint32_t* twhi = reinterpret_cast<uint32_t*>(ti + kTabEntries);
    uint32_t* twlo = twhi + kTwEntries;
    const uint32_t wL = na_powmod(g, (p - 1) >> kNaL, p);
    const uint32_t R = (uint32_t)((1ull << 32) % p);
    const uint64_t order = 1ull << kNaL;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < kTabEntries; e += gridDim.x * blockDim.x) {
        uint32_t wf = 1, wi = 1;
        if (e > 0) {
            const int b = 31 - __clz(e);
            const uint64_t step = 1ull << (kNaL - b - 1);
            const uint64_t x = (uint64_t)(e - (1 << b)) * step;
            wf = na_powmod(wL, x, p);
            wi = na_powmod(wL, (order - x) & (order - 1), p);
        }
        tf[e] = make_uint2(wf, (uint32_t)(((uint64_t)wf << 32) / p));
        ti[e] = make_uint2(wi, (uint32_t)(((uint64_t)wi << 32) / p));
        twhi[e] = (uint32_t)((uint64_t)na_powmod(wL, ((uint64_t)e << kTwLevelBits) & (order - 1), p) * R % p);
        twlo[e] = (uint32_t)((uint64_t)na_powmod(wL, (uint64_t)e & (order - 1), p) * R % p);
    }
}

struct NoAllocDevice {
    bool ready = false;
    uint32_t* scratch = nullptr;
    int* err = nullptr;
    FieldArgs field{};
};

static std::mutex g_noalloc_mu;
static NoAllocDevice g_noalloc_dev[64];

static uint32_t na_mulmod(uint32_t a, uint32_t b, uint32_t m) { return (uint32_t)((uint64_t)a * b % m); }

static uint32_t na_hpow(uint32_t b, uint64_t e, uint32_t m) {
    uint64_t r = 1, x = b % m;
    while (e) {
        if (e & 1) r = r * x % m;
        x = x * x % m;
        e >>= 1;
    }
    return (uint32_t)r;
}

static ShoupC na_shoup(uint32_t w, uint32_t p) { return ShoupC{w, (uint32_t)(((uint64_t)w << 32) / p)}; }

// Garner constants for a 2^k-point transform (the same derivation as the
// library context's plan).
static CrtConst na_crt(int k) {
    const uint32_t* kNaP = set_primes(kNaSet);
    const uint32_t p1 = kNaP[0], p2 = kNaP[1], p3 = kNaP[2];
    uint32_t s[kPrimes];
    for (int j = 0; j < kPrimes; ++j) {
        const uint32_t P = kNaP[j];
        s[j] = na_mulmod((uint32_t)((1ull << 32) % P), na_hpow((uint32_t)((1ull << k) % P), P - 2, P), P);
    }
    const uint32_t c12 = na_hpow(p1 % p2, p2 - 2, p2), c13 = na_hpow(p1 % p3, p3 - 2, p3);
    const uint32_t c23 = na_hpow(p2 % p3, p3 - 2, p3), c1323 = na_mulmod(c13, c23, p3);
    CrtConst c;
    c.s1 = na_shoup(s[0], p1);
    c.k21 = na_shoup(c12, p2);
    c.k22 = na_shoup(na_mulmod(s[1], c12, p2), p2);
    c.k31 = na_shoup(c1323, p3);
    c.k32 = na_shoup(c23, p3);
    c.k33 = na_shoup(na_mulmod(s[2], c1323, p3), p3);
    c.fold[0] = na_mulmod(c.s1.w, (uint32_t)((1ull << 32) % p1), p1);
    c.fold[1] = na_mulmod(c.k22.w, (uint32_t)((1ull << 32) % p2), p2);
    c.fold[2] = na_mulmod(c.k33.w, (uint32_t)((1ull << 32) % p3), p3);
    return c;
}

static int na_code(cudaError_t e) {
    if (e == cudaSuccess) return PREC_GPU_OK;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return PREC_GPU_E_NODEV;
    return PREC_GPU_E_CUDA;
}

// Once per device, with that device current: device addresses of the
// static arrays, shared-memory opt-ins and the tables (a kernel on
// `stream`, waited for).  No allocation of any kind.
static int noalloc_setup(int dev, cudaStream_t stream, NoAllocDevice*& out) {
    if (dev < 0 || dev >= 64) return PREC_GPU_E_ARG;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    NoAllocDevice& d = g_noalloc_dev[dev];
    if (!d.ready) {
        void* scratch = nullptr;
        void* tables = nullptr;
        void* err = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&scratch, g_noalloc_scratch);
        if (e == cudaSuccess) e = cudaGetSymbolAddress(&tables, g_noalloc_tables);
        if (e == cudaSuccess) e = cudaGetSymbolAddress(&err, g_noalloc_err);
        if (e != cudaSuccess) return na_code(e);
        e = (cudaError_t)ntt_configure_kernels();
        if (e != cudaSuccess) return na_code(e);
        const uint32_t* P = set_primes(kNaSet);
        const uint32_t* G = set_generators(kNaSet);
        k_noalloc_tables<<<dim3(kTabEntries / 256, kPrimes), 256, 0, stream>>>(static_cast<uint8_t*>(tables), P[0],
                                                                               P[1], P[2], G[0], G[1], G[2]);
        count_launches(1);
        e = cudaGetLastError();
        // the error word starts clear (it keeps its bits across calls until
        // prec_gpu_stream_check reads them)
        if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(int), stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) return na_code(e);
        FieldArgs& f = d.field;
        f.max_log2 = kNaL;
        f.nprimes = kPrimes;
        for (int j = 0; j < kPrimes; ++j) {
            f.pc[j] = prime_constants(P[j]);
            const uint8_t* base = static_cast<const uint8_t*>(tables) + kTabBytesPerPrime * j;
            f.tf[j] = reinterpret_cast<const uint2*>(base);
            f.ti[j] = f.tf[j] + kTabEntries;
            f.twhi[j] = reinterpret_cast<const uint32_t*>(f.ti[j] + kTabEntries);
            f.twlo[j] = f.twhi[j] + kTwEntries;
        }
        d.scratch = static_cast<uint32_t*>(scratch);
        d.err = static_cast<int*>(err);
        d.ready = true;
    }
    out = &d;
    return PREC_GPU_OK;
}

static NoAllocDevice* current_device() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    return g_noalloc_dev[dev].ready ? &g_noalloc_dev[dev] : nullptr;
}

bool noalloc_ready() { return current_device() != nullptr; }

int noalloc_take_err() {
    NoAllocDevice* d = current_device();
    if (!d) return PREC_GPU_OK;
    int h = 0;
    cudaError_t e = cudaMemcpy(&h, d->err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && h) e = cudaMemset(d->err, 0, sizeof(int));
    if (e != cudaSuccess) return na_code(e);
    if (h & kDevErrTimeout) return PREC_GPU_E_TIMEOUT;
    return h ? PREC_GPU_E_INTERNAL : PREC_GPU_OK;
}

}  // namespace precgpu

using namespace precgpu;

extern "C" int prec_gpu_mul_device_noalloc(const uint64_t* d_a, size_t an, const uint64_t* d_b, size_t bn,
                                           uint64_t* d_out, void* stream) {
    // sizes first, each bounded before any arithmetic on them (no wrap)
    if (an > kNoAllocMaxLimbs || bn > kNoAllocMaxLimbs || an + bn > kNoAllocMaxLimbs)
        return PREC_GPU_E_TOO_LARGE;  // an + bn must not exceed 131072 limbs
    if (!d_a || !d_b || !d_out || an == 0 || bn == 0) return PREC_GPU_E_ARG;
    const uint64_t need = 2 * (uint64_t)an + 2 * (uint64_t)bn - 1;  // digits of the full product
    int k = kSmallMinLog2;
    while ((1ull << k) < need) ++k;  // k <= kNoAllocMaxLog2 by the bound above
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return na_code(e);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    NoAllocDevice* d = nullptr;
    int r = noalloc_setup(dev, st, d);
    if (r) return r;
    const uint64_t lout = (uint64_t)an + bn;
    if (k <= kSmallMaxLog2) {
        SmallDesc s{};
        s.a = d_a;
        s.b = d_b;
        s.out = d_out;
        s.la = an;
        s.lb = bn;
        s.lout = lout;
        s.k = k;
        ntt_launch_small(nullptr, &s, 1, k, d->field, na_crt(k), st);
    } else {
        ProdArgs args{};
        args.a = d_a;
        args.b = d_b;
        args.out = d_out;
        args.work = d->scratch;
        args.scratch = d->scratch + ((size_t)2 * kPrimes << k);  // zeroed by the first kernel of each call
        args.err = d->err;
        args.la = an;
        args.lb = bn;
        args.lout = lout;
        args.k = k;
        args.k1 = k / 2;
        args.k2 = k - args.k1;
        ntt_row_threads(args.k2, 1 << args.k1, &args.rows);
        const uint64_t bl = (uint64_t)kCarryThreads * kCarryLimbs;
        args.nblk = (int)((lout + bl - 1) / bl);
        args.crt = na_crt(k);
        args.f = d->field;
        ntt_launch_4step(0, args, st);
    }
    return na_code(cudaGetLastError());
}
