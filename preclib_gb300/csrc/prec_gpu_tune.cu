// prec_gpu_tune.cu -- kernel configuration table and the autotuner.
//
// Every four-step transform length 2^k (k = 13 .. 26) has one kernel
// configuration: the column/row split (k1), columns per column-pass CTA,
// the column pass radix cap, rows per row-pass CTA and whether a single
// product runs each prime's kernels on its own stream.  plan_for reads the
// table for every product (single, batch, serving loop), so a tuned length
// changes every later product of that length.  The autotuner times the
// candidates on the device with balanced random operands, keeps a
// candidate only if its product equals the default configuration's bit for
// bit, and installs the fastest.  The reference has nothing to tune (one
// CPU code path, src/mul_ntt.cpp); the table replaces the fixed choices a
// GPU port would otherwise hard-code.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/prec_gpu.h"
#include "prec_gpu_internal.h"

namespace precgpu {

namespace {

constexpr int kTuneMin = kSmallMaxLog2 + 1;         // first four-step length
constexpr int kTuneMax = kMaxLog2;                 // 26
constexpr int kSplitMinLog2 = 19;  // default: per-prime streams from 2^19 points

struct Entry {
    bool tuned = false;
    KernelConfig cfg;
    float ms = 0.f, default_ms = 0.f;
};

std::mutex g_tune_mu;
Entry g_tune[kTuneMax + 1];

int set_of(int k) { return k <= kSetMaxLog2[0] ? 0 : 1; }

bool pow2(int x) { return x > 0 && (x & (x - 1)) == 0; }

}  // namespace

static KernelConfig default_config_set(int k, int set) {
    KernelConfig c;
    // column length N1 = 2^k1, row length N2 = 2^k2; set 1 keeps the rows at
    // 2^13 so its column CTAs stay within a third of shared memory
    c.k1 = set == 0 ? k / 2 : k - 13;
    int cg, mr;
    col_config(set, c.k1, 0, 0, cg, mr);
    c.cg = cg;
    c.cmr = mr;
    c.rmr = row_radix_cap(k - c.k1, 0);
    ntt_row_threads(k - c.k1, 1 << c.k1, &c.rows);
    c.split = k >= kSplitMinLog2 ? 1 : 0;
    return c;
}

KernelConfig default_config(int k) { return default_config_set(k, set_of(k)); }

bool config_valid(int k, const KernelConfig& c) {
    if (k < kTuneMin || k > kTuneMax) return false;
    const int set = set_of(k), k2 = k - c.k1;
    if (set == 0) {
        if (c.k1 < 6 || c.k1 > 11 || k2 < 7 || k2 > 12) return false;
    } else {
        if (c.k1 < 11 || c.k1 > 13 || k2 != 13) return false;
    }
    if (c.cg != 4 && c.cg != 8) return false;
    if (set == 1 && c.k1 >= 12 && c.cg != 4) return false;
    if (c.cmr != 4 && c.cmr != 6) return false;
    if (c.rmr != 4 && c.rmr != 6) return false;
    if (!pow2(c.rows) || c.rows > (1 << c.k1)) return false;
    const int threads = c.rows << (k2 - 5);
    if (threads < 32 || threads > 256) return false;
    return c.split == 0 || c.split == 1;
}

KernelConfig tuned_config(int k) {
    if (k >= kTuneMin && k <= kTuneMax) {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        if (g_tune[k].tuned) return g_tune[k].cfg;
    }
    return default_config(k);
}

KernelConfig config_for(int k, int set) {
    const int base = set_base(set);
    return base == set_of(k) ? tuned_config(k) : default_config_set(k, base);
}

void apply_config(Plan& pl, const KernelConfig& c) {
    pl.k1 = c.k1;
    pl.k2 = pl.k - c.k1;
    pl.cg = c.cg;
    pl.cmr = c.cmr;
    pl.rmr = c.rmr;
    pl.rows = c.rows;
    pl.split = c.split;
}

namespace {

__global__ void k_tune_fill(uint64_t* p, size_t n, uint64_t seed) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ull;  // SplitMix64
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        p[i] = z ^ (z >> 31);
    }
}

__global__ void k_tune_diff(const uint64_t* x, const uint64_t* y, size_t n, int* flag) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        if (x[i] != y[i]) atomicOr(flag, 1);
}

void to_entry(int k, const KernelConfig& c, float ms, float dms, prec_gpu_tune_entry_t* e) {
    e->log2_n = k;
    e->log2_cols = c.k1;
    e->col_group = c.cg;
    e->col_radix_cap = c.cmr;
    e->row_radix_cap = c.rmr;
    e->rows_per_cta = c.rows;
    e->split_primes = c.split;
    e->ms = ms;
    e->default_ms = dms;
}

KernelConfig from_entry(const prec_gpu_tune_entry_t* e) {
    KernelConfig c;
    c.k1 = e->log2_cols;
    c.cg = e->col_group;
    c.cmr = e->col_radix_cap;
    c.rmr = e->row_radix_cap;
    c.rows = e->rows_per_cta;
    c.split = e->split_primes;
    return c;
}

bool same(const KernelConfig& a, const KernelConfig& b) {
    return a.k1 == b.k1 && a.cg == b.cg && a.cmr == b.cmr && a.rmr == b.rmr && a.rows == b.rows &&
           a.split == b.split;
}

// Device buffers and timing of one tuning run.
struct Tuner {
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    uint64_t *a = nullptr, *b = nullptr, *out = nullptr, *ref = nullptr;
    uint8_t* flush = nullptr;
    int* flag = nullptr;
    size_t flush_bytes = (size_t)256 << 20;  // twice the L2
    int reps = 5;

    ~Tuner() {
        if (st) cudaStreamSynchronize(st);
        cudaFree(a);
        cudaFree(b);
        cudaFree(out);
        cudaFree(ref);
        cudaFree(flush);
        cudaFree(flag);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (st) cudaStreamDestroy(st);
    }

    int init(size_t max_limbs) {
        cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        if (!e) e = cudaEventCreate(&e0);
        if (!e) e = cudaEventCreate(&e1);
        if (!e) e = cudaMalloc(&a, max_limbs * sizeof(uint64_t));
        if (!e) e = cudaMalloc(&b, max_limbs * sizeof(uint64_t));
        if (!e) e = cudaMalloc(&out, 2 * max_limbs * sizeof(uint64_t));
        if (!e) e = cudaMalloc(&ref, 2 * max_limbs * sizeof(uint64_t));
        if (!e) e = cudaMalloc(&flush, flush_bytes);
        if (!e) e = cudaMalloc(&flag, sizeof(int));
        return cuda_code(e);
    }

    // median product time of configuration c for length 2^k (la = lb =
    // 2^(k-2) limbs); -1 if it fails or differs from the reference product
    float time(int k, const Plan& base, const KernelConfig& c, bool make_ref) {
        const uint64_t n = 1ull << (k - 2);
        Plan pl = base;
        apply_config(pl, c);
        if (ctx_enqueue_ntt_locked(a, n, b, n, out, pl, st)) return -1.f;
        if (cudaStreamSynchronize(st) != cudaSuccess) return -1.f;
        if (make_ref) {
            if (cudaMemcpyAsync(ref, out, 2 * n * sizeof(uint64_t), cudaMemcpyDeviceToDevice, st)) return -1.f;
        } else {
            int h = 0;
            cudaMemsetAsync(flag, 0, sizeof(int), st);
            k_tune_diff<<<8 * device_sm_count(), 256, 0, st>>>(out, ref, 2 * n, flag);
            count_launches(1);
            cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, st);
            if (cudaStreamSynchronize(st) != cudaSuccess || h) return -1.f;
        }
        std::vector<float> ms;
        for (int r = 0; r < reps; ++r) {
            cudaMemsetAsync(flush, r & 0xFF, flush_bytes, st);
            cudaEventRecord(e0, st);
            if (ctx_enqueue_ntt_locked(a, n, b, n, out, pl, st)) return -1.f;
            cudaEventRecord(e1, st);
            if (cudaEventSynchronize(e1) != cudaSuccess) return -1.f;
            float t = 0.f;
            cudaEventElapsedTime(&t, e0, e1);
            ms.push_back(t);
        }
        std::sort(ms.begin(), ms.end());
        return ms[ms.size() / 2];
    }
};

// Coordinate descent from the default configuration of length 2^k.
int tune_one(Tuner& T, int k, KernelConfig& best, float& best_ms, float& default_ms) {
    const uint64_t n = 1ull << (k - 2);
    Plan base;
    int r = plan_for(2 * n, 2 * n, 2 * n, base);
    if (r) return r;
    if (base.path != 1 || base.k != k) return PREC_GPU_E_INTERNAL;
    k_tune_fill<<<8 * device_sm_count(), 256, 0, T.st>>>(T.a, n, 0x1234567ull + k);
    k_tune_fill<<<8 * device_sm_count(), 256, 0, T.st>>>(T.b, n, 0x7654321ull + k);
    count_launches(2);
    if (cudaGetLastError() != cudaSuccess) return PREC_GPU_E_CUDA;
    best = default_config(k);
    best_ms = default_ms = T.time(k, base, best, true);
    if (best_ms < 0) return PREC_GPU_E_INTERNAL;
    auto consider = [&](const KernelConfig& c) {
        if (!config_valid(k, c) || same(c, best)) return;
        const float t = T.time(k, base, c, false);
        if (t > 0 && t < best_ms * 0.99f) {
            best = c;
            best_ms = t;
        }
    };
    auto tune_rows = [&]() {
        const KernelConfig start = best;
        for (int rows = 1; rows <= 256; rows <<= 1) {
            KernelConfig c = start;
            c.rows = rows;
            consider(c);
        }
    };
    {
        KernelConfig c = best;
        c.split ^= 1;
        consider(c);
    }
    tune_rows();
    {
        KernelConfig c = best;
        c.cg = c.cg == 8 ? 4 : 8;
        consider(c);
    }
    {
        KernelConfig c = best;
        c.cmr = c.cmr == 6 ? 4 : 6;
        consider(c);
    }
    {
        KernelConfig c = best;
        c.rmr = c.rmr == 6 ? 4 : 6;
        consider(c);
    }
    const KernelConfig before = best;
    for (int d = -1; d <= 1; d += 2) {
        KernelConfig c = before;
        c.k1 += d;
        if (c.k1 < 1) continue;
        int cg, mr;
        col_config(set_of(k), c.k1, c.cg, c.cmr, cg, mr);
        c.cg = cg;
        c.cmr = mr;
        c.rmr = row_radix_cap(k - c.k1, 0);
        ntt_row_threads(k - c.k1, 1 << c.k1, &c.rows);
        consider(c);
    }
    if (!same(before, best)) tune_rows();  // rows per CTA of the new split
    return 0;
}

}  // namespace
}  // namespace precgpu

using namespace precgpu;

extern "C" {

int prec_gpu_autotune(int kmin, int kmax, prec_gpu_tune_entry_t* out, size_t cap, size_t* count) {
    if (count) *count = 0;
    kmin = std::max(kmin, kTuneMin);
    kmax = std::min(kmax, kTuneMax);
    if (kmin > kmax) return PREC_GPU_E_ARG;
    std::lock_guard<std::mutex> lk(ctx_mutex());
    int r = ctx_init_locked(-1);
    if (r) return r;
    Plan top;
    if ((r = plan_for(1ull << (kmax - 1), 1ull << (kmax - 1), 1ull << (kmax - 1), top))) return r;
    // the largest workspace of any candidate: the same for every split
    if ((r = ctx_ensure_ws_locked(top.work_bytes))) return r;
    Tuner T;
    if ((r = T.init(1ull << (kmax - 2)))) return r;
    size_t n = 0;
    for (int k = kmin; k <= kmax; ++k) {
        KernelConfig best;
        float ms = 0.f, dms = 0.f;
        if ((r = tune_one(T, k, best, ms, dms))) return r;
        {
            std::lock_guard<std::mutex> tl(g_tune_mu);
            g_tune[k].tuned = true;
            g_tune[k].cfg = best;
            g_tune[k].ms = ms;
            g_tune[k].default_ms = dms;
        }
        if (out && n < cap) to_entry(k, best, ms, dms, &out[n]);
        ++n;
    }
    if (count) *count = n;
    return cuda_code(cudaGetLastError());
}

int prec_gpu_tune_get(int log2_n, prec_gpu_tune_entry_t* e) {
    if (!e || log2_n < kTuneMin || log2_n > kTuneMax) return PREC_GPU_E_ARG;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    const Entry& t = g_tune[log2_n];
    to_entry(log2_n, t.tuned ? t.cfg : default_config(log2_n), t.tuned ? t.ms : 0.f, t.tuned ? t.default_ms : 0.f,
             e);
    return PREC_GPU_OK;
}

int prec_gpu_tune_set(const prec_gpu_tune_entry_t* e) {
    if (!e) return PREC_GPU_E_ARG;
    const KernelConfig c = from_entry(e);
    if (!config_valid(e->log2_n, c)) return PREC_GPU_E_ARG;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[e->log2_n].tuned = true;
    g_tune[e->log2_n].cfg = c;
    g_tune[e->log2_n].ms = e->ms;
    g_tune[e->log2_n].default_ms = e->default_ms;
    return PREC_GPU_OK;
}

int prec_gpu_tune_reset(void) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    for (Entry& t : g_tune) t = Entry{};
    return PREC_GPU_OK;
}

// Text format: a header line "# prec_gpu tune 2", then per tuned length
// "log2_n log2_cols col_group col_radix_cap row_radix_cap rows_per_cta
// split_primes ms default_ms".
int prec_gpu_tune_save(const char* path) {
    if (!path) return PREC_GPU_E_ARG;
    FILE* f = std::fopen(path, "w");
    if (!f) return PREC_GPU_E_ARG;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    std::fprintf(f, "# prec_gpu tune 2\n");
    for (int k = kTuneMin; k <= kTuneMax; ++k) {
        const Entry& t = g_tune[k];
        if (!t.tuned) continue;
        std::fprintf(f, "%d %d %d %d %d %d %d %.6f %.6f\n", k, t.cfg.k1, t.cfg.cg, t.cfg.cmr, t.cfg.rmr, t.cfg.rows,
                     t.cfg.split, t.ms, t.default_ms);
    }
    const bool ok = std::fclose(f) == 0;
    return ok ? PREC_GPU_OK : PREC_GPU_E_ARG;
}

int prec_gpu_tune_load(const char* path) {
    if (!path) return PREC_GPU_E_ARG;
    FILE* f = std::fopen(path, "r");
    if (!f) return PREC_GPU_E_ARG;
    char line[256];
    std::vector<prec_gpu_tune_entry_t> got;
    bool header = false, bad = false;
    while (std::fgets(line, sizeof line, f)) {
        if (!header) {
            header = std::strncmp(line, "# prec_gpu tune 2", 17) == 0;
            if (!header) {
                bad = true;
                break;
            }
            continue;
        }
        if (line[0] == '\n' || line[0] == '#') continue;
        prec_gpu_tune_entry_t e{};
        if (std::sscanf(line, "%d %d %d %d %d %d %d %f %f", &e.log2_n, &e.log2_cols, &e.col_group, &e.col_radix_cap,
                        &e.row_radix_cap, &e.rows_per_cta, &e.split_primes, &e.ms, &e.default_ms) != 9 ||
            !config_valid(e.log2_n, from_entry(&e))) {
            bad = true;
            break;
        }
        got.push_back(e);
    }
    std::fclose(f);
    if (bad || !header) return PREC_GPU_E_ARG;
    for (const prec_gpu_tune_entry_t& e : got) prec_gpu_tune_set(&e);
    return PREC_GPU_OK;
}

}  // extern "C"
