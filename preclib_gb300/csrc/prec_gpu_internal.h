// prec_gpu_internal.h -- library-internal interface between the host-side
// translation units (context and plans in prec_gpu_host.cu; batch form in
// prec_gpu_batch.cu; serving loop in prec_gpu_serve.cu).
#pragma once
#include <cuda_runtime.h>

#include <nvtx3/nvToolsExt.h>

#include <cstdarg>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <mutex>

#include "ntt_kernels.cuh"

namespace precgpu {

// A named NVTX range for the scope (header-only NVTX: without a profiler
// attached a push/pop costs a few nanoseconds).  Nsight Systems shows the
// library's host calls and their phases on the calling thread's row.
struct NvtxRange {
    explicit NvtxRange(const char* fmt, ...) {
        char buf[96];
        va_list ap;
        va_start(ap, fmt);
        std::vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        nvtxRangePushA(buf);
    }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// transform plan of one product on the NTT band
struct Plan {
    int k = 0, k1 = 0, k2 = 0;
    int set = 0;
    int path = 0;  // 0 single CTA, 1 four-step
    int nblk = 0;
    int rows = 0;  // rows per CTA of the row pass
    int cg = 0;    // columns per column-pass CTA (0: default)
    int cmr = 0;   // column pass radix cap (0: default)
    int rmr = 0;   // row pass radix cap (0: default)
    int split = 0; // per-prime stream chains for a single product
    int nprimes = 3;
    CrtConst crt{};   // sets 0 and 1
    Crt5Const crt5{}; // set 2
    size_t work_bytes = 0;  // work buffer + carry words of the four-step path
};

// da, db: 32-bit digit counts (upper bounds are fine); lout = La + Lb.
// The four-step kernel configuration comes from the tuning table (the
// autotuner's choice for the length, else the default configuration).
// `wide`: the plan may take set 2 (whole 64-bit limbs as digits, five
// primes, half the points) where that costs fewer butterflies; single
// products, the batch form and the serving loop pass wide_digits(), the
// autotuner keeps 32-bit digits.
int plan_for(uint64_t da, uint64_t db, uint64_t lout, Plan& pl, bool wide = false);
// log2 of the 64-bit-digit transform for la x lb limbs, or 0 where the
// 32-bit plan of 2^k32 points stays: it needs 2^13 .. 2^25 points, both
// operands in the lower half, min(la, lb) within the five primes' bound,
// and fewer butterflies (5 N' log N' < 3 N log N)
int wide_log2(uint64_t la, uint64_t lb, int k32);
// the five-prime set of a 64-bit-digit transform of 2^kw points (2 or 3)
int wide_set(int kw);
// 64-bit digits allowed (prec_gpu_set_wide_digits; PREC_GPU_WIDE_DIGITS)
bool wide_digits();

// Whether a batch class of plan `pl` can run as one persistent kernel
// (ntt_class.cu: set 0's 2^13 .. 2^16-point classes in their default
// kernel configuration).
bool class_persistent_supported(const Plan& pl);

// Kernel configuration of one four-step transform length (the autotuner's
// unit; prec_gpu_tune.cu).
struct KernelConfig {
    int k1 = 0;     // log2 column length (row length 2^(k - k1))
    int cg = 0;     // columns per column-pass CTA: 4 or 8
    int cmr = 0;    // column pass radix cap: 4 or 6
    int rmr = 0;    // row pass radix cap: 4 or 6
    int rows = 0;   // rows per row-pass CTA
    int split = 0;  // per-prime stream chains
};
KernelConfig default_config(int k);
// the configuration of length 2^k for a prime set: the table's (tuned or
// default) where the length's own set shares the set's kernels, else the
// default configuration of the set's kernel family
KernelConfig config_for(int k, int set);
bool config_valid(int k, const KernelConfig& c);
// the table's configuration for length 2^k (k >= 13)
KernelConfig tuned_config(int k);
// fills the four-step fields of a plan from a configuration
void apply_config(Plan& pl, const KernelConfig& c);

// Enqueues one NTT-band product with plan `pl` on device pointers (the
// library workspace must hold pl.work_bytes: ctx_ensure_ws_locked).  Call
// with the context lock held.
int ctx_enqueue_ntt_locked(const uint64_t* d_a, uint64_t la, const uint64_t* d_b, uint64_t lb, uint64_t* d_out,
                           const Plan& pl, cudaStream_t st);
int ctx_ensure_ws_locked(size_t bytes);

// the process-wide context: its lock, initialisation (idempotent, call
// with the lock held), prime-set tables and device error word
std::mutex& ctx_mutex();
int ctx_init_locked(int device);
const FieldArgs& ctx_field(int set);
int* ctx_device_err();
// reads and clears the device error bits (takes the library lock); 0 or a
// PREC_GPU_E_* code
int ctx_take_device_err();
// the library's stream-ordered memory pool (freed memory stays resident):
// workspace of one-shot batches
cudaMemPool_t ctx_pool();

int cuda_code(cudaError_t e);

// the primes and generators of prime set `set` (kSetPrimes[set] entries)
const uint32_t* set_primes(int set);
const uint32_t* set_generators(int set);
// every per-prime constant of PrimeC for the prime p
PrimeC prime_constants(uint32_t p);

// The no-allocation entry point's device error word on the current device:
// whether that device has been set up for it, and the word read and
// cleared (0 or a PREC_GPU_E_* code; the caller has synchronised the work).
bool noalloc_ready();
int noalloc_take_err();

}  // namespace precgpu
