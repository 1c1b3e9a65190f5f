// ntt_class.cu -- the batch form's persistent kernel per length class.
//
// The batch form normally runs a length class as four kernels (forward
// columns, rows, inverse columns, CRT/carry) over all its products.  Here
// one launch does all four: a grid of resident CTAs takes work items from an
// atomic ticket, in phase order (every forward column tile of every product,
// then the row tiles, the inverse column tiles and the carry blocks).  A
// tile whose inputs come from an earlier phase waits until that product's
// counter for the phase is complete.  Every item it waits on has an earlier
// ticket and is held by a running CTA, so the smallest unfinished item never
// waits and the launch cannot deadlock, with any grid size and no
// cooperative launch.
//
// Every wait is bounded (ClassRun::spin_limit polls): when one runs out, the
// CTA sets kDevErrTimeout in the product's error word and the class's abort
// word, and every CTA stops at its next item or poll; the host reads the
// error through prec_gpu_stream_check.  ClassRun::never_signal (tests only)
// makes the forward tiles leave their counters untouched, so the first row
// tile's wait runs out.
//
// Counters are released by the producing CTA (barrier, device fence, atomic
// add) and acquired by the waiting CTA's thread 0 (ld.acquire.gpu, then a
// barrier); data written earlier in the launch is read through L2 (the row
// and carry tiles' COH loads; the inverse columns stage by cp.async.cg).
//
// Instantiated for the default configurations of set 0's 2^13 .. 2^16-point
// classes (8 columns per column tile, column radix cap 6, row radix cap 4);
// a class with another configuration runs the four kernels.
#include <cuda_runtime.h>

#include "ntt_carry.cuh"
#include "ntt_cols.cuh"
#include "ntt_rows.cuh"
#include "prec_gpu_internal.h"

namespace precgpu {

namespace {

constexpr int kClassC = 8;    // columns per column tile
constexpr int kClassCMR = 6;  // column pass radix cap
constexpr int kClassRMR = 4;  // row pass radix cap

// waits until *ctr >= target: false when the class was aborted or after
// `limit` polls (about 0.25 us apart)
__device__ __forceinline__ bool wait_at_least(const uint32_t* ctr, uint32_t target, const uint32_t* abort,
                                              uint32_t limit) {
    for (uint32_t it = 0;; ++it) {
        uint32_t v;
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(ctr) : "memory");
        if (v >= target) return true;
        if (it >= limit || *reinterpret_cast<const volatile uint32_t*>(abort)) return false;
        __nanosleep(256);
    }
}

// resident CTAs per SM the kernel is compiled for (3: at most 85 registers)
#ifndef PREC_CLASS_MINB
#define PREC_CLASS_MINB 3
#endif

template <int M1, int M2, bool SQ>
__global__ void __launch_bounds__(256, PREC_CLASS_MINB) k_class(ProdArgs args, const ProdPtrs* __restrict__ batch, ClassRun run) {
    extern __shared__ uint32_t sm[];
    __shared__ uint32_t s_item, s_go;
    constexpr int C = kClassC;
    const uint32_t nbx = (1u << args.k2) / C;         // column tiles per (prime, operand)
    const uint32_t fwd_per_prime = SQ ? nbx : 2 * nbx;
    const uint32_t tiles0 = 3 * fwd_per_prime;         // forward column tiles of a product
    const uint32_t nrow = (1u << args.k1) / args.rows;  // row tiles per prime
    const uint32_t tiles1 = 3 * nrow;
    const uint32_t tiles2 = 3 * nbx;
    const uint32_t tiles3 = (uint32_t)run.max_nblk;
    const uint32_t n = (uint32_t)run.count;
    const uint32_t e0 = n * tiles0, e1 = e0 + n * tiles1, e2 = e1 + n * tiles2, e3 = e2 + n * tiles3;
    uint32_t* next = run.sched;
    uint32_t* abort = run.sched + 1;
    for (;;) {
        if (threadIdx.x == 0)
            s_item = *reinterpret_cast<volatile uint32_t*>(abort) ? e3 : atomicAdd(next, 1u);
        __syncthreads();
        const uint32_t item = s_item;
        if (item >= e3) break;
        int phase;
        uint32_t p, t;
        if (item < e0) {
            phase = 0, p = item / tiles0, t = item - p * tiles0;
        } else if (item < e1) {
            phase = 1, p = (item - e0) / tiles1, t = (item - e0) - p * tiles1;
        } else if (item < e2) {
            phase = 2, p = (item - e1) / tiles2, t = (item - e1) - p * tiles2;
        } else {
            phase = 3, p = (item - e2) / tiles3, t = (item - e2) - p * tiles3;
        }
        uint32_t* ctr = run.sched + kClassHdrWords + (size_t)p * kClassProdWords;
        // the tile's prime and its counter: forward [0..2], rows [3..5], inverse [6]
        int prime = 0, signal = -1;
        if (phase == 0) prime = SQ ? t / nbx : t / (2 * nbx), signal = prime;
        else if (phase == 1) prime = t / nrow, signal = 3 + prime;
        else if (phase == 2) prime = t / nbx, signal = 6;
        if (threadIdx.x == 0) {
            bool ok = true;
            if (phase == 1) ok = wait_at_least(ctr + prime, fwd_per_prime, abort, run.spin_limit);
            else if (phase == 2) ok = wait_at_least(ctr + 3 + prime, nrow, abort, run.spin_limit);
            else if (phase == 3) ok = wait_at_least(ctr + 6, tiles2, abort, run.spin_limit);
            if (!ok) {
                atomicExch(abort, 1u);
                atomicOr(args.err, kDevErrTimeout);
            }
            __threadfence();
            s_go = ok ? 1u : 0u;
        }
        __syncthreads();
        if (!s_go) break;
        if (phase == 0) {
            fwd_cols_tile<0, M1, C, kClassCMR>(args, batch, TileIdx{t % nbx, t / nbx, p, nbx}, sm);
        } else if (phase == 1) {
            rows_tile<0, M2, SQ, kClassRMR, true>(args, batch, TileIdx{t % nrow, (uint32_t)prime, p, nrow}, sm);
        } else if (phase == 2) {
            inv_cols_tile<0, M1, C, kClassCMR>(args, batch, TileIdx{t % nbx, (uint32_t)prime, p, nbx}, sm);
        } else {
            crt_carry_tile<0, true>(args, batch, TileIdx{t, 0, p, tiles3});
        }
        __syncthreads();
        if (threadIdx.x == 0 && signal >= 0 && !(phase == 0 && run.never_signal)) {
            __threadfence();
            atomicAdd(ctr + signal, 1u);
        }
    }
}

// (log2 N1, log2 N2) of set 0's 2^13 .. 2^16-point classes (k1 = k / 2)
#define PREC_CLASS_CONFIGS(X) X(6, 7) X(7, 7) X(7, 8) X(8, 8)

size_t class_smem(int m1, int m2, int rows) {
    const size_t cs = col_smem(m1, kClassC);
    const size_t rs = (size_t)rows * 2 * astride_for(m2) * sizeof(uint32_t);
    return cs > rs ? cs : rs;
}

// resident CTAs per SM of each instantiation, read once
template <int M1, int M2, bool SQ>
int class_occupancy(size_t smem) {
    static int occ = -1;
    if (occ < 0) {
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_class<M1, M2, SQ>, 256, smem) != cudaSuccess) n = 1;
        occ = n > 0 ? n : 1;
    }
    return occ;
}

}  // namespace

int class_rows(int k1, int k2) {
    const int rows = 256 >> (k2 - 5);
    return rows < (1 << k1) ? rows : (1 << k1);
}

bool class_persistent_supported(const Plan& pl) {
    if (pl.set != 0 || pl.path != 1 || pl.k < 13 || pl.k > 16) return false;
    int cg, mr;
    col_config(0, pl.k1, pl.cg, pl.cmr, cg, mr);
    if (cg != kClassC || mr != kClassCMR || row_radix_cap(pl.k2, pl.rmr) != kClassRMR) return false;
#define X(A, B) \
    if (pl.k1 == A && pl.k2 == B) return true;
    PREC_CLASS_CONFIGS(X)
#undef X
    return false;
}

int launch_class_persistent(const ProdArgs& a, const ProdPtrs* batch, const ClassRun& run, cudaStream_t st) {
    ProdArgs args = a;
    args.rows = run.rows;
    args.prime0 = 0;
    const size_t smem = class_smem(args.k1, args.k2, run.rows);
    const int nbx = (1 << args.k2) / kClassC;
    const uint64_t items = (uint64_t)run.count *
                           ((uint64_t)3 * (args.square ? nbx : 2 * nbx) + 3 * ((1 << args.k1) / run.rows) + 3 * nbx +
                            (uint64_t)run.max_nblk);
#define X(A, B)                                                                                  \
    if (args.k1 == A && args.k2 == B) {                                                          \
        if (args.square) {                                                                       \
            const uint64_t g = (uint64_t)class_occupancy<A, B, true>(smem) * device_sm_count();  \
            launch_kernel(k_class<A, B, true>, dim3((unsigned)(items < g ? items : g)), 256, smem, st, args, batch, run); \
        } else {                                                                                 \
            const uint64_t g = (uint64_t)class_occupancy<A, B, false>(smem) * device_sm_count(); \
            launch_kernel(k_class<A, B, false>, dim3((unsigned)(items < g ? items : g)), 256, smem, st, args, batch, run); \
        }                                                                                        \
        count_launches(1);                                                                       \
        return 0;                                                                                \
    }
    PREC_CLASS_CONFIGS(X)
#undef X
    return -1;
}

int configure_class() {
    cudaError_t e = cudaSuccess;
#define X(A, B)                                                                                           \
    if (!e) e = cudaFuncSetAttribute(k_class<A, B, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                                     (int)class_smem(A, B, class_rows(A, B)));                           \
    if (!e) e = cudaFuncSetAttribute(k_class<A, B, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,   \
                                     (int)class_smem(A, B, class_rows(A, B)));
    PREC_CLASS_CONFIGS(X)
#undef X
    return (int)e;
}

}  // namespace precgpu
