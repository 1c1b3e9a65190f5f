// ntt_kernels.cuh -- declarations shared by the NTT kernels and the host.
#pragma once
#include <cstddef>
#include <cstdint>
#include <tuple>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "ntt_field.cuh"

namespace precgpu {

// Constants and device tables of one prime set, passed to every kernel by
// value (kernel parameter space).
struct FieldArgs {
    PrimeC pc[kMaxPrimes];
    const uint2* tf[kMaxPrimes];      // tf[(1<<b)+j] = (w_{2^{b+1}}^j, Shoup), b < 13
    const uint2* ti[kMaxPrimes];      // ti[(1<<b)+j] = (w_{2^{b+1}}^-j, Shoup)
    const uint32_t* twhi[kMaxPrimes]; // w_{2^L}^(h*2^13) * 2^32 mod p, L = set cap
    const uint32_t* twlo[kMaxPrimes]; // w_{2^L}^l * 2^32 mod p, l < 2^13
    int max_log2;                     // L
    int nprimes;                      // primes of the set
};

// CRT constants of one transform length (Garner with the transform's
// scale 2^32 * N^-1 folded in; see crt3 in ntt_engine.cuh).  The
// single-CTA path multiplies prime j's outputs by sigma_j in the CRT (s1,
// k22, k33 hold sigma_1, sigma_2 c12, sigma_3 c13 c23); the four-step path
// applies those products in its inverse column pass instead, through
// fold[j] = (that constant) * 2^32 mod p_j (Montgomery form) on the running
// twiddle, and its CRT multiplies by k21, k31, k32 only.
struct CrtConst {
    ShoupC s1, k21, k22, k31, k32, k33;
    uint32_t fold[3];
};

// Garner constants of the five-prime set for one transform length:
// v_j = y_j * a_j - sum_{i<j} v_i * b_{ij} (mod p_j), with
// a_j = 2^32 N^-1 (p_0 .. p_{j-1})^-1 and b_{ij} = (p_i .. p_{j-1})^-1 mod p_j;
// b_{ij} is b[j(j-1)/2 + i] (primes counted from 0).  The inverse column
// pass multiplies prime j's values by a_j (fold[j] = a_j * 2^32 mod p_j,
// Montgomery form, on its running twiddle), so the CRT starts from
// y_j * a_j directly.
struct Crt5Const {
    ShoupC b[10];
    uint32_t fold[5];
};

struct ProdPtrs;

// One product of the multi-pass (four-step) path.
struct ProdArgs {
    const uint64_t* a;
    const uint64_t* b;
    uint64_t* out;
    uint32_t* work;     // [prime][operand][N] residues
    uint32_t* scratch;  // carry look-back: [0] block ticket, [1..nblk] status words
    int* err;           // error bits (kDevErr*)
    uint64_t la, lb, lout;
    int k, k1, k2;      // log2 of N, of the column length N1, of the row length N2
    int nblk;           // blocks of the carry kernel
    int rows;           // rows per CTA of the row pass
    int square;         // a == b: one operand transform, pointwise square
    int prime0;         // first prime of this launch of the transform kernels (grid.y covers the rest)
    int cg;             // columns per column-pass CTA (0: default)
    int cmr;            // column pass radix cap, 4 or 6 (0: default)
    int operand_only;   // forward columns of one operand: 1 = a, 2 = b (0: both)
    int rmr;            // row pass radix cap, 4 or 6 (0: default)
    int crt_chunk;      // CRT in limb chunks (chunk_words set): this launch's chunk
    int crt_blk0;       //   its first carry block
    int crt_last;       //   whether it is the last chunk
    uint32_t* chunk_words;  // per chunk: [2c] finished blocks, [2c+1] carry into chunk c (nullptr: one launch)
    ProdPtrs* publish;      // forward columns store the product's ProdPtrs here for the later kernels (or nullptr)
    CrtConst crt;       // sets 0 and 1
    Crt5Const crt5;     // set 2
    FieldArgs f;
};

// Per-product part of ProdArgs in the batch form: a length class shares
// k, k1, k2, rows, crt and f; each product (blockIdx.z) has its own
// operands, output, work buffer and carry words.
struct ProdPtrs {
    const uint64_t* a;
    const uint64_t* b;
    uint64_t* out;
    uint32_t* work;
    uint32_t* scratch;
    uint64_t la, lb, lout;
    int nblk;
    int pad;
};

#ifdef __CUDACC__
// the product this CTA works on: the launch's own arguments, or entry
// blockIdx.z of a batch's descriptor array (a separate value, so the kernel
// parameter block is never written and stays in the constant bank)
__device__ __forceinline__ ProdPtrs select_product_at(const ProdArgs& args, const ProdPtrs* __restrict__ batch,
                                                      uint32_t z) {
    if (batch) return batch[z];
    ProdPtrs p;
    p.a = args.a;
    p.b = args.b;
    p.out = args.out;
    p.work = args.work;
    p.scratch = args.scratch;
    p.la = args.la;
    p.lb = args.lb;
    p.lout = args.lout;
    p.nblk = args.nblk;
    p.pad = 0;
    return p;
}
// Where a tile of a four-step pass finds its indices: GridIdx (one tile per
// CTA) reads blockIdx/gridDim where they are used, exactly as a kernel
// written for one tile does; TileIdx carries the indices a persistent kernel
// assigned.
struct GridIdx {
    __device__ __forceinline__ uint32_t x() const { return blockIdx.x; }
    __device__ __forceinline__ uint32_t y() const { return blockIdx.y; }
    __device__ __forceinline__ uint32_t z() const { return blockIdx.z; }
    __device__ __forceinline__ uint32_t nx() const { return gridDim.x; }
};
struct TileIdx {
    uint32_t bx, by, bz, nbx;
    __device__ __forceinline__ uint32_t x() const { return bx; }
    __device__ __forceinline__ uint32_t y() const { return by; }
    __device__ __forceinline__ uint32_t z() const { return bz; }
    __device__ __forceinline__ uint32_t nx() const { return nbx; }
};
__device__ __forceinline__ ProdPtrs select_product(const ProdArgs& args, const ProdPtrs* __restrict__ batch) {
    return select_product_at(args, batch, blockIdx.z);
}
#endif

// One product of the single-CTA path (transforms up to 2^12 points; also
// the batch form's small length classes).  Always prime set 0.
struct SmallDesc {
    const uint64_t* a;
    const uint64_t* b;
    uint64_t* out;
    uint64_t la, lb, lout;
    int k;
    int square;  // a == b (the single-CTA kernel reads the operand twice)
    // (the length's CRT constants are a kernel argument: one copy per launch,
    // not one per product of a batch class)
};

// device error bits
constexpr int kDevErrTimeout = 1;
constexpr int kDevErrCarry = 2;
constexpr int kDevErrPlan = 8;  // a kernel was given a product its plan does not cover

constexpr int kSmallMaxLog2 = 12;
constexpr int kSmallMinLog2 = 5;
constexpr int kCarryThreads = 256;
// build-time tunables (defaults are the measured best on GB300)
#ifndef PREC_CARRY_LIMBS
#define PREC_CARRY_LIMBS 4
#endif
#ifndef PREC_COL_GROUP
#define PREC_COL_GROUP 8
#endif
constexpr int kCarryLimbs = PREC_CARRY_LIMBS;  // limbs per thread in the carry kernel
// limbs one CRT/carry block outputs: kCarryThreads * kCarryLimbs for the
// 32-bit-digit sets; the 64-bit-digit sets' blocks give their first thread
// the coefficients just below the block (it outputs no limbs), one thread's
// worth fewer
constexpr int kCarryBlockLimbs = kCarryThreads * kCarryLimbs;
constexpr int kWideCarryBlockLimbs = kCarryBlockLimbs - kCarryLimbs;
__host__ __device__ constexpr int crt_block_limbs(int set) {
    return set_wide(set) ? kWideCarryBlockLimbs : kCarryBlockLimbs;
}
constexpr int kColGroup = PREC_COL_GROUP;      // adjacent columns per column-pass CTA (4 when N1 = 2^13)

// Explicit graph construction.  While a thread has a recorder installed,
// the library's launchers (launch_kernel) add kernel nodes to the
// recorder's graph instead of launching: a node depends on the node last
// recorded for the same stream handle, or on the recorder's fork point for
// that stream.  The library's graphs are built this way rather than by
// stream capture: a capture in progress can be broken by a device-wide
// synchronising call (cudaFree, cudaDeviceSynchronize, ...) that another
// thread of the process makes at the same time, and callers and lanes run
// products from several threads.
struct GraphRecorder {
    cudaGraph_t graph = nullptr;
    std::vector<std::pair<cudaStream_t, cudaGraphNode_t>> last;  // per stream handle
    cudaGraphNode_t first = nullptr;  // the first node recorded
    cudaError_t err = cudaSuccess;
    uint64_t nodes = 0;
    cudaGraphNode_t tail(cudaStream_t st) const;
    void set_tail(cudaStream_t st, cudaGraphNode_t n);
    // `to` starts after what is recorded on `from` so far (a fork)
    void fork(cudaStream_t from, cudaStream_t to) { set_tail(to, tail(from)); }
    void add_kernel(const void* func, dim3 grid, dim3 block, size_t smem, void** args, cudaStream_t st);
    void add_memset(void* dst, size_t bytes, cudaStream_t st);  // zero fill
};
// the calling thread's recorder (null: launchers launch)
GraphRecorder*& thread_recorder();

template <class Tuple, size_t... I>
inline void arg_ptrs(Tuple& t, void** p, std::index_sequence<I...>) {
    ((p[I] = static_cast<void*>(&std::get<I>(t))), ...);
}

// k<<<grid, block, smem, st>>>(args...), or a node of the thread's recorder
template <class... P, class... A>
inline void launch_kernel(void (*k)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, A&&... args) {
    if (GraphRecorder* r = thread_recorder()) {
        std::tuple<P...> vals(std::forward<A>(args)...);
        void* ptrs[sizeof...(P) > 0 ? sizeof...(P) : 1];
        arg_ptrs(vals, ptrs, std::index_sequence_for<P...>{});
        r->add_kernel(reinterpret_cast<const void*>(k), grid, block, smem, ptrs, st);
    } else {
        k<<<grid, block, smem, st>>>(std::forward<A>(args)...);
    }
}

// Kernel launches issued by the library (process-wide, prec_gpu_launch_count);
// every launcher adds its launches.  launches_this_thread() lets a graph
// recording take back the launches it only recorded.
void count_launches(uint64_t n);
uint64_t launches_this_thread();
void uncount_launches(uint64_t n);

// host-side launchers; `ev` (optional) gets an event recorded before the
// first kernel and after each kernel.
size_t ntt_small_smem_bytes(int k);
int ntt_small_threads(int k);
void ntt_launch_small(const SmallDesc* d_descs, const SmallDesc* single, int count, int k,
                      const FieldArgs& f, const CrtConst& crt, cudaStream_t st, cudaEvent_t* ev = nullptr);
// Side streams of a single product: each prime's transform kernels run as
// an independent chain (fork from and join to the caller's stream), so
// one prime's tail wave overlaps another prime's work.
struct PrimeStreams {
    cudaStream_t s[kMaxPrimes];
    cudaEvent_t fork;
    cudaEvent_t join[kMaxPrimes];
};
// The CRT of a single product in limb chunks, launched in order: `done[c]`
// is recorded after chunk c, whose limbs are then final (the caller copies
// them out while the next chunks run).  `words` (2 * count words) must be
// zero in stream order before the first chunk.
constexpr int kCrtMaxChunks = 4;
struct CrtChunks {
    int count;
    int blk0[kCrtMaxChunks + 1];  // chunk c: carry blocks blk0[c] .. blk0[c+1]-1
    uint32_t* words;
    cudaEvent_t done[kCrtMaxChunks];
};
// With side streams, `a_ready` / `b_ready` (recorded on `st` after each
// operand's upload) let each prime's forward columns of a start while b is
// still being copied.
void ntt_launch_4step(int set, const ProdArgs& args, cudaStream_t st, cudaEvent_t* ev = nullptr,
                      const PrimeStreams* ps = nullptr, cudaEvent_t a_ready = nullptr,
                      cudaEvent_t b_ready = nullptr, const CrtChunks* chunks = nullptr);
// the batch form: `count` products of one length class (class-wide fields
// from `args`, per-product fields from the device array `batch`);
// max_nblk = the largest carry grid of the class
void ntt_launch_4step_batch(int set, const ProdArgs& args, const ProdPtrs* batch, int count, int max_nblk,
                            cudaStream_t st);
int ntt_row_threads(int k2, int n1, int* rows);
// SMs of the current device (cudaDevAttrMultiProcessorCount, cached per
// device); GB300's 152 where no device answers (plan queries on a host
// without a GPU)
int device_sm_count();
int ntt_configure_kernels();  // opt-in shared-memory sizes; returns a cudaError_t

// launchers of each translation unit (ntt_cols.cu, ntt_rows.cu, ntt_carry.cu, ntt_small.cu)
// (primes a.prime0 .. a.prime0 + nprimes - 1; 0 = every prime of the set).
// The row and inverse column kernels of sets 2 and 3 are those of sets 0
// and 1: the same arithmetic on residues, with their primes and tables in a.f.
void launch_fwd_cols(int set, const ProdArgs& a, cudaStream_t st, const ProdPtrs* batch = nullptr, int count = 1,
                     int nprimes = 0);
void launch_rows(int set, const ProdArgs& a, cudaStream_t st, const ProdPtrs* batch = nullptr, int count = 1,
                 int nprimes = 0);
void launch_inv_cols(int set, const ProdArgs& a, cudaStream_t st, const ProdPtrs* batch = nullptr, int count = 1,
                     int nprimes = 0);
// (nblk_launch: the blocks of one chunk of a chunked CRT, a.crt_blk0 ..)
void launch_crt_carry(int set, const ProdArgs& a, cudaStream_t st, const ProdPtrs* batch = nullptr, int count = 1,
                      int max_nblk = 0, int nblk_launch = 0);
int configure_fwd_cols();
int configure_inv_cols();

// Column-pass configuration instantiated for (set, m = log2 N1) closest to
// the requested columns per CTA and radix cap (0 = default: 8 columns,
// radix cap 6).  The radix cap only changes the schedule of 2^10- and
// 2^11-point columns; set 1's 2^12- and 2^13-point columns take 4 columns.
// Row-pass radix cap instantiated for m = log2 N2 (0 = default): the cap
// changes the schedule of 2^10- and 2^11-point rows only; by default 2^10
// rows run as two radix-32 passes (7% faster on GB300) and 2^11 rows as
// radix-8, -8, -32 passes (a radix-64 pass costs them registers).
inline int row_radix_cap(int m, int req) {
    if (m != 10 && m != 11) return 4;
    return req == 4 || req == 6 ? req : (m == 10 ? 6 : 4);
}

inline void col_config(int set, int m, int req_cg, int req_mr, int& cg, int& mr) {
    set = set_base(set);
    cg = (req_cg == 4 || req_cg == 8) ? req_cg : kColGroup;
    if (set == 1 && m >= 12) cg = 4;
    mr = (m == 10 || m == 11) && req_mr == 4 ? 4 : 6;
}
int configure_rows();
int configure_small();
int configure_class();

// The batch form's persistent kernel per length class (ntt_class.cu): its
// scheduling words, zeroed before each launch, are kClassHdrWords (the next
// work item, the abort word) then kClassProdWords per product (forward
// column tiles done per prime, row tiles done per prime, inverse column
// tiles done).
constexpr int kClassHdrWords = 2;
constexpr int kClassProdWords = 7;
struct ClassRun {
    uint32_t* sched;      // the scheduling words
    int count;            // products of this launch (entries of the descriptor array)
    int max_nblk;         // carry blocks of its longest product
    int rows;             // row slots per row tile (class_rows)
    uint32_t spin_limit;  // polls before a dependency wait gives up (about 0.25 us each)
    int never_signal;     // tests: forward tiles leave their counters untouched
};
// row slots per row tile of the class kernel (256 threads)
int class_rows(int k1, int k2);
// one launch of the class kernel for `run.count` products of batch; -1 when
// the configuration is not instantiated
int launch_class_persistent(const ProdArgs& a, const ProdPtrs* batch, const ClassRun& run, cudaStream_t st);

// out[0 .. n) += t[0 .. nt) (nt <= n), the carry running on into out's
// higher limbs (ntt_add.cu); scratch holds add_into_scratch_words(nt)
// words; a carry past out[n - 1] sets kDevErrCarry in *err
size_t add_into_scratch_words(uint64_t nt);
void launch_add_into(uint64_t* out, uint64_t n, const uint64_t* t, uint64_t nt, uint32_t* scratch, int* err,
                     cudaStream_t st);

}  // namespace precgpu
