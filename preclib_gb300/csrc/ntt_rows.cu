// ntt_rows.cu -- the row kernel of the four-step NTT (one tile of
// rows_tile, ntt_rows.cuh, per CTA), its instantiations and launcher.
// pass radix cap of the row transforms (radix-8/16 passes: two operands'
// radix-64 items would not fit the register budget)
#ifndef PREC_ROWS_MAXRB
#define PREC_ROWS_MAXRB 4
#endif
#ifndef PREC_SCH_MAXRB
#define PREC_SCH_MAXRB PREC_ROWS_MAXRB
#endif
#include "ntt_rows.cuh"

// threads of a row-pass CTA (rows x 2^(M-5)), at most 256: one 2^11-point
// row per 64-thread CTA syncs only its own two warps (13% faster than four
// rows per 256-thread CTA on GB300)
#ifndef PREC_ROWS_THREADS
#define PREC_ROWS_THREADS 64
#endif

namespace precgpu {

template <int SET, int M, bool SQ, int MR>
__global__ void __launch_bounds__(256, MR == 6 ? 2 : PREC_ROWS_MINB) k_rows(ProdArgs args, const ProdPtrs* __restrict__ batch) {
    extern __shared__ uint32_t sm[];
    rows_tile<SET, M, SQ, MR>(args, batch, GridIdx{}, sm);
}

// ---------------------------------------------------------------------------

static size_t row_smem(int m, int rows) { return (size_t)rows * 2 * astride_for(m) * sizeof(uint32_t); }

// rows per CTA: PREC_ROWS_THREADS / 2^(M-5), fewer when the transform has
// too few rows to fill the GPU, never under one warp
int ntt_row_threads(int k2, int n1, int* rows_out) {
    int rows = PREC_ROWS_THREADS >> (k2 - 5);
    if (rows < 1) rows = 1;
    const int sms = device_sm_count();
    while (rows > 1 && (n1 / rows) * kPrimes < 2 * sms) rows >>= 1;
    int min_rows = k2 >= 10 ? 1 : (1 << (10 - k2));  // >= 32 threads
    if (rows < min_rows) rows = min_rows;
    if (rows > n1) rows = n1;
    *rows_out = rows;
    return rows << (k2 - 5);
}

// (set, M, radix cap): the cap changes the schedule of 2^10- and 2^11-point rows only
#define PREC_ROWS1(X, SQ)                                                                                      \
    X(0, 7, SQ, 4) X(0, 8, SQ, 4) X(0, 9, SQ, 4) X(0, 10, SQ, 4) X(0, 10, SQ, 6) X(0, 11, SQ, 4) X(0, 11, SQ, 6) \
    X(0, 12, SQ, 4) X(1, 13, SQ, 4)
#define PREC_ROWS(X) PREC_ROWS1(X, false) PREC_ROWS1(X, true)

void launch_rows(int set, const ProdArgs& a, cudaStream_t st, const ProdPtrs* batch, int count, int nprimes) {
    if (nprimes <= 0) nprimes = kSetPrimes[set];
    set = set_base(set);  // sets 2 and 3: the same kernel on their residues
    const int m = a.k2;
    const dim3 grid((1u << a.k1) / a.rows, nprimes, count);
    const int threads = a.rows << (m - 5);
    const size_t smem = row_smem(m, a.rows);
    const int mr = row_radix_cap(m, a.rmr);
#define X(S, MM, SQ, RR)                                                                  \
    if (set == S && m == MM && (a.square != 0) == SQ && mr == RR) {                       \
        launch_kernel(k_rows<S, MM, SQ, RR>, grid, threads, smem, st, a, batch);                 \
        count_launches(1);                                                              \
        return;                                                                         \
    }
    PREC_ROWS(X)
#undef X
}

int configure_rows() {
    cudaError_t e = cudaSuccess;
#define X(S, MM, SQ, RR)                                                                                      \
    if (!e) e = cudaFuncSetAttribute(k_rows<S, MM, SQ, RR>, cudaFuncAttributeMaxDynamicSharedMemorySize,     \
                                     (int)row_smem(MM, 256 >> (MM - 5) > 0 ? 256 >> (MM - 5) : 1));
    PREC_ROWS(X)
#undef X
    return (int)e;
}

}  // namespace precgpu
