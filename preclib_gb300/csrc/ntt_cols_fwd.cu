// ntt_cols_fwd.cu -- instantiations and launcher of the forward column
// kernel (k_fwd_cols, ntt_cols.cuh).
#include "ntt_cols.cuh"

namespace precgpu {

void launch_fwd_cols(int set, const ProdArgs& a, cudaStream_t st, const ProdPtrs* batch, int count, int nprimes) {
    if (nprimes <= 0) nprimes = kSetPrimes[set];
    int cg, mr;
    col_config(set_base(set), a.k1, a.cg, a.cmr, cg, mr);
    const dim3 grid((1u << a.k2) / cg, (a.square || a.operand_only ? 1 : 2) * nprimes, count);
    const size_t smem = col_smem(a.k1, cg);
    // one prime of a single product's per-prime chains on the first
    // five-prime set at 2^10-point columns (the 1M x 1M class), both operands
    // at once: the pipelined kernel.  (On set 3's 4M x 4M it measured slower,
    // 0.723 -> 0.735 ms; for the host-pointer form's launches of one uploaded
    // operand each, e2e 0.344 -> 0.353 ms.)
    if (nprimes == 1 && !batch && !a.operand_only && a.k1 == 10 && cg == 8 && mr == 6 && set == kWideSet) {
        const dim3 pg((grid.x + kFwdPipeTiles - 1) / kFwdPipeTiles, grid.y, grid.z);
        launch_kernel(k_fwd_cols_pipe<kWideSet, 10, 8, 6>, pg, 256, 2 * smem, st, a, batch);
        count_launches(1);
        return;
    }
#define X(S, MM, CC, RR)                                                     \
    if (set == S && a.k1 == MM && cg == CC && mr == RR) {                     \
        launch_kernel(k_fwd_cols<S, MM, CC, RR>, grid, 32 * CC, smem, st, a, batch); \
        count_launches(1);                                                  \
        return;                                                             \
    }
    PREC_COLS_CONFIGS(X)
    PREC_COLS_WIDE_CONFIGS(X)
#undef X
}

int configure_fwd_cols() {
    cudaError_t e = cudaSuccess;
    e = cudaFuncSetAttribute(k_fwd_cols_pipe<kWideSet, 10, 8, 6>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(2 * col_smem(10, 8)));
#define X(S, MM, CC, RR)                                                                                   \
    if (!e) e = cudaFuncSetAttribute(k_fwd_cols<S, MM, CC, RR>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                     (int)col_smem(MM, CC));
    PREC_COLS_CONFIGS(X)
    PREC_COLS_WIDE_CONFIGS(X)
#undef X
    return (int)e;
}

}  // namespace precgpu
