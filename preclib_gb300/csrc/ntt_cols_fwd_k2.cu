// ntt_cols_fwd_k2.cu -- the forward column kernels of the default
// configurations compiled for their constant row length
// (PREC_COLS_FWD_K2_CONFIGS, ntt_cols.cuh), and the pipelined forward
// columns of the 1M x 1M class.
#include "ntt_cols.cuh"

namespace precgpu {

bool launch_fwd_cols_k2(int set, const ProdArgs& a, int cg, int mr, dim3 grid, size_t smem, cudaStream_t st,
                        const ProdPtrs* batch, bool one_prime) {
    // one prime of a single product's per-prime chains on the first
    // five-prime set at 2^10 x 2^11 points (the 1M x 1M class), both
    // operands at once: the pipelined kernel (1M x 1M 0.1690 -> 0.1672 ms
    // against the one-tile kernel).  On set 3's 4M x 4M it measured slower
    // (0.688 -> 0.705 ms), and so did the host-pointer form's launches of
    // one uploaded operand each (e2e 0.344 -> 0.353 ms).
    if (one_prime && !batch && !a.operand_only && set == kWideSet && a.k1 == 10 && a.k2 == 11 && cg == 8 &&
        mr == 6) {
        const dim3 pg((grid.x + kFwdPipeTiles - 1) / kFwdPipeTiles, grid.y, grid.z);
        launch_kernel(k_fwd_cols_pipe<kWideSet, 10, 8, 6, 11>, pg, 256, 2 * smem, st, a, batch);
        return true;
    }
#define X(S, MM, CC, RR, KK)                                                                   \
    if (set == S && a.k1 == MM && cg == CC && mr == RR && a.k2 == KK) {                         \
        launch_kernel(k_fwd_cols<S, MM, CC, RR, KK>, grid, 32 * CC, smem, st, a, batch);        \
        return true;                                                                            \
    }
    PREC_COLS_FWD_K2_CONFIGS(X)
#undef X
    return false;
}

int configure_fwd_cols_k2() {
    cudaError_t e = cudaFuncSetAttribute(k_fwd_cols_pipe<kWideSet, 10, 8, 6, 11>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(2 * col_smem(10, 8)));
#define X(S, MM, CC, RR, KK)                                                                             \
    if (!e) e = cudaFuncSetAttribute(k_fwd_cols<S, MM, CC, RR, KK>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                     (int)col_smem(MM, CC));
    PREC_COLS_FWD_K2_CONFIGS(X)
#undef X
    return (int)e;
}

}  // namespace precgpu
