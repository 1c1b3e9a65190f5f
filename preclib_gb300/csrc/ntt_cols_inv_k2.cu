// ntt_cols_inv_k2.cu -- the inverse column kernels of the default
// configurations compiled for their constant row length
// (PREC_COLS_INV_K2_CONFIGS, ntt_cols.cuh).
#include "ntt_cols.cuh"

namespace precgpu {

bool launch_inv_cols_k2(int set, const ProdArgs& a, int cg, int mr, dim3 grid, size_t smem, cudaStream_t st,
                        const ProdPtrs* batch) {
#define X(S, MM, CC, RR, KK)                                                                   \
    if (set == S && a.k1 == MM && cg == CC && mr == RR && a.k2 == KK) {                         \
        launch_kernel(k_inv_cols<S, MM, CC, RR, KK>, grid, 32 * CC, smem, st, a, batch);        \
        return true;                                                                            \
    }
    PREC_COLS_INV_K2_CONFIGS(X)
#undef X
    return false;
}

int configure_inv_cols_k2() {
    cudaError_t e = cudaSuccess;
#define X(S, MM, CC, RR, KK)                                                                             \
    if (!e) e = cudaFuncSetAttribute(k_inv_cols<S, MM, CC, RR, KK>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                     (int)col_smem(MM, CC));
    PREC_COLS_INV_K2_CONFIGS(X)
#undef X
    return (int)e;
}

}  // namespace precgpu
