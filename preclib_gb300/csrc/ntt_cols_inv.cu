// ntt_cols_inv.cu -- instantiations and launcher of the inverse column
// kernel (k_inv_cols, ntt_cols.cuh).
#include "ntt_cols.cuh"

namespace precgpu {

void launch_inv_cols(int set, const ProdArgs& a, cudaStream_t st, const ProdPtrs* batch, int count, int nprimes) {
    if (nprimes <= 0) nprimes = kSetPrimes[set];
    set = set_base(set);  // sets 2 and 3: the same kernel on their residues
    int cg, mr;
    col_config(set, a.k1, a.cg, a.cmr, cg, mr);
    const dim3 grid((1u << a.k2) / cg, nprimes, count);
    const size_t smem = col_smem(a.k1, cg);
    if (launch_inv_cols_k2(set, a, cg, mr, grid, smem, st, batch)) {
        count_launches(1);
        return;
    }
#define X(S, MM, CC, RR)                                                     \
    if (set == S && a.k1 == MM && cg == CC && mr == RR) {                     \
        launch_kernel(k_inv_cols<S, MM, CC, RR>, grid, 32 * CC, smem, st, a, batch); \
        count_launches(1);                                                  \
        return;                                                             \
    }
    PREC_COLS_CONFIGS(X)
#undef X
}

int configure_inv_cols() {
    cudaError_t e = (cudaError_t)configure_inv_cols_k2();
#define X(S, MM, CC, RR)                                                                                   \
    if (!e) e = cudaFuncSetAttribute(k_inv_cols<S, MM, CC, RR>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                     (int)col_smem(MM, CC));
    PREC_COLS_CONFIGS(X)
#undef X
    return (int)e;
}

}  // namespace precgpu
