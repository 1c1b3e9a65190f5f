// prec_gpu_internal.h -- library-internal interface between the host-side
// translation units (context and plans in prec_gpu_host.cu; batch form in
// prec_gpu_batch.cu; serving loop in prec_gpu_serve.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <mutex>

#include "ntt_kernels.cuh"

namespace precgpu {

// transform plan of one product on the NTT band
struct Plan {
    int k = 0, k1 = 0, k2 = 0;
    int set = 0;
    int path = 0;  // 0 single CTA, 1 four-step
    int nblk = 0;
    int rows = 0;  // rows per CTA of the row pass
    CrtConst crt{};
    size_t work_bytes = 0;  // work buffer + carry words of the four-step path
};

// da, db: 32-bit digit counts (upper bounds are fine); lout = La + Lb
int plan_for(uint64_t da, uint64_t db, uint64_t lout, Plan& pl);

// the process-wide context: its lock, initialisation (idempotent, call
// with the lock held), prime-set tables and device error word
std::mutex& ctx_mutex();
int ctx_init_locked(int device);
const FieldArgs& ctx_field(int set);
int* ctx_device_err();

int cuda_code(cudaError_t e);

}  // namespace precgpu
