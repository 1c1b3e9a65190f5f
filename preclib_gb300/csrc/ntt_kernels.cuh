// ntt_kernels.cuh -- shared declarations between the NTT kernels and the host.
#pragma once
#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

#include "ntt_field.cuh"

namespace precgpu {

// CRT constants of one transform length (Garner with the transform's
// scaling folded in; see crt3 in ntt_kernels.cu).
struct CrtConst {
    ShoupC s1, k21, k22, k31, k32, k33;
};

// Device tables of the three primes (set once per device).
struct TableSet {
    const uint2* tf[kPrimes];      // tf[(1<<b)+j] = (w_{2^{b+1}}^j, Shoup), b < 13
    const uint2* ti[kPrimes];      // ti[(1<<b)+j] = (w_{2^{b+1}}^{-j}, Shoup)
    const uint32_t* twhi[kPrimes]; // w_{2^26}^{h*2^13} * 2^32 mod p, h < 2^13
    const uint32_t* twlo[kPrimes]; // w_{2^26}^{l} * 2^32 mod p, l < 2^13
};

// One product of the multi-pass (four-step) path.
struct ProdArgs {
    const uint64_t* a;
    const uint64_t* b;
    uint64_t* out;
    uint32_t* work;     // [prime][operand][N] residues
    uint32_t* scratch;  // carry look-back: [0] block ticket, [1..nblk] status words
    int* err;           // error bits (PREC_GPU_DEVERR_*)
    uint64_t la, lb, lout;
    int k, k1, k2;      // log2 of N, of the column length N1, of the row length N2
    int nblk;           // blocks of the carry kernel
    CrtConst crt;
};

// One product of the single-CTA path (small transforms, also the batch
// form's small length classes).
struct SmallDesc {
    const uint64_t* a;
    const uint64_t* b;
    uint64_t* out;
    uint64_t la, lb, lout;
    int k;
    int pad;
    CrtConst crt;
};

// device error bits
constexpr int kDevErrTimeout = 1;
constexpr int kDevErrCarry = 2;

// host-side launchers (ntt_kernels.cu)
void ntt_set_tables(const PrimeC* primes, const TableSet& tabs);
int ntt_small_max_log2();
size_t ntt_small_smem_bytes(int k);
// d_descs: device array of `count` products, or null with `single` (by value)
void ntt_launch_small(const SmallDesc* d_descs, const SmallDesc* single, int count, int k, cudaStream_t st);
void ntt_launch_4step(const ProdArgs& args, cudaStream_t st);
int ntt_carry_block_limbs();
int ntt_configure_kernels();  // opt-in shared memory sizes; returns cudaError_t

}  // namespace precgpu
