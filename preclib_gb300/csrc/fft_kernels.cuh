// fft_kernels.cuh -- FP64 FFT band: arguments and launchers.
#pragma once
#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

#include "ntt_kernels.cuh"

namespace precgpu {

constexpr int kFftMaxLog2 = 16;     // largest FP64 transform (6144 x 6144 limbs fits)
constexpr int kDevErrFftRound = 4;  // device error bit: max distance above 0.25

struct FftArgs {
    const uint64_t* a;
    const uint64_t* bp;
    uint64_t* out;
    double2* work;        // N complex values
    long long* coef;      // N rounded coefficients
    double* maxdist;      // max |x - round(x)| of this product
    int* err;
    const double2* tw;    // e^(2 pi i e / 2^16), e < 2^15
    uint64_t la, lb, lout;
    uint64_t da, db;      // balanced digit counts
    uint64_t ncoef;       // N
    int b;                // digit width in bits
    int k, k1, k2;        // log2 N = k1 + k2 (column length 2^k1, row length 2^k2)
};

constexpr int fpad_host(int i) { return i + (i >> 4); }

size_t fft_table_bytes();
void fft_build_table(double2* tw, cudaStream_t st);
int fft_configure_kernels();
// The product's 4 kernels: the first takes the arguments by value and
// stores them at `d_args` (device) for the others; one graph replay
// (built for `cap` once per length and argument buffer), or, with `ev`
// (or without `cap`), plain launches with an event before the first and
// after each.  Returns a cudaError_t.  The caller runs one product at a
// time per argument buffer (its library lane's lock).
int fft_launch(const FftArgs& f, FftArgs* d_args, cudaStream_t st, cudaEvent_t* ev = nullptr,
               cudaStream_t cap = nullptr);
// destroys the cached graphs of one argument buffer (a lane's), or all
void fft_release_graphs(const FftArgs* d_args = nullptr);

}  // namespace precgpu
