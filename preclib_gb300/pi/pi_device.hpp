// pi_device.hpp -- device-side signed sums of the binary-splitting tree.
//
// A level of the tree forms every parent's T = Tl*Qr + Tr*Pl from the two
// products and the children's signs.  With the level's values resident in
// device memory, the sums run on the device too: one call adds (or
// subtracts, by sign) any number of pairs of magnitudes, each pair cut into
// chunks of kAddChunkLimbs limbs (pi_kernels.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace precpi {

constexpr int kAddThreads = 256;
constexpr int kAddLimbsPerThread = 4;
constexpr uint32_t kAddChunkLimbs = kAddThreads * kAddLimbsPerThread;

// z = (-1)^*sx x + (-1)^*sy y for magnitudes x (nx limbs) and y (ny limbs);
// z has nz = max(nx, ny) + 1 limbs and its sign goes to *sz.
struct AddPair {
    const uint64_t* x;
    const uint64_t* y;
    uint64_t* z;
    const int8_t* sx;
    const int8_t* sy;
    int8_t* sz;
    uint32_t nx, ny, nz;
    uint32_t chunk0;  // first entry of this pair in the chunk table
};

inline uint32_t add_chunks(uint32_t nz) { return (nz + kAddChunkLimbs - 1) / kAddChunkLimbs; }

// Device scratch of one call: top[npairs] (int64), agg[nchunks] (uint8)
// and a counter.
size_t signed_add_scratch_bytes(size_t npairs, size_t nchunks);

// Enqueues the sums of `npairs` pairs (device array) on `st`; chunk_pair
// (device, nchunks entries) maps chunk -> pair, in pair order.
cudaError_t signed_add_many(const AddPair* pairs, size_t npairs, const uint32_t* chunk_pair, size_t nchunks,
                            void* scratch, cudaStream_t st);

// kernels launched by signed_add_many so far
uint64_t signed_add_launches();

}  // namespace precpi
