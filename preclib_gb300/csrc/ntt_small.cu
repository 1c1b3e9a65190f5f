// ntt_small.cu -- single-CTA products (transforms of 2^5 .. 2^12 points).
//
// One CTA runs the whole of the reference's mul_ntt (src/mul_ntt.cpp:494-518)
// for one product in shared memory: digits of both operands, forward DIF,
// pointwise product and inverse DIT for each of the three primes, then CRT
// and the carry chain (block-wide scan).  With a descriptor array the same
// kernel runs one product per CTA for a whole batch of a length class.
#include "ntt_engine.cuh"

namespace precgpu {

// coefficient i of the product from the three residue arrays (0 outside)
template <int M>
__device__ __forceinline__ u128 small_coef(const uint32_t* sm, int64_t i, const CrtConst& cc, const FieldArgs& f) {
    constexpr int AS = astride_for(M);
    if (i < 0 || i >= (1 << M)) return 0;
    const int pi = padded((int)i);
    return crt3(sm[2 * AS + pi], sm[3 * AS + pi], sm[4 * AS + pi], cc, f);
}

template <int M>
__global__ void __launch_bounds__(256) k_small(const SmallDesc* __restrict__ descs, SmallDesc single, FieldArgs f,
                                               CrtConst crt) {
    extern __shared__ uint32_t sm[];
    __shared__ BlockCarryShared sh;
    constexpr int NP = sch_np(M);
    constexpr int AS = astride_for(M);
    const SmallDesc d = descs ? descs[blockIdx.x] : single;
    const uint32_t* __restrict__ da = reinterpret_cast<const uint32_t*>(d.a);
    const uint32_t* __restrict__ db = reinterpret_cast<const uint32_t*>(d.b);
    const uint64_t nda = 2 * d.la, ndb = 2 * d.lb;

    for (int prime = 0; prime < kPrimes; ++prime) {
        const PrimeC pc = f.pc[prime];
        const uint2* __restrict__ twf = f.tf[prime];
        const uint2* __restrict__ twi = f.ti[prime];
        uint32_t* res = sm + (2 + prime) * AS;
        if constexpr (NP == 1) {
            // 32 points: one register pass does everything
            if (threadIdx.x == 0) {
                uint32_t x[2][32];
#pragma unroll
                for (int q = 0; q < 32; ++q) {
                    x[0][q] = (uint64_t)q < nda ? Ar<0>::digit(__ldg(&da[q]), pc) : 0u;
                    x[1][q] = (uint64_t)q < ndb ? Ar<0>::digit(__ldg(&db[q]), pc) : 0u;
                }
                regs_pass<0, M, 0, false, 2>(x, 0, twf, pc);
                uint32_t y[1][32];
#pragma unroll
                for (int q = 0; q < 32; ++q) y[0][q] = Ar<0>::mul(x[0][q], x[1][q], pc);
                regs_pass<0, M, 0, true, 1>(y, 0, twi, pc);
#pragma unroll
                for (int q = 0; q < 32; ++q) res[q] = y[0][q];
            }
        } else {
            {   // top DIF pass from the limbs
                using G = Geom<M, 0>;
                for (int w = threadIdx.x; w < (1 << G::LGI); w += blockDim.x) {
                    const uint32_t u = w;
                    const uint32_t base = G::base(u);
                    uint32_t x[2][G::R];
#pragma unroll
                    for (int q = 0; q < G::R; ++q) {
                        const uint32_t i = base + ((uint32_t)q << G::LO);
                        x[0][q] = i < nda ? Ar<0>::digit(__ldg(&da[i]), pc) : 0u;
                        x[1][q] = i < ndb ? Ar<0>::digit(__ldg(&db[i]), pc) : 0u;
                    }
                    regs_pass<0, M, 0, false, 2>(x, u, twf, pc);
                    uint32_t* s = sm + G::pbase(u);
#pragma unroll
                    for (int q = 0; q < G::R; ++q) {
                        s[q * G::QS] = x[0][q];
                        s[AS + q * G::QS] = x[1][q];
                    }
                }
                __syncthreads();
            }
            row_passes<0, M, 1, NP - 2, false, 2>(sm, AS, 2, twf, pc);
            {   // bottom: last DIF stages, product, first DIT stages
                using G = Geom<M, NP - 1>;
                for (int w = threadIdx.x; w < (1 << G::LGI); w += blockDim.x) {
                    const uint32_t u = w;
                    uint32_t* s = sm + 33 * u;
                    uint32_t x[2][32];
#pragma unroll
                    for (int q = 0; q < 32; ++q) {
                        x[0][q] = s[q];
                        x[1][q] = s[AS + q];
                    }
                    regs_pass<0, M, NP - 1, false, 2>(x, u, twf, pc);
                    uint32_t y[1][32];
#pragma unroll
                    for (int q = 0; q < 32; ++q) y[0][q] = Ar<0>::mul(x[0][q], x[1][q], pc);
                    regs_pass<0, M, NP - 1, true, 1>(y, u, twi, pc);
#pragma unroll
                    for (int q = 0; q < 32; ++q) s[q] = y[0][q];
                }
                __syncthreads();
            }
            row_passes<0, M, NP - 2, 1, true, 1>(sm, AS, 1, twi, pc);
            {   // top DIT pass into this prime's residue array
                using G = Geom<M, 0>;
                for (int w = threadIdx.x; w < (1 << G::LGI); w += blockDim.x) {
                    const uint32_t u = w;
                    const uint32_t pb = G::pbase(u);
                    uint32_t x[1][G::R];
#pragma unroll
                    for (int q = 0; q < G::R; ++q) x[0][q] = sm[pb + q * G::QS];
                    regs_pass<0, M, 0, true, 1>(x, u, twi, pc);
#pragma unroll
                    for (int q = 0; q < G::R; ++q) res[pb + q * G::QS] = x[0][q];
                }
            }
        }
        __syncthreads();
    }

    // CRT + carries over the block, L limbs per thread per round
    constexpr int L = 8;
    bool carry = false;
    for (int64_t r0 = 0; r0 < (int64_t)d.lout; r0 += (int64_t)blockDim.x * L) {
        const int64_t m0 = r0 + threadIdx.x * L;
        u128 T[L];
#pragma unroll
        for (int k = 0; k < L; ++k)
            T[k] = small_coef<M>(sm, 2 * (m0 + k), crt, f) + (small_coef<M>(sm, 2 * (m0 + k) + 1, crt, f) << 32);
        uint64_t prev_hi = 0;
        if (m0 > 0) {
            const u128 tp = small_coef<M>(sm, 2 * m0 - 2, crt, f) + (small_coef<M>(sm, 2 * m0 - 1, crt, f) << 32);
            prev_hi = (uint64_t)(tp >> 64);
        }
        uint64_t v[L];
        uint32_t gbits;
        bool G, P;
        limbs_from_sums<L>(T, prev_hi, v, gbits, G, P);
        auto cin_fn = [&](bool Gb, bool Pb) -> bool {
            sh.block_cin = (Gb || (Pb && carry)) ? 1u : 0u;
            return carry;
        };
        const bool cin = block_carry(G, P, sh, cin_fn);
        limbs_finish<L>(m0, d.lout, v, gbits, cin, d.out);
        __syncthreads();
        carry = sh.block_cin != 0;
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------

size_t ntt_small_smem_bytes(int k) { return (size_t)5 * astride_for(k) * sizeof(uint32_t); }

int ntt_small_threads(int k) {
    int t = 1 << (k > 3 ? k - 3 : 0);
    return t < 64 ? 64 : (t > 256 ? 256 : t);
}

#define PREC_SMALL(X) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12)

void ntt_launch_small(const SmallDesc* d_descs, const SmallDesc* single, int count, int k, const FieldArgs& f,
                      const CrtConst& crt, cudaStream_t st, cudaEvent_t* ev) {
    SmallDesc one{};
    if (single) one = *single;
    if (ev) cudaEventRecord(ev[0], st);
    const int threads = ntt_small_threads(k);
    const size_t smem = ntt_small_smem_bytes(k);
#define X(MM) \
    if (k == MM) {                                                     \
        launch_kernel(k_small<MM>, count, threads, smem, st, d_descs, one, f, crt); \
        count_launches(1);                                             \
    }
    PREC_SMALL(X)
#undef X
    if (ev) cudaEventRecord(ev[1], st);
}

int configure_small() {
    cudaError_t e = cudaSuccess;
#define X(MM)                                                                                    \
    if (!e) e = cudaFuncSetAttribute(k_small<MM>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                     (int)ntt_small_smem_bytes(MM));
    PREC_SMALL(X)
#undef X
    return (int)e;
}

}  // namespace precgpu
