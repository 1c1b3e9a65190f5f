// ntt_carry.cu -- CRT recombination and carry propagation of the four-step
// path: the reference's ntt_crt2/ntt_crt3 and serial ntt_from_residues
// carry loop (src/mul_ntt.cpp:405-487) as one pass over the natural-order
// residues with a decoupled look-back scan for the carries.
//
// Each thread turns 8 coefficients into 4 limbs; the limb carry chain is
// resolved per warp (ballot), per block, then across blocks: a block whose
// limbs cannot pass a carry through publishes its carry-out at once, the
// others publish their (G, P) aggregate and look back.  Blocks take their
// position from a ticket counter, so a block only waits on blocks already
// running, and every wait is bounded (kSpinLimit polls, then an error bit).
#include "ntt_engine.cuh"

namespace precgpu {

constexpr int kSpinLimit = 1 << 20;

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(uint32_t* p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <int SET>
__global__ void __launch_bounds__(kCarryThreads) k_crt_carry(ProdArgs args) {
    __shared__ BlockCarryShared sh;
    __shared__ uint32_t s_ticket;
    if (threadIdx.x == 0) s_ticket = atomicAdd(&args.scratch[0], 1u);
    __syncthreads();
    const uint32_t bid = s_ticket;
    const uint64_t N = 1ull << args.k;
    const uint32_t* __restrict__ r0 = args.work;
    const uint32_t* __restrict__ r1 = args.work + 2 * N;
    const uint32_t* __restrict__ r2 = args.work + 4 * N;
    const int lane = threadIdx.x & 31;
    const int64_t m0 = (int64_t)bid * (kCarryThreads * kCarryLimbs) + threadIdx.x * kCarryLimbs;
    const uint64_t i0 = 2 * (uint64_t)m0;

    u128 T[kCarryLimbs];
    if (i0 + 2 * kCarryLimbs <= N) {
        uint32_t y[3][2 * kCarryLimbs];
#pragma unroll
        for (int h = 0; h < 2 * kCarryLimbs / 4; ++h) {
            const uint4 a = __ldg(reinterpret_cast<const uint4*>(r0 + i0) + h);
            const uint4 b = __ldg(reinterpret_cast<const uint4*>(r1 + i0) + h);
            const uint4 c = __ldg(reinterpret_cast<const uint4*>(r2 + i0) + h);
            y[0][4 * h] = a.x; y[0][4 * h + 1] = a.y; y[0][4 * h + 2] = a.z; y[0][4 * h + 3] = a.w;
            y[1][4 * h] = b.x; y[1][4 * h + 1] = b.y; y[1][4 * h + 2] = b.z; y[1][4 * h + 3] = b.w;
            y[2][4 * h] = c.x; y[2][4 * h + 1] = c.y; y[2][4 * h + 2] = c.z; y[2][4 * h + 3] = c.w;
        }
#pragma unroll
        for (int k = 0; k < kCarryLimbs; ++k) {
            const u128 c0 = crt3(y[0][2 * k], y[1][2 * k], y[2][2 * k], args.crt, args.f);
            const u128 c1 = crt3(y[0][2 * k + 1], y[1][2 * k + 1], y[2][2 * k + 1], args.crt, args.f);
            T[k] = c0 + (c1 << 32);
        }
    } else {
#pragma unroll
        for (int k = 0; k < kCarryLimbs; ++k) {
            u128 c[2];
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const uint64_t i = i0 + 2 * k + e;
                c[e] = i < N ? crt3(r0[i], r1[i], r2[i], args.crt, args.f) : (u128)0;
            }
            T[k] = c[0] + (c[1] << 32);
        }
    }
    // hi(T) of the limb just below this thread's first limb
    uint64_t prev_hi = __shfl_up_sync(0xffffffffu, (uint64_t)(T[kCarryLimbs - 1] >> 64), 1);
    if (lane == 0) {
        prev_hi = 0;
        if (m0 > 0 && i0 - 1 < N) {
            const u128 c0 = crt3(r0[i0 - 2], r1[i0 - 2], r2[i0 - 2], args.crt, args.f);
            const u128 c1 = crt3(r0[i0 - 1], r1[i0 - 1], r2[i0 - 1], args.crt, args.f);
            prev_hi = (uint64_t)((c0 + (c1 << 32)) >> 64);
        }
    }
    uint64_t v[kCarryLimbs];
    uint32_t gbits;
    bool G, P;
    limbs_from_sums<kCarryLimbs>(T, prev_hi, v, gbits, G, P);

    uint32_t* status = args.scratch + 1;
    auto cin_fn = [&](bool Gb, bool Pb) -> bool {
        // status word: bit0 aggregate ready, bit1 carry-out ready,
        // bit2 G (or the carry-out), bit3 P
        if (bid == 0) {
            st_release(&status[0], 2u | (Gb ? 4u : 0u));
            return false;
        }
        if (!Pb) st_release(&status[bid], 2u | (Gb ? 4u : 0u));
        else st_release(&status[bid], 1u | (Gb ? 4u : 0u) | 8u);
        bool accG = false, accP = true, cin = false;
        for (int64_t j = (int64_t)bid - 1; j >= 0; --j) {
            uint32_t s = 0;
            int spins = 0;
            while (((s = ld_acquire(&status[j])) & 3u) == 0) {
                if (++spins > kSpinLimit) {
                    atomicOr(args.err, kDevErrTimeout);
                    s = 2u;  // give up with carry 0; the error bit fails the product
                    break;
                }
                __nanosleep(64);
            }
            const bool g = (s & 4u) != 0;
            if (s & 2u) {
                cin = accG || (accP && g);
                break;
            }
            accG = accG || (accP && g);
            accP = accP && ((s & 8u) != 0);
        }
        if (Pb) st_release(&status[bid], 2u | ((Gb || cin) ? 4u : 0u));
        return cin;
    };
    const bool cin = block_carry(G, P, sh, cin_fn);
    limbs_finish<kCarryLimbs>(m0, args.lout, v, gbits, cin, args.out);
    if (bid + 1 == gridDim.x && threadIdx.x == blockDim.x - 1) {
        bool c = cin;
#pragma unroll
        for (int k = 0; k < kCarryLimbs; ++k) c = ((gbits >> k) & 1) || (v[k] == ~0ull && c);
        if (c) atomicOr(args.err, kDevErrCarry);  // a product never overflows La+Lb limbs
    }
}

void launch_crt_carry(int set, const ProdArgs& a, cudaStream_t st) {
    if (set == 0) k_crt_carry<0><<<a.nblk, kCarryThreads, 0, st>>>(a);
    else k_crt_carry<1><<<a.nblk, kCarryThreads, 0, st>>>(a);
}

void ntt_launch_4step(int set, const ProdArgs& args, cudaStream_t st, cudaEvent_t* ev) {
    if (ev) cudaEventRecord(ev[0], st);
    launch_fwd_cols(set, args, st);
    if (ev) cudaEventRecord(ev[1], st);
    launch_rows(set, args, st);
    if (ev) cudaEventRecord(ev[2], st);
    launch_inv_cols(set, args, st);
    if (ev) cudaEventRecord(ev[3], st);
    launch_crt_carry(set, args, st);
    if (ev) cudaEventRecord(ev[4], st);
}

int ntt_configure_kernels() {
    int e = configure_cols();
    if (!e) e = configure_rows();
    if (!e) e = configure_small();
    return e;
}

}  // namespace precgpu
