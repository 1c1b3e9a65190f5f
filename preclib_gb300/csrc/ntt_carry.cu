// ntt_carry.cu -- the CRT/carry kernel of the four-step path (one block of
// crt_carry_tile, ntt_carry.cuh, per CTA), its launchers, and the four-step
// product's launch sequence.
#include "ntt_carry.cuh"

namespace precgpu {

template <int SET>
__global__ void __launch_bounds__(kCarryThreads) k_crt_carry(ProdArgs args, const ProdPtrs* __restrict__ batch) {
    crt_carry_tile<SET>(args, batch, GridIdx{});
}

void launch_crt_carry(int set, const ProdArgs& a, cudaStream_t st, const ProdPtrs* batch, int count, int max_nblk,
                      int nblk_launch) {
    const dim3 grid(batch ? max_nblk : (nblk_launch > 0 ? nblk_launch : a.nblk), 1, count);
    if (set == 0) launch_kernel(k_crt_carry<0>, grid, kCarryThreads, 0, st, a, batch);
    else if (set == 1) launch_kernel(k_crt_carry<1>, grid, kCarryThreads, 0, st, a, batch);
    else if (set == kWideSet) launch_kernel(k_crt_carry<kWideSet>, grid, kCarryThreads, 0, st, a, batch);
    else launch_kernel(k_crt_carry<kWideSetL>, grid, kCarryThreads, 0, st, a, batch);
    count_launches(1);
}

void ntt_launch_4step_batch(int set, const ProdArgs& args, const ProdPtrs* batch, int count, int max_nblk,
                            cudaStream_t st) {
    launch_fwd_cols(set, args, st, batch, count);
    launch_rows(set, args, st, batch, count);
    launch_inv_cols(set, args, st, batch, count);
    launch_crt_carry(set, args, st, batch, count, max_nblk);
}

static void launch_crt_chunks(int set, const ProdArgs& args, cudaStream_t st, const CrtChunks& ch) {
    for (int c = 0; c < ch.count; ++c) {
        ProdArgs a = args;
        a.chunk_words = ch.words;
        a.crt_chunk = c;
        a.crt_blk0 = ch.blk0[c];
        a.crt_last = c == ch.count - 1;
        launch_crt_carry(set, a, st, nullptr, 1, 0, ch.blk0[c + 1] - ch.blk0[c]);
        cudaEventRecord(ch.done[c], st);
    }
}

void ntt_launch_4step(int set, const ProdArgs& args, cudaStream_t st, cudaEvent_t* ev, const PrimeStreams* ps,
                      cudaEvent_t a_ready, cudaEvent_t b_ready, const CrtChunks* chunks) {
    if (ps && !ev) {
        // one chain per prime; the CRT kernel joins them
        const bool staged = a_ready && b_ready && !args.square;
        if (!staged) cudaEventRecord(ps->fork, st);
        for (int p = 0; p < kSetPrimes[set]; ++p) {
            cudaStream_t s = ps->s[p];
            ProdArgs a = args;
            a.prime0 = p;
            if (staged) {
                cudaStreamWaitEvent(s, a_ready, 0);
                a.operand_only = 1;
                launch_fwd_cols(set, a, s, nullptr, 1, 1);
                cudaStreamWaitEvent(s, b_ready, 0);
                a.operand_only = 2;
                launch_fwd_cols(set, a, s, nullptr, 1, 1);
                a.operand_only = 0;
            } else {
                cudaStreamWaitEvent(s, ps->fork, 0);
                launch_fwd_cols(set, a, s, nullptr, 1, 1);
            }
            launch_rows(set, a, s, nullptr, 1, 1);
            launch_inv_cols(set, a, s, nullptr, 1, 1);
            cudaEventRecord(ps->join[p], s);
            cudaStreamWaitEvent(st, ps->join[p], 0);
        }
        if (chunks) launch_crt_chunks(set, args, st, *chunks);
        else launch_crt_carry(set, args, st);
        return;
    }
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
    int e = configure_fwd_cols();
    if (!e) e = configure_inv_cols();
    if (!e) e = configure_rows();
    if (!e) e = configure_small();
    if (!e) e = configure_class();
    return e;
}

}  // namespace precgpu
