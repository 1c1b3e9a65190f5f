// prec_gpu_serve.cu -- serving loop: continuous admission of multiply
// requests with device-resident operands.
//
// The reference has no server; its callers issue products one at a time.
// Here a worker thread owns `slots` CUDA streams and a private memory pool:
//   * submit() appends a request (device operands, output) and returns a
//     ticket at once;
//   * the worker admits pending requests whenever a stream slot is free and
//     the plan's HBM footprint (the four-step work buffer and carry words)
//     fits the byte budget -- first come first served, with a bounded
//     bypass so small requests do not wait behind one that cannot fit yet;
//   * each admitted request runs on its own stream, so requests that arrive
//     while others are on the GPU overlap with them; its workspace is
//     allocated and freed stream-ordered from the pool;
//   * completion is seen through an event per slot; the latency of a
//     request is host time from submit() to the observed completion;
//   * each slot has its own device error word, copied to pinned host memory
//     on the slot's stream before the completion event, so a finished
//     request reports what its kernels flagged.
// Results do not depend on what else runs: each request has its own
// workspace, and the kernels are deterministic.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/prec_gpu.h"
#include "prec_gpu_internal.h"

using namespace precgpu;

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    uint64_t ticket = 0;
    prec_gpu_product_t p{};
    Plan pl;
    size_t bytes = 0;  // HBM footprint of the plan
    Clock::time_point t_submit;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    bool busy = false;
    Request req;
};

struct TicketState {
    int status = -1;  // -1 pending, else PREC_GPU_* code
    double latency_ms = 0.0;
};

constexpr int kMaxBypass = 8;  // requests admitted past a head that does not fit

}  // namespace

struct prec_gpu_server {
    size_t budget = 0;
    std::vector<Slot> slots;
    cudaMemPool_t pool = nullptr;
    int* err = nullptr;    // device error word per slot
    int* h_err = nullptr;  // its pinned host copy, written before the slot's completion event
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request> pending;
    std::vector<TicketState> tickets;
    std::vector<double> latencies;  // of completed requests
    size_t in_flight_bytes = 0, peak_bytes = 0;
    int in_flight = 0, peak_in_flight = 0;
    uint64_t submitted = 0, completed = 0, failed = 0;
    Clock::time_point t_first, t_last;
    bool stop = false;
    std::thread worker;
    int device = 0;
};

static size_t footprint(const Plan& pl) { return pl.path == 1 ? pl.work_bytes : 0; }

// launches one admitted request on its slot (worker thread, lock not held)
static int launch_request(prec_gpu_server* s, Slot& sl) {
    const Request& r = sl.req;
    NvtxRange range("serve request %llu: %zux%zu", (unsigned long long)r.ticket, r.p.an, r.p.bn);
    cudaStream_t st = sl.stream;
    const prec_gpu_product_t& p = r.p;
    const size_t si = (size_t)(&sl - s->slots.data());
    s->h_err[si] = 0;  // the slot is idle: no copy into it is in flight
    if (p.an == 0 || p.bn == 0) {
        if (p.an + p.bn) cudaMemsetAsync(p.out, 0, (p.an + p.bn) * sizeof(uint64_t), st);
    } else if (r.pl.path == 0) {
        SmallDesc d{};
        d.a = p.a;
        d.b = p.b;
        d.out = p.out;
        d.la = p.an;
        d.lb = p.bn;
        d.lout = p.an + p.bn;
        d.k = r.pl.k;
        ntt_launch_small(nullptr, &d, 1, r.pl.k, ctx_field(0), r.pl.crt, st);
    } else {
        void* ws = nullptr;
        cudaError_t e = cudaMallocFromPoolAsync(&ws, r.bytes, s->pool, st);
        if (e != cudaSuccess) return cuda_code(e);
        ProdArgs args{};
        args.a = p.a;
        args.b = p.b;
        args.out = p.out;
        args.work = static_cast<uint32_t*>(ws);
        args.scratch = args.work + ((size_t)2 * r.pl.nprimes << r.pl.k);
        args.err = s->err + si;
        args.la = p.an;
        args.lb = p.bn;
        args.lout = p.an + p.bn;
        args.k = r.pl.k;
        args.k1 = r.pl.k1;
        args.k2 = r.pl.k2;
        args.nblk = r.pl.nblk;
        args.rows = r.pl.rows;
        args.cg = r.pl.cg;
        args.cmr = r.pl.cmr;
        args.rmr = r.pl.rmr;
        args.crt = r.pl.crt;
        args.crt5 = r.pl.crt5;
        args.f = ctx_field(r.pl.set);
        ntt_launch_4step(r.pl.set, args, st);
        cudaFreeAsync(ws, st);
        cudaMemcpyAsync(s->h_err + si, s->err + si, sizeof(int), cudaMemcpyDeviceToHost, st);
        cudaMemsetAsync(s->err + si, 0, sizeof(int), st);
    }
    cudaEventRecord(sl.done, st);
    return cuda_code(cudaGetLastError());
}

static void finish(prec_gpu_server* s, Slot& sl, int status) {
    const auto now = Clock::now();
    TicketState& t = s->tickets[sl.req.ticket];
    t.status = status;
    t.latency_ms = std::chrono::duration<double, std::milli>(now - sl.req.t_submit).count();
    s->latencies.push_back(t.latency_ms);
    s->t_last = now;
    ++s->completed;
    if (status) ++s->failed;
    s->in_flight_bytes -= sl.req.bytes;
    --s->in_flight;
    sl.busy = false;
}

static void worker_loop(prec_gpu_server* s) {
    cudaSetDevice(s->device);
    std::vector<int> to_launch;
    for (;;) {
        to_launch.clear();
        {
            std::unique_lock<std::mutex> lk(s->mu);
            // completions
            for (Slot& sl : s->slots) {
                if (!sl.busy) continue;
                const cudaError_t q = cudaEventQuery(sl.done);
                if (q == cudaErrorNotReady) continue;
                const int e = s->h_err[&sl - s->slots.data()];
                const int ok = e == 0 ? PREC_GPU_OK : (e & kDevErrTimeout) ? PREC_GPU_E_TIMEOUT : PREC_GPU_E_INTERNAL;
                finish(s, sl, q == cudaSuccess ? ok : cuda_code(q));
                s->cv_done.notify_all();
            }
            // admission: FIFO, bounded bypass of a head that does not fit
            int bypassed = 0;
            for (auto it = s->pending.begin(); it != s->pending.end();) {
                Slot* free_slot = nullptr;
                for (Slot& sl : s->slots)
                    if (!sl.busy) {
                        free_slot = &sl;
                        break;
                    }
                if (!free_slot) break;
                if (s->in_flight_bytes + it->bytes > s->budget) {
                    if (++bypassed > kMaxBypass) break;
                    ++it;
                    continue;
                }
                free_slot->busy = true;
                free_slot->req = *it;
                s->in_flight_bytes += it->bytes;
                s->peak_bytes = std::max(s->peak_bytes, s->in_flight_bytes);
                ++s->in_flight;
                s->peak_in_flight = std::max(s->peak_in_flight, s->in_flight);
                to_launch.push_back((int)(free_slot - s->slots.data()));
                it = s->pending.erase(it);
            }
            if (to_launch.empty()) {
                if (s->stop && s->in_flight == 0 && s->pending.empty()) return;
                if (s->in_flight == 0) {
                    s->cv_work.wait(lk, [&] { return s->stop || !s->pending.empty(); });
                    continue;
                }
            }
        }
        for (int i : to_launch) {
            const int rc = launch_request(s, s->slots[i]);
            if (rc) {
                std::lock_guard<std::mutex> lk(s->mu);
                cudaStreamSynchronize(s->slots[i].stream);
                finish(s, s->slots[i], rc);
                s->cv_done.notify_all();
            }
        }
        if (to_launch.empty()) std::this_thread::sleep_for(std::chrono::microseconds(5));
    }
}

extern "C" {

int prec_gpu_serve_create(size_t hbm_budget_bytes, int slots, prec_gpu_server_t** out) {
    if (!out || slots < 1 || slots > 256) return PREC_GPU_E_ARG;
    *out = nullptr;
    {
        std::lock_guard<std::mutex> lk(ctx_mutex());
        int r = ctx_init_locked(-1);
        if (r) return r;
    }
    prec_gpu_server* s = new prec_gpu_server();
    cudaGetDevice(&s->device);
    s->budget = hbm_budget_bytes;
    s->slots.resize(slots);
    cudaError_t e = cudaSuccess;
    for (Slot& sl : s->slots) {
        if (!e) e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
        if (!e) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
    }
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = s->device;
    if (!e) e = cudaMemPoolCreate(&s->pool, &props);
    if (!e) {
        uint64_t keep = ~0ull;  // keep freed workspace in the pool, resident
        e = cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (!e) e = cudaMalloc(&s->err, slots * sizeof(int));
    if (!e) e = cudaMemset(s->err, 0, slots * sizeof(int));
    if (!e) e = cudaMallocHost(&s->h_err, slots * sizeof(int));
    if (!e) std::fill(s->h_err, s->h_err + slots, 0);
    if (e) {
        prec_gpu_serve_destroy(s);
        return cuda_code(e);
    }
    s->worker = std::thread(worker_loop, s);
    *out = s;
    return PREC_GPU_OK;
}

int prec_gpu_serve_submit(prec_gpu_server_t* s, const uint64_t* d_a, size_t an, const uint64_t* d_b, size_t bn,
                          uint64_t* d_out, uint64_t* ticket) {
    if (!s || !ticket || (an && !d_a) || (bn && !d_b) || (an + bn && !d_out)) return PREC_GPU_E_ARG;
    Request r;
    r.p = prec_gpu_product_t{d_a, an, d_b, bn, d_out};
    if (an && bn) {
        const int rc = plan_for(2 * (uint64_t)an, 2 * (uint64_t)bn, an + bn, r.pl, wide_digits());
        if (rc) return rc;
        r.bytes = footprint(r.pl);
        if (r.bytes > s->budget) return PREC_GPU_E_NOMEM;  // could never be admitted
    }
    r.t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        r.ticket = s->tickets.size();
        s->tickets.push_back(TicketState());
        if (s->submitted == 0) s->t_first = r.t_submit;
        ++s->submitted;
        s->pending.push_back(r);
    }
    s->cv_work.notify_one();
    *ticket = r.ticket;
    return PREC_GPU_OK;
}

int prec_gpu_serve_wait(prec_gpu_server_t* s, uint64_t ticket, double timeout_s, double* latency_ms) {
    if (!s) return PREC_GPU_E_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    if (ticket >= s->tickets.size()) return PREC_GPU_E_ARG;
    const bool ok = s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                        [&] { return s->tickets[ticket].status >= 0; });
    if (!ok) return PREC_GPU_E_TIMEOUT;
    if (latency_ms) *latency_ms = s->tickets[ticket].latency_ms;
    return s->tickets[ticket].status;
}

int prec_gpu_serve_drain(prec_gpu_server_t* s, double timeout_s) {
    if (!s) return PREC_GPU_E_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    const bool ok = s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                        [&] { return s->completed == s->submitted; });
    return ok ? PREC_GPU_OK : PREC_GPU_E_TIMEOUT;
}

int prec_gpu_serve_stats(prec_gpu_server_t* s, prec_gpu_serve_stats_t* st) {
    if (!s || !st) return PREC_GPU_E_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    std::vector<double> l = s->latencies;
    std::sort(l.begin(), l.end());
    auto pct = [&](double q) { return l.empty() ? 0.0 : l[std::min(l.size() - 1, (size_t)(q * (l.size() - 1) + 0.5))]; };
    st->submitted = s->submitted;
    st->completed = s->completed;
    st->failed = s->failed;
    st->p50_ms = pct(0.50);
    st->p99_ms = pct(0.99);
    st->max_ms = l.empty() ? 0.0 : l.back();
    double sum = 0;
    for (double x : l) sum += x;
    st->mean_ms = l.empty() ? 0.0 : sum / l.size();
    const double span = std::chrono::duration<double>(s->t_last - s->t_first).count();
    st->products_per_s = span > 0 ? s->completed / span : 0.0;
    st->peak_bytes = s->peak_bytes;
    st->peak_in_flight = s->peak_in_flight;
    return PREC_GPU_OK;
}

void prec_gpu_serve_destroy(prec_gpu_server_t* s) {
    if (!s) return;
    if (s->worker.joinable()) {
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stop = true;
        }
        s->cv_work.notify_all();
        s->worker.join();
    }
    for (Slot& sl : s->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream), cudaStreamDestroy(sl.stream);
        if (sl.done) cudaEventDestroy(sl.done);
    }
    if (s->pool) cudaMemPoolDestroy(s->pool);
    if (s->err) cudaFree(s->err);
    if (s->h_err) cudaFreeHost(s->h_err);
    delete s;
}

}  // extern "C"
