// prec_gpu_batch.cu -- the batch form: many products of uneven sizes.
//
// The reference multiplies one pair per call (precn_t operator*,
// src/mul_basic.cpp:278-284); its only producer of many independent products
// is binary splitting (pi/pi_chudnovsky.cpp:141-144), one tree level at a
// time.  Here a batch of device-resident products is planned once:
//   * every product gets its transform length 2^k (the same plan as a single
//     product), and products of one length form a length class;
//   * classes up to 2^12 points run one single-CTA product per CTA in one
//     launch; larger classes run the four-step kernels once per pass over
//     all their products (grid.z = product, per-product pointers in a
//     device descriptor array), in chunks bounded by a workspace budget;
//   * each class gets its own stream branch, so classes overlap on the GPU;
//   * the first prec_gpu_batch_run records all of it into one CUDA graph
//     (descriptors and workspaces have fixed addresses), later runs replay
//     the graph with a single launch;
//   * with PREC_GPU_BATCH_PERSISTENT=1, set 0's 2^13 .. 2^16-point classes
//     run as one persistent kernel per class (ntt_class.cu) instead of four
//     phase kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/prec_gpu.h"
#include "prec_gpu_internal.h"

using namespace precgpu;

namespace {

struct Chunk {
    int first = 0, count = 0;  // entries of the class's descriptor array
    int max_nblk = 0;
};

struct Cls {
    int k = 0;
    int square = 0;               // every product of the class is a square
    Plan pl;                      // class-wide plan (k, set, k1, k2, rows, crt)
    std::vector<int> items;       // indices into the batch's products
    size_t ws_per = 0;            // workspace bytes per product (four-step)
    int per_chunk = 0;            // products per chunk
    std::vector<Chunk> chunks;
    SmallDesc* d_small = nullptr; // device descriptors (single-CTA classes)
    ProdPtrs* d_ptrs = nullptr;   // device descriptors (four-step classes)
    uint8_t* ws = nullptr;        // workspace of one chunk
    bool persistent = false;      // one persistent kernel per chunk (ntt_class.cu)
    uint32_t* sched = nullptr;    // its scheduling words (kClassHdrWords + kClassProdWords per product)
    cudaStream_t stream = nullptr;
    cudaEvent_t join = nullptr;
};

size_t env_bytes(const char* name, size_t dflt) {
    const char* s = std::getenv(name);
    if (!s) return dflt;
    const double v = std::atof(s);
    return v > 0 ? (size_t)v : dflt;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

struct prec_gpu_batch {
    std::vector<prec_gpu_product_t> items;
    std::vector<Cls> classes;
    std::vector<int> zero_items;  // products with a zero-length operand
    void* d_mem = nullptr;
    size_t d_bytes = 0;
    cudaStream_t oneshot = nullptr;  // one-shot form: d_mem from the library pool on this stream
    bool pooled = false;
    cudaStream_t cap = nullptr;
    cudaEvent_t fork = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t graph_launches = 0;  // kernels in the recorded graph
    int* err = nullptr;
    uint32_t spin_limit = 0;      // persistent class kernels: polls per dependency wait
    int never_signal = 0;         // tests: their forward tiles never complete a counter
};

static void batch_free(prec_gpu_batch* b) {
    if (!b) return;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (Cls& c : b->classes) {
        if (c.stream) cudaStreamDestroy(c.stream);
        if (c.join) cudaEventDestroy(c.join);
    }
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->cap) cudaStreamDestroy(b->cap);
    if (b->d_mem) {
        if (b->pooled) cudaFreeAsync(b->d_mem, b->oneshot);
        else cudaFree(b->d_mem);
    }
    delete b;
}

#define BCK(x)                                  \
    do {                                        \
        cudaError_t _e = (x);                   \
        if (_e != cudaSuccess) {                \
            batch_free(b);                      \
            return cuda_code(_e);               \
        }                                       \
    } while (0)

// all of the batch's device work, enqueued on the class streams (forked
// from and joined to `origin`), or on `origin` alone when `branch` is false.
// With a graph recorder installed on the thread, the same work becomes
// nodes: one independent chain per class stream, the zero fills on `origin`.
static void batch_enqueue(prec_gpu_batch* b, cudaStream_t origin, bool branch) {
    GraphRecorder* rec = thread_recorder();
    if (branch && !rec) cudaEventRecord(b->fork, origin);
    for (int i : b->zero_items) {
        const prec_gpu_product_t& p = b->items[i];
        if (!(p.an + p.bn)) continue;
        if (rec) rec->add_memset(p.out, (p.an + p.bn) * sizeof(uint64_t), origin);
        else cudaMemsetAsync(p.out, 0, (p.an + p.bn) * sizeof(uint64_t), origin);
    }
    for (Cls& c : b->classes) {
        cudaStream_t st = branch ? c.stream : origin;
        if (branch && !rec) cudaStreamWaitEvent(st, b->fork, 0);
        if (c.pl.path == 0) {
            ntt_launch_small(c.d_small, nullptr, (int)c.items.size(), c.k, ctx_field(0), c.pl.crt, st);
        } else {
            ProdArgs args{};
            args.err = b->err;
            args.k = c.pl.k;
            args.k1 = c.pl.k1;
            args.k2 = c.pl.k2;
            args.rows = c.pl.rows;
            args.cg = c.pl.cg;
            args.cmr = c.pl.cmr;
            args.rmr = c.pl.rmr;
            args.square = c.square;
            args.crt = c.pl.crt;
            args.crt5 = c.pl.crt5;
            args.f = ctx_field(c.pl.set);
            for (const Chunk& ch : c.chunks) {
                if (c.persistent) {
                    const size_t bytes = (kClassHdrWords + (size_t)kClassProdWords * ch.count) * sizeof(uint32_t);
                    if (rec) rec->add_memset(c.sched, bytes, st);
                    else cudaMemsetAsync(c.sched, 0, bytes, st);
                    const ClassRun run{c.sched, ch.count, ch.max_nblk, class_rows(c.pl.k1, c.pl.k2), b->spin_limit,
                                       b->never_signal};
                    if (launch_class_persistent(args, c.d_ptrs + ch.first, run, st) == 0) continue;
                }
                ntt_launch_4step_batch(c.pl.set, args, c.d_ptrs + ch.first, ch.count, ch.max_nblk, st);
            }
        }
        if (branch && !rec) {
            cudaEventRecord(c.join, st);
            cudaStreamWaitEvent(origin, c.join, 0);
        }
    }
}

// Plans a batch and uploads its descriptors.  `oneshot` (prec_gpu_mul_batch):
// the device memory comes stream-ordered from the library pool on that
// stream (no device-wide allocation or free per call), and no stream
// branches or capture stream are made.
static int batch_build(const prec_gpu_product_t* items, size_t count, bool oneshot, cudaStream_t ost,
                       prec_gpu_batch** out) {
    if (!out || (!items && count)) return PREC_GPU_E_ARG;
    *out = nullptr;
    std::lock_guard<std::mutex> lk(ctx_mutex());
    int r = ctx_init_locked(-1);
    if (r) return r;
    prec_gpu_batch* b = new prec_gpu_batch();
    b->oneshot = ost;
    b->items.assign(items, items + count);
    b->err = ctx_device_err();
    // classes by key (64-bit digits << 8 | k << 1 | square): a dense table,
    // not a map lookup per product (a binary-splitting level has ~10^6 of them)
    std::vector<int> cls_of(1 << 9, -1);
    std::vector<Cls> found;
    const bool wide = wide_digits();
    for (size_t i = 0; i < count; ++i) {
        const prec_gpu_product_t& p = items[i];
        if ((p.an && !p.a) || (p.bn && !p.b) || (p.an + p.bn && !p.out)) {
            batch_free(b);
            return PREC_GPU_E_ARG;
        }
        if (p.an == 0 || p.bn == 0) {
            b->zero_items.push_back((int)i);
            continue;
        }
        // the transform length and digit width pick the class; the class
        // plan (CRT constants, kernel configuration) is made once, for its
        // first product
        const uint64_t need = 2 * (uint64_t)p.an + 2 * (uint64_t)p.bn - 1;
        int k = kSmallMinLog2;
        while ((1ull << k) < need) ++k;
        if (k > kMaxLog2) {
            batch_free(b);
            return PREC_GPU_E_TOO_LARGE;
        }
        const int kw = wide ? wide_log2(p.an, p.bn, k) : 0;
        if (kw) k = kw;
        const int sq = (p.a == p.b && p.an == p.bn && k > kSmallMaxLog2) ? 1 : 0;
        int& ci = cls_of[(kw ? 1 << 8 : 0) | k << 1 | sq];
        if (ci < 0) {
            ci = (int)found.size();
            found.emplace_back();
        }
        Cls& c = found[ci];
        if (c.items.empty()) {
            if ((r = plan_for(2 * (uint64_t)p.an, 2 * (uint64_t)p.bn, p.an + p.bn, c.pl, wide))) {
                batch_free(b);
                return r;
            }
            if (c.pl.k != k || set_wide(c.pl.set) != (kw != 0)) {  // the key and the plan agree
                batch_free(b);
                return PREC_GPU_E_INTERNAL;
            }
            c.k = c.pl.k;
            c.square = sq;
        }
        c.items.push_back((int)i);
    }
    // device layout: descriptors, then one workspace per four-step class
    // (and, for a persistent class, its scheduling words)
    const size_t budget = env_bytes("PREC_GPU_BATCH_CLASS_BYTES", (size_t)1 << 30);
    const char* pe = std::getenv("PREC_GPU_BATCH_PERSISTENT");
    const bool persistent = pe && pe[0] == '1';
    // a dependency wait gives up after about a second (PREC_GPU_BATCH_SPIN_LIMIT polls
    // of ~0.25 us; tests shorten it); PREC_GPU_BATCH_NEVER_SIGNAL=1 (tests)
    // makes every such wait run out
    b->spin_limit = (uint32_t)env_bytes("PREC_GPU_BATCH_SPIN_LIMIT", (size_t)1 << 22);
    const char* ns = std::getenv("PREC_GPU_BATCH_NEVER_SIGNAL");
    b->never_signal = ns && ns[0] == '1' ? 1 : 0;
    std::vector<size_t> sched_off;
    size_t bytes = 0;
    std::vector<size_t> desc_off, ws_off;
    for (int ci : cls_of) {
        if (ci < 0) continue;  // key order, as before
        Cls& c = found[ci];
        const size_t n = c.items.size();
        desc_off.push_back(bytes);
        bytes += align256(n * (c.pl.path == 0 ? sizeof(SmallDesc) : sizeof(ProdPtrs)));
        if (c.pl.path == 1) {
            // a product of 2^k points has at most 2^(k-1) + 1 limbs on 32-bit
            // digits, 2^k + 1 on 64-bit digits
            const uint64_t lout_max = set_wide(c.pl.set) ? (1ull << c.k) + 1 : (1ull << c.k) / 2 + 1;
            const size_t carry_words = (size_t)(lout_max / crt_block_limbs(c.pl.set)) + 2;
            c.ws_per = align256(((size_t)2 * c.pl.nprimes << c.k) * sizeof(uint32_t) + carry_words * sizeof(uint32_t));
            c.per_chunk = (int)std::min<size_t>({n, std::max<size_t>(1, budget / c.ws_per), 65535});
            ws_off.push_back(bytes);
            bytes += c.ws_per * c.per_chunk;
            c.persistent = persistent && class_persistent_supported(c.pl);
            sched_off.push_back(bytes);
            if (c.persistent) bytes += align256((kClassHdrWords + (size_t)kClassProdWords * c.per_chunk) * sizeof(uint32_t));
        } else {
            ws_off.push_back(0);
            sched_off.push_back(0);
        }
        b->classes.push_back(std::move(c));
    }
    b->d_bytes = bytes;
    if (bytes && oneshot) {
        BCK(cudaMallocFromPoolAsync(&b->d_mem, bytes, ctx_pool(), ost));
        b->pooled = true;
    } else if (bytes) {
        BCK(cudaMalloc(&b->d_mem, bytes));
    }
    auto upload = [&](void* dst, const void* src, size_t n) {
        return oneshot ? cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, ost)
                       : cudaMemcpy(dst, src, n, cudaMemcpyHostToDevice);
    };
    uint8_t* base = static_cast<uint8_t*>(b->d_mem);
    for (size_t ci = 0; ci < b->classes.size(); ++ci) {
        Cls& c = b->classes[ci];
        const size_t n = c.items.size();
        if (c.pl.path == 0) {
            std::vector<SmallDesc> h(n);
            for (size_t j = 0; j < n; ++j) {
                const prec_gpu_product_t& p = items[c.items[j]];
                SmallDesc& d = h[j];
                d.a = p.a;
                d.b = p.b;
                d.out = p.out;
                d.la = p.an;
                d.lb = p.bn;
                d.lout = p.an + p.bn;
                d.k = c.k;
                d.square = p.a == p.b && p.an == p.bn;
            }
            c.d_small = reinterpret_cast<SmallDesc*>(base + desc_off[ci]);
            BCK(upload(c.d_small, h.data(), n * sizeof(SmallDesc)));
        } else {
            c.ws = base + ws_off[ci];
            if (c.persistent) c.sched = reinterpret_cast<uint32_t*>(base + sched_off[ci]);
            std::vector<ProdPtrs> h(n);
            const uint64_t bl = (uint64_t)crt_block_limbs(c.pl.set);
            for (size_t j = 0; j < n; ++j) {
                const prec_gpu_product_t& p = items[c.items[j]];
                ProdPtrs& d = h[j];
                uint8_t* w = c.ws + c.ws_per * (j % c.per_chunk);  // chunks reuse the workspace
                d.a = p.a;
                d.b = p.b;
                d.out = p.out;
                d.work = reinterpret_cast<uint32_t*>(w);
                d.scratch = d.work + ((size_t)2 * c.pl.nprimes << c.k);
                d.la = p.an;
                d.lb = p.bn;
                d.lout = p.an + p.bn;
                d.nblk = (int)((d.lout + bl - 1) / bl);
                d.pad = 0;
            }
            for (size_t f = 0; f < n; f += c.per_chunk) {
                Chunk ch;
                ch.first = (int)f;
                ch.count = (int)std::min<size_t>(c.per_chunk, n - f);
                for (int j = 0; j < ch.count; ++j) ch.max_nblk = std::max(ch.max_nblk, h[f + j].nblk);
                c.chunks.push_back(ch);
            }
            c.d_ptrs = reinterpret_cast<ProdPtrs*>(base + desc_off[ci]);
            BCK(upload(c.d_ptrs, h.data(), n * sizeof(ProdPtrs)));
        }
        if (oneshot) continue;
        BCK(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
        BCK(cudaEventCreateWithFlags(&c.join, cudaEventDisableTiming));
    }
    if (!oneshot) {
        BCK(cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking));
        BCK(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    }
    *out = b;
    return PREC_GPU_OK;
}

extern "C" {

int prec_gpu_batch_create(const prec_gpu_product_t* items, size_t count, prec_gpu_batch_t** out) {
    return batch_build(items, count, false, nullptr, out);
}

int prec_gpu_batch_run(prec_gpu_batch_t* b, void* stream) {
    if (!b) return PREC_GPU_E_ARG;
    NvtxRange range("prec_gpu_batch_run %zu products, %zu classes", b->items.size(), b->classes.size());
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (!b->exec) {
        // the graph built node by node (no stream capture: another thread's
        // device-wide synchronising call cannot break it)
        GraphRecorder rec;
        cudaError_t e = cudaGraphCreate(&rec.graph, 0);
        if (e != cudaSuccess) return cuda_code(e);
        const uint64_t before = launches_this_thread();
        thread_recorder() = &rec;
        batch_enqueue(b, b->cap, true);
        thread_recorder() = nullptr;
        // recorded, not launched: counted at every replay instead
        b->graph_launches = launches_this_thread() - before;
        uncount_launches(b->graph_launches);
        b->graph = rec.graph;
        if (rec.err != cudaSuccess) return cuda_code(rec.err);
        e = cudaGraphInstantiate(&b->exec, b->graph, 0);
        if (e != cudaSuccess) return cuda_code(e);
    }
    const cudaError_t e = cudaGraphLaunch(b->exec, st);
    if (e == cudaSuccess) count_launches(b->graph_launches);
    return cuda_code(e);
}

int prec_gpu_batch_info(const prec_gpu_batch_t* b, size_t* classes, size_t* device_bytes) {
    if (!b) return PREC_GPU_E_ARG;
    if (classes) *classes = b->classes.size();
    if (device_bytes) *device_bytes = b->d_bytes;
    return PREC_GPU_OK;
}

void prec_gpu_batch_destroy(prec_gpu_batch_t* b) {
    if (b) cudaDeviceSynchronize();
    batch_free(b);
}

int prec_gpu_mul_batch(const prec_gpu_product_t* items, size_t count, void* stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    prec_gpu_batch_t* b = nullptr;
    int r = batch_build(items, count, true, st, &b);
    if (r) return r;
    batch_enqueue(b, st, false);
    cudaError_t e = cudaGetLastError();
    batch_free(b);  // the workspace returns to the pool after the batch's work on `st`
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_code(e);
    return ctx_take_device_err();  // what the batch's kernels reported
}

}  // extern "C"
