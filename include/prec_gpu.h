/*
 * prec_gpu.h -- C ABI of the GB300 large-operand multiply.
 *
 * Drop-in boundary for the two size bands of preclib's multiply dispatcher
 * that this library replaces:
 *   precn_t mul_ntt(const precn_t&, const precn_t&)   prec.hpp:102,
 *       src/mul_ntt.cpp:494 (called from src/mul_basic.cpp:264 for >6144 limbs)
 *   precn_t mul_fft(const precn_t&, const precn_t&)   prec.hpp:94,
 *       src/mul_fft.cpp:386 (called from src/mul_basic.cpp:203, 268 for 193-6144 limbs)
 * Those C++ entry points take and return precn_t {asiz, rsiz, a} with
 * little-endian uint64 limbs (prec.hpp:49-52).  This header flattens them to
 * plain pointers and sizes; prec_gpu_precn.cpp rebuilds the C++ symbols on
 * top of it for a build that links the reference's other sources.
 *
 * Limbs: value = a[0] + a[1]*2^64 + ...  The product of an and bn limbs is
 * written as exactly an+bn limbs (high limbs zero-padded); the caller trims.
 * Every entry point returns 0 on success or one of the PREC_GPU_E_* codes.
 * Nothing here falls back to a CPU multiply: without a usable CUDA device
 * every call fails with PREC_GPU_E_NODEV.
 */
#ifndef PREC_GPU_H
#define PREC_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    PREC_GPU_OK = 0,
    PREC_GPU_E_ARG = 1,          /* null pointer, zero or inconsistent size */
    PREC_GPU_E_TOO_LARGE = 2,    /* product beyond the 2^26-point transform (batch and serving forms) */
    PREC_GPU_E_NOMEM = 3,        /* device allocation failed */
    PREC_GPU_E_CUDA = 4,         /* other CUDA runtime error */
    PREC_GPU_E_TIMEOUT = 5,      /* a bounded device-side wait ran out */
    PREC_GPU_E_FFT_ROUNDING = 6, /* FP64 band: distance to integer > 0.25 */
    PREC_GPU_E_NODEV = 7,        /* no CUDA device / library not initialised */
    PREC_GPU_E_INTERNAL = 8      /* internal consistency check failed */
};

/* Per-product report of the most recent call on the calling thread. */
typedef struct prec_gpu_stats {
    int path;                 /* 0 single-CTA NTT, 1 four-step NTT, 2 FP64 FFT, 3 blocked NTT */
    int log2_n;               /* transform length */
    int primes;               /* NTT primes (3, or 5 for 64-bit digits); 0 for the FFT */
    int digit_bits;           /* bits per transform digit (NTT 32 or 64; FFT 8 .. 16) */
    size_t limbs_a, limbs_b;  /* operand sizes used */
    double fft_max_distance;  /* FP64 band: max |x - round(x)|; 0 for NTT */
    double device_ms;         /* device time of the product (events) */
} prec_gpu_stats_t;

/* Selects and initialises the device (idempotent; device -1 = current).
 * Replaces: nothing (the reference keeps thread_local NTT plans,
 * src/mul_ntt.cpp:182-191, and a static FFT plan cache, src/mul_fft.cpp:78-100). */
int prec_gpu_init(int device);

/* Releases every device resource of the library.  Call it only when no
 * other thread is inside the library. */
void prec_gpu_shutdown(void);

/* Full product of two host limb vectors, out[0 .. an+bn) written.
 * Band routing inside: max(an,bn) <= 6144 limbs -> FP64 FFT band
 * (replaces mul_fft, src/mul_fft.cpp:386-394), larger -> NTT band
 * (replaces mul_ntt, src/mul_ntt.cpp:494-518).  Squares above 6144 limbs
 * and products of any size below 193 limbs also run on the GPU.
 * Thread-safe: each calling thread has its own stream, workspace and
 * staging buffers (up to 16 threads; more share them round-robin), so
 * products called from different threads run concurrently on the device,
 * as the reference's per-thread NTT plans let its threads multiply in
 * parallel (src/mul_ntt.cpp:182-191). */
int prec_gpu_mul(const uint64_t *a, size_t an, const uint64_t *b, size_t bn, uint64_t *out);

/* NTT band forced, host pointers (replaces mul_ntt, src/mul_ntt.cpp:494). */
int prec_gpu_mul_ntt(const uint64_t *a, size_t an, const uint64_t *b, size_t bn, uint64_t *out);

/* FP64 FFT band forced, host pointers (replaces mul_fft, src/mul_fft.cpp:386).
 * Products with max(an,bn) <= 6144 limbs run the FP64 FFT: balanced digits
 * of the widest width (16 .. 8 bits) whose worst-case rounding bound stays
 * below 1/4; the product's max distance to the nearest integer is reported
 * in prec_gpu_stats_t.fft_max_distance, and a distance above 0.25 returns
 * PREC_GPU_E_FFT_ROUNDING with `out` untouched.  Larger products (squares
 * that precn_sqr sends to mul_fft, src/mul_basic.cpp:203) run the NTT band. */
int prec_gpu_mul_fft(const uint64_t *a, size_t an, const uint64_t *b, size_t bn, uint64_t *out);

/* Square of a host limb vector, out[0 .. 2an) written (replaces precn_sqr,
 * src/mul_basic.cpp:193-204, above its schoolbook base case).  The operand
 * is copied to the device once and, on the NTT band's four-step path,
 * transformed once per prime (a product transforms both operands).
 * prec_gpu_mul, prec_gpu_mul_ntt and
 * prec_gpu_mul_device take the same route when a == b and an == bn. */
int prec_gpu_sqr(const uint64_t *a, size_t an, uint64_t *out);

/* ---- Autotuner ------------------------------------------------------------
 * Kernel configuration of one four-step NTT length 2^log2_n (13 .. 26):
 * the column/row split, columns per column-pass CTA, the column and row
 * pass radix caps, rows per row-pass CTA, and whether a single product
 * runs each prime's kernels on its own stream.  Every product (single, batch,
 * serving loop) uses the configuration of its length.  Defaults apply until
 * a length is tuned, set or loaded; PREC_GPU_TUNE_FILE names a table that
 * prec_gpu_init loads. */
typedef struct {
    int log2_n;
    int log2_cols;      /* column length 2^log2_cols, row length 2^(log2_n - log2_cols) */
    int col_group;      /* columns per column-pass CTA: 4 or 8 */
    int col_radix_cap;  /* largest radix 2^cap of a column pass: 4 or 6 */
    int row_radix_cap;  /* largest radix 2^cap of a row pass: 4 or 6 */
    int rows_per_cta;   /* rows per row-pass CTA */
    int split_primes;   /* 1: per-prime stream chains for a single product */
    float ms;           /* measured product time (0: not measured) */
    float default_ms;   /* the default configuration's time (0: not measured) */
} prec_gpu_tune_entry_t;

/* Times the configurations of every length 2^kmin .. 2^kmax (clamped to
 * 13 .. 26) on the current device with balanced random operands of
 * 2^(k-2) limbs each, by coordinate descent from the default (per-prime
 * streams, rows per CTA, columns per CTA, radix caps, then the column/row
 * split).  A candidate counts only if its product equals the default
 * configuration's bit for bit; the fastest is installed.  Writes up to
 * `cap` entries to `out` (may be NULL) and the number of lengths to *count. */
int prec_gpu_autotune(int kmin, int kmax, prec_gpu_tune_entry_t *out, size_t cap, size_t *count);

/* The configuration length 2^log2_n uses now (tuned, set, loaded or default). */
int prec_gpu_tune_get(int log2_n, prec_gpu_tune_entry_t *entry);

/* Installs a configuration; PREC_GPU_E_ARG if no kernel exists for it. */
int prec_gpu_tune_set(const prec_gpu_tune_entry_t *entry);

/* Every length back to its default configuration. */
int prec_gpu_tune_reset(void);

/* The table as text, one line per tuned length.  Loading validates every
 * line and installs nothing if one is invalid (PREC_GPU_E_ARG). */
int prec_gpu_tune_save(const char *path);
int prec_gpu_tune_load(const char *path);

/* Kernel launches the library has issued in this process (every product,
 * batch graph replays included): a caller's own count of the GPU work
 * behind its calls. */
uint64_t prec_gpu_launch_count(void);

/* Digit width (bits) the FP64 band uses for an x bn limbs; 0 outside the band. */
int prec_gpu_fft_digit_bits(size_t an, size_t bn);

/* Same product on device pointers, enqueued on `stream` (a cudaStream_t;
 * NULL = legacy default stream) without host synchronisation.  Operands
 * stay as given (no trimming of zero high limbs).  The call returns after
 * enqueueing; device-side failures (bounded waits) are reported by
 * prec_gpu_stream_check.  Successive calls from one thread share that
 * thread's workspace and are ordered after one another even across
 * streams; calls from different threads use separate workspaces and may
 * run concurrently.  d_out must not
 * overlap the operands.  Operands above the block size run blocked (see
 * prec_gpu_set_block_limbs). */
int prec_gpu_mul_device(const uint64_t *d_a, size_t an, const uint64_t *d_b, size_t bn,
                        uint64_t *d_out, void *stream);

/* Diagnostic form of prec_gpu_mul_device: records a CUDA event on `stream`
 * before the first and after every kernel of the product, synchronises,
 * and writes each kernel's device time (ms) to stage_ms[0 .. *nstages)
 * (at most 8).  Kernel names: prec_gpu_stage_name(path, i) with the path of
 * prec_gpu_stats_t.  Replaces: the wall-clock phase timers of the
 * reference's benches (test/bench_ntt.cpp:25-58, pi/pi_chudnovsky.cpp:183-188). */
int prec_gpu_mul_device_profile(const uint64_t *d_a, size_t an, const uint64_t *d_b, size_t bn,
                                uint64_t *d_out, void *stream, float *stage_ms, int *nstages);

/* Kernel name of stage `stage` of path `path` ("" if out of range). */
const char *prec_gpu_stage_name(int path, int stage);

/* The product of prec_gpu_mul_device for callers that cannot allocate device
 * memory (their memory is owned by their own pool allocator, they cannot
 * accept the device-wide synchronisation that cudaFree implies, or their
 * host forbids allocation after start-up).  No counterpart in the
 * reference.  Allocates nothing: the caller passes inputs and output on
 * the device; all other memory is a fixed array inside the library
 * (about 6.6 MiB, held by every device that loads the library until the
 * process exits).  Limit: an + bn <= 131072 limbs (transforms up to 2^18
 * points); larger products return PREC_GPU_E_TOO_LARGE.  The first call on
 * a device sets that device up (fills the library's twiddle tables with a
 * kernel on `stream` and waits for it), so make the first call before any
 * stream capture.  A device reset (cudaDeviceReset) discards those tables:
 * after one, use this entry point only in a new process.  Calls share the
 * one array: calls that overlap on the GPU (other streams, other threads)
 * race and corrupt each other's result; serialise them.  Asynchronous
 * otherwise: the call itself reports size and argument errors (sizes are
 * checked first, before any CUDA call) and launch errors; an error bit its
 * kernels raise (an internal fault) stays in a library word until
 * prec_gpu_stream_check, which reads and clears it without allocating. */
int prec_gpu_mul_device_noalloc(const uint64_t *d_a, size_t an, const uint64_t *d_b, size_t bn,
                                uint64_t *d_out, void *stream);

/* ---- batch form: many independent products of uneven sizes -------------
 * Replaces: nothing one-to-one; the reference forms products one at a time
 * (operator*, src/mul_basic.cpp:278-284), including the independent
 * products of one binary-splitting level (pi/pi_chudnovsky.cpp:141-144).
 * All pointers are device pointers; out receives an+bn limbs.  The products
 * run concurrently: no output may overlap an operand or another output of
 * the same batch. */
typedef struct prec_gpu_product {
    const uint64_t *a;
    size_t an;
    const uint64_t *b;
    size_t bn;
    uint64_t *out;
} prec_gpu_product_t;

typedef struct prec_gpu_batch prec_gpu_batch_t;

/* Plans a batch: groups the products by transform length (length classes),
 * allocates their descriptors and workspaces.  No product is computed. */
int prec_gpu_batch_create(const prec_gpu_product_t *items, size_t count, prec_gpu_batch_t **batch);

/* Computes every product of the batch on `stream` (asynchronous).  The first
 * call records the work into a CUDA graph, built node by node (one branch
 * per length class); later calls replay it, recomputing the products from the current
 * contents of the same operand buffers.  Device-side failures are reported
 * by prec_gpu_stream_check. */
int prec_gpu_batch_run(prec_gpu_batch_t *batch, void *stream);

/* Number of length classes and device bytes the batch holds. */
int prec_gpu_batch_info(const prec_gpu_batch_t *batch, size_t *classes, size_t *device_bytes);

/* Waits for the device and frees the batch. */
void prec_gpu_batch_destroy(prec_gpu_batch_t *batch);

/* One-shot batch on `stream`, synchronous (plan, run without a graph, free);
 * returns the device-side failures too (as prec_gpu_stream_check would). */
int prec_gpu_mul_batch(const prec_gpu_product_t *items, size_t count, void *stream);

/* ---- serving loop: continuous admission of requests ---------------------
 * Replaces: nothing in the reference (single-threaded, one product per
 * call).  A server owns `slots` CUDA streams, a private memory pool and a
 * worker thread.  Requests (device-resident operands and output) are
 * admitted while a slot is free and the transform workspace fits
 * `hbm_budget_bytes`; admitted requests run concurrently on their own
 * streams.  Latency = host time from submit to observed completion. */
typedef struct prec_gpu_server prec_gpu_server_t;

typedef struct prec_gpu_serve_stats {
    uint64_t submitted, completed, failed;
    double p50_ms, p99_ms, mean_ms, max_ms;  /* latency of completed requests */
    double products_per_s;                   /* completed / (last completion - first submit) */
    size_t peak_bytes;                       /* largest admitted workspace total */
    int peak_in_flight;                      /* most requests on the GPU at once */
} prec_gpu_serve_stats_t;

int prec_gpu_serve_create(size_t hbm_budget_bytes, int slots, prec_gpu_server_t **server);

/* Queues one product; returns at once with its ticket.  PREC_GPU_E_NOMEM if
 * its workspace alone exceeds the budget. */
int prec_gpu_serve_submit(prec_gpu_server_t *server, const uint64_t *d_a, size_t an, const uint64_t *d_b,
                          size_t bn, uint64_t *d_out, uint64_t *ticket);

/* Waits (host side, at most timeout_s) for one ticket; returns its status
 * and latency, or PREC_GPU_E_TIMEOUT. */
int prec_gpu_serve_wait(prec_gpu_server_t *server, uint64_t ticket, double timeout_s, double *latency_ms);

/* Waits (host side, at most timeout_s) until every submitted request completed. */
int prec_gpu_serve_drain(prec_gpu_server_t *server, double timeout_s);

int prec_gpu_serve_stats(prec_gpu_server_t *server, prec_gpu_serve_stats_t *stats);

/* Finishes the queued work, stops the worker and frees the server. */
void prec_gpu_serve_destroy(prec_gpu_server_t *server);

/* Synchronises `stream` and reports any device-side error raised by work
 * the library enqueued (PREC_GPU_E_TIMEOUT, PREC_GPU_E_INTERNAL) or a
 * CUDA error. */
int prec_gpu_stream_check(void *stream);

/* Report of the last completed host-pointer call on this thread. */
int prec_gpu_last_stats(prec_gpu_stats_t *st);

/* Transform length log2 the NTT band uses for an x bn limbs; 0 when the
 * product runs blocked (an operand above the block size). */
int prec_gpu_ntt_log2(size_t an, size_t bn);

/* Digits of NTT-band products (prec_gpu_mul, prec_gpu_sqr,
 * prec_gpu_mul_ntt, prec_gpu_mul_device, the batch form and the serving
 * loop).  1 (the default; the environment variable PREC_GPU_WIDE_DIGITS=0
 * starts at 0): a product whose operands both fit in the lower half of a
 * transform of 2^18 .. 2^25 points takes whole 64-bit limbs as digits over
 * five primes -- half the points of the 32-bit-digit transform -- when
 * that needs fewer butterflies.  0: 32-bit digits over three primes.  The
 * result is the same either way.  Returns the previous setting.  No
 * counterpart in the reference, whose mul_ntt splits limbs into 16-bit
 * digits (src/mul_ntt.cpp:331-342). */
int prec_gpu_set_wide_digits(int on);

/* Block size of blocked products, in limbs (default and maximum 2^24 =
 * 16,777,216; at least 1024; 0 restores the default).  A product through
 * prec_gpu_mul, prec_gpu_sqr, prec_gpu_mul_ntt or prec_gpu_mul_device
 * whose larger operand exceeds it is cut into blocks of at most this many
 * limbs: every pair of blocks is one NTT-band product, added into the
 * result at its offset on the device.  Replaces: the reference's mul_ntt
 * guard that hands operands above 2^24 limbs to mul_fft
 * (src/mul_ntt.cpp:494-518).  Returns the previous setting. */
size_t prec_gpu_set_block_limbs(size_t limbs);

/* Static text for an error code. */
const char *prec_gpu_strerror(int code);

#ifdef __cplusplus
}
#endif

#endif /* PREC_GPU_H */
