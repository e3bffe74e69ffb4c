/*
 * gbfft -- batched power-of-two complex-to-complex FFT for GB300 (sm_103a).
 *
 * C ABI behind which the GB300 kernels sit.  It is the boundary a binding of
 * larsjoost/wgls-rs-fft's `GpuFft` (src/lib.rs:75-950) calls: plain pointers
 * and sizes, no CUDA or torch types in the signatures (streams are `void*`
 * holding a cudaStream_t).
 *
 * Data layout: complex<f32> interleaved (re, im), transforms stored
 * back-to-back (batch-major), exactly the layout the reference uploads
 * (src/lib.rs:539-548).
 *
 * Transform definitions (src/lib.rs:433-488):
 *   forward  (GBFFT_FORWARD):  X_k = sum_n x_n e^{-2 pi i k n / N}   (unscaled)
 *   inverse  (GBFFT_INVERSE):  x_n = (1/N) sum_k X_k e^{+2 pi i k n / N}
 * The reference computes the inverse as conj(FFT(conj x)) * (1/N)
 * (src/lib.rs:571-579, 661-669); that is the same transform.
 *
 * A context is not thread-safe: use one per host thread, as the reference's
 * GpuFft (RefCell cache, src/lib.rs:81) is single-threaded.
 */
#ifndef GBFFT_H
#define GBFFT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBFFT_FORWARD (-1)
#define GBFFT_INVERSE (+1)

/* Status codes.  Messages for the first two are the reference's own strings. */
typedef enum gbfft_status {
    GBFFT_OK = 0,
    /* "Transform length must be a non-zero power of two" (src/lib.rs:506-511) */
    GBFFT_ERR_INVALID_SIZE = 1,
    /* "All input vectors in a batch must have the same length" (src/lib.rs:526-533) */
    GBFFT_ERR_LENGTH_MISMATCH = 2,
    GBFFT_ERR_INVALID_ARGUMENT = 3, /* null pointer, bad direction or precision */
    GBFFT_ERR_NO_DEVICE = 4,        /* no usable GB300 (sm_103) device */
    GBFFT_ERR_OUT_OF_MEMORY = 5,    /* device or pinned host allocation failed */
    GBFFT_ERR_CUDA = 6,             /* a CUDA runtime call failed; see gbfft_last_error */
    GBFFT_ERR_TIMEOUT = 7,          /* a bounded device-side wait gave up */
    GBFFT_ERR_UNSUPPORTED = 8       /* size/precision combination not provided */
} gbfft_status;

/* Arithmetic used for the butterflies. */
typedef enum gbfft_precision {
    GBFFT_PREC_FP32 = 0,      /* plain FP32 Stockham form (every size) */
    GBFFT_PREC_TC_FP16 = 1,   /* radix-16 sub-DFTs as tcgen05 matrix products, FP16 hi+lo operands
                                 (3 products), per-vector power-of-two scaling, FP32 accumulation;
                                 N >= 16 (TF32: single-pass sizes up to 2^13, then N >= 2^15) */
    GBFFT_PREC_TC_BF16X3 = 2, /* same with BF16 hi+lo operands */
    GBFFT_PREC_TC_TF32 = 3,   /* same with TF32 hi+lo operands (hi = the value rounded to TF32,
                                 lo = the exact rest); TF32 keeps FP32's exponent range, so no
                                 scaling */
    GBFFT_PREC_TC_BF16X6 = 4  /* BF16 operands split in three (hi + mid + lo: 24 significant bits),
                                 six products (hh, hm, mh, hl, lh, mm), no scaling: the BF16 form
                                 inside the FP32 form's error budget */
} gbfft_precision;

typedef struct gbfft_ctx gbfft_ctx;

/* Replaces GpuFft::is_gpu_available (src/lib.rs:381-389): 1 when a usable
 * sm_103 device is present, else 0.  Creates no context. */
int gbfft_is_available(void);

/* Replaces GpuFft::new (src/lib.rs:285-330): selects `device`, creates the
 * context's stream.  No kernel JIT; plans are built on first use of a size. */
int gbfft_create(int device, gbfft_ctx **out_ctx);

/* Replaces Drop for GpuFft: frees plans, device buffers, pinned staging. */
void gbfft_destroy(gbfft_ctx *ctx);

/* Message for the most recent failing call on `ctx` ("" if none).  The string
 * is owned by the context and valid until the next call on it. */
const char *gbfft_last_error(const gbfft_ctx *ctx);

/* Static description of a status code. */
const char *gbfft_status_string(int status);

/* Replaces GpuFft::fft / GpuFft::ifft (src/lib.rs:433-438, 483-488) via
 * transform_batch_internal (src/lib.rs:517-568) for a contiguous host batch:
 * `in` and `out` hold batch*n interleaved complex<f32> (they may alias).
 * Copies to the device, transforms, copies back and returns when `out` holds
 * the result.  batch == 0 returns GBFFT_OK without touching the pointers
 * (src/lib.rs:522-524). */
int gbfft_c2c_host(gbfft_ctx *ctx, const float *in, float *out, uint64_t n,
                   uint64_t batch, int direction);

/* Same, for the reference's own argument shape &[Vec<Complex<f32>>]
 * (src/lib.rs:433, 517-533): `batch` separate rows, row i at in_rows[i] with
 * row_lengths[i] complex values, result row i written to out_rows[i].
 * All lengths must be equal (GBFFT_ERR_LENGTH_MISMATCH) and a power of two
 * (GBFFT_ERR_INVALID_SIZE), checked in the reference's order.  Where the
 * device reaches pageable host memory through the host's page tables
 * (cudaDevAttrPageableMemoryAccess: NVLink-C2C on Grace), the GPU gathers the
 * rows into device memory and scatters the results into out_rows itself,
 * chunk by chunk; elsewhere they are copied through pinned staging on host
 * threads.  Either way out_rows[i] may be in_rows[i] (in place) but must not
 * overlap any other input row.  The same applies to gbfft_c2c_host with a
 * pageable (not cudaHostAlloc'd) batch. */
int gbfft_c2c_host_rows(gbfft_ctx *ctx, const float *const *in_rows,
                        const uint64_t *row_lengths, float *const *out_rows,
                        uint64_t batch, int direction);

/* Device-resident entry point (new; no reference counterpart -- the reference
 * always round-trips through host memory).  `d_in`/`d_out` are device
 * pointers to batch*n interleaved complex<f32>; they may alias and need only
 * the alignment of complex<f32> (8 bytes: every kernel reads and writes
 * caller memory one sample at a time; wider accesses touch only the
 * library's own buffers).  Work is
 * enqueued on `stream` (a cudaStream_t; NULL is the CUDA default stream, as
 * everywhere in CUDA) and the call returns without synchronising. */
int gbfft_c2c_device(gbfft_ctx *ctx, const void *d_in, void *d_out, uint64_t n,
                     uint64_t batch, int direction, void *stream);

/* Allocation-free variant of gbfft_c2c_device (no counterpart in the
 * reference).  For callers that may not allocate GPU memory -- code inside
 * another library's allocator hook (allocating there would re-enter the
 * allocator), under a memory pool that owns all of the device's memory, or on
 * a latency path where cudaMalloc/cudaFree and the synchronisation they imply
 * are not acceptable.  It never calls cudaMalloc, cudaFree or any allocating
 * routine, and it needs no context.  It launches kernels, so like any CUDA
 * call it must not be made from a stream's host callback.
 *
 * Limits: n a power of two with 2^15 <= n <= 2^20 and n * batch <= 2^22
 * (the library's built-in 32 MiB scratch array); anything larger or smaller
 * returns GBFFT_ERR_UNSUPPORTED, a non-power-of-two n GBFFT_ERR_INVALID_SIZE.
 * Device pointers and stream as for gbfft_c2c_device; runs on the current
 * device.  The first call on each device sets up (looks up the scratch and
 * twiddle arrays and fills the tables) and synchronises `stream`: make that
 * first call before any stream capture; the set-up is not redone after a
 * cudaDeviceReset, so do not call this entry on a device after resetting it.
 * All calls on a device share the one scratch array, so calls that overlap on
 * the GPU race: serialise them.  It runs the plain two-pass schedule (one
 * launch per pass), 10-15 % slower at these sizes than gbfft_c2c_device's
 * fused pass pair. */
int gbfft_c2c_device_noalloc(const void *d_in, void *d_out, uint64_t n,
                             uint64_t batch, int direction, void *stream);

/* ---- ragged batches (no reference counterpart: the reference rejects rows
 * of different lengths, src/lib.rs:526-533, so mixed sizes cost one call per
 * size there) ---------------------------------------------------------------
 * Transforms of mixed power-of-two lengths (2^0 .. 2^18) and directions,
 * packed anywhere in one device buffer, run in ONE persistent kernel launch
 * fed by a device work queue.  Descriptor i transforms the 2^log2n complex
 * samples starting `offset` samples into d_in and writes them at the same
 * offset in d_out.  Transforms must not overlap each other; d_in may equal
 * d_out. */
typedef struct gbfft_ragged_desc {
    uint64_t offset;   /* in complex samples */
    uint32_t log2n;    /* 0 .. 18 */
    int32_t direction; /* GBFFT_FORWARD or GBFFT_INVERSE */
} gbfft_ragged_desc;

typedef struct gbfft_ragged_plan gbfft_ragged_plan;

/* Options for gbfft_ragged_plan_set. */
#define GBFFT_RAGGED_OPT_SPIN_LIMIT 1          /* polls before a dependency wait gives up */
#define GBFFT_RAGGED_OPT_TEST_DROP_PRODUCERS 2 /* test hook: omit first-pass items */
#define GBFFT_RAGGED_OPT_LAG 3                 /* queue distance from a transform's first-pass items to its
                                                  second-pass items, in items per SM (1..64, default 4):
                                                  larger waits less, smaller keeps the intermediate in L2 */

/* Build the work queue, twiddle tables and workspace for a descriptor set
 * (validated here; errors are reported on `ctx`). */
int gbfft_ragged_plan_create(gbfft_ctx *ctx, const gbfft_ragged_desc *descs, uint32_t count,
                             gbfft_ragged_plan **out_plan);

int gbfft_ragged_plan_set(gbfft_ragged_plan *plan, int option, uint64_t value);

/* Enqueue the plan on `stream` (NULL = default stream).  `capacity` is the
 * size of d_in and of d_out in complex samples; a descriptor reaching past it
 * is rejected (GBFFT_ERR_INVALID_ARGUMENT) before anything is launched.  With
 * use_graph != 0 the reset + launch sequence is captured once into a CUDA
 * graph (per (d_in, d_out) pair) and replayed.  Asynchronous: call
 * gbfft_ragged_wait. */
int gbfft_ragged_execute(gbfft_ragged_plan *plan, const void *d_in, void *d_out, uint64_t capacity,
                         int use_graph, void *stream);

/* Synchronise `stream` and report GBFFT_ERR_TIMEOUT if a dependency wait of
 * the last execution gave up. */
int gbfft_ragged_wait(gbfft_ragged_plan *plan, void *stream);

/* Number of kernel launches issued by the plan so far. */
uint64_t gbfft_ragged_launch_count(const gbfft_ragged_plan *plan);

void gbfft_ragged_plan_destroy(gbfft_ragged_plan *plan);

/* One-shot: create, execute (no graph), wait, destroy. */
int gbfft_ragged_device(gbfft_ctx *ctx, const void *d_in, void *d_out, uint64_t capacity,
                        const gbfft_ragged_desc *descs, uint32_t count, void *stream);

/* Replaces GpuFftTrait::benchmark_gpu_only (src/lib.rs:108-156, 673-707):
 * device-only timing of `iters` transforms of an n x batch device batch after
 * `warmup` untimed ones, with CUDA events on the context's stream.  Writes the
 * mean seconds per transform. */
int gbfft_bench_device(gbfft_ctx *ctx, uint64_t n, uint64_t batch, int direction,
                       int warmup, int iters, double *seconds_per_iter);

/* Select the butterfly arithmetic for later calls on `ctx`. */
int gbfft_set_precision(gbfft_ctx *ctx, int precision);

/* Window applied to every input sample as the transform loads it (fused: no
 * extra pass over memory).  GBFFT_WINDOW_HANN multiplies sample n of each
 * length-N row by w_n = 0.5 (1 - cos(2 pi n / (N - 1))) -- the reference's
 * host-side Hann window (tests/test_utils.rs:39-48, examples/windowed_fft.rs:
 * 14-23) -- with w computed in FP64 and rounded once to f32; N = 1 uses w = 1.
 * Applies to later gbfft_c2c_host / _host_rows / _device calls on `ctx` with
 * N <= 2^24 (larger N returns GBFFT_ERR_UNSUPPORTED while a window is set). */
#define GBFFT_WINDOW_NONE 0
#define GBFFT_WINDOW_HANN 1
int gbfft_set_window(gbfft_ctx *ctx, int window);

/* Gaussian noise added to every input sample as the transform loads it (fused:
 * no extra pass), before the window: the reference pipeline's NOISE stage
 * (examples/parallel_pipeline.rs:30-62).  Sample n of row b receives
 * (r cos u2, r sin u2) with h1 = pcg(n * 1234567 + b * 7654321 + seed),
 * h2 = pcg(h1 + 999983), u1 = max(h1 / 2^32, 1e-7), u2 = 2 pi h2 / 2^32,
 * r = sigma sqrt(-2 ln u1) (the reference uses sigma = 0.1).  The hash is
 * exact; log/sqrt/sin/cos are FP32 library functions.  sigma = 0 turns it off.
 * With the Hann window on an inverse transform this gives the reference's
 * noise -> FFT -> window -> IFFT -> scale pipeline in two launches. */
int gbfft_set_noise(gbfft_ctx *ctx, uint32_t seed, float sigma);

/* Autotuner (no reference counterpart; the reference's find_optimal_batch
 * example only sweeps batch sizes, examples/find_optimal_batch.rs:28).  Times
 * every plan variant for (n, batch, direction, current precision) -- global
 * pass split, plain or persistent tile-loop kernels, fused pass pairs,
 * transforms per CTA of the single-pass kernel, columns per CTA of a
 * three-pass first pass, 16 or 32 samples a thread -- on the context's own
 * scratch buffers (caller data is never touched), keeps the fastest for later
 * calls with that size, direction, precision and a batch of the same power of
 * two, and writes the mean seconds per transform of the winner.  If the
 * environment variable GBFFT_AUTOTUNE_CACHE names a file, results are loaded
 * from it when a context is created and appended to it here.  Setting
 * GBFFT_AUTOTUNE=1 makes the first call of every untuned combination tune
 * itself. */
int gbfft_autotune(gbfft_ctx *ctx, uint64_t n, uint64_t batch, int direction, double *best_seconds);

/* Environment read by the library:
 *   GBFFT_AUTOTUNE, GBFFT_AUTOTUNE_CACHE   see gbfft_autotune
 *   GBFFT_AUTOTUNE_VERBOSE=1               print every timed plan variant to stderr
 *   GBFFT_PRECISION=tc_fp16|tc_bf16x3|tc_tf32|tc_bf16x6  default precision of new contexts
 *   GBFFT_HOST_CHUNK_BYTES=<bytes>         chunk of the host-batch pipeline (32 MB)
 *   GBFFT_HOST_PATH=staged                 pageable host batches go through pinned
 *                                          staging even where the GPU could reach
 *                                          them directly
 *   GBFFT_HOST_PATH=gather                 the GPU copies pageable rows into device
 *                                          memory and back around every transform
 *                                          instead of the transform reading and
 *                                          writing them itself
 *   GBFFT_PREFAULT=0                       do not populate absent pages of a pageable
 *                                          output before the GPU writes it (by
 *                                          default outputs of 128 KB and more are
 *                                          checked with mincore and their absent
 *                                          pages populated: a GPU write to a page
 *                                          the process has never touched faults
 *                                          through the SMMU, ~20 us per 64 KB page)
 *   GBFFT_DEVICE_ALLOC_CAP=<bytes>         device requests above it fail with
 *                                          GBFFT_ERR_OUT_OF_MEMORY (tests the
 *                                          out-of-memory paths without a real one) */

/* Number of kernel launches this context has issued since creation (all
 * entry points).  Lets callers count GPU work without a profiler. */
uint64_t gbfft_launch_count(const gbfft_ctx *ctx);

/* Library version string. */
const char *gbfft_version(void);

#ifdef __cplusplus
}
#endif

#endif /* GBFFT_H */
