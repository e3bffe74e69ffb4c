// C ABI of the GB300 FFT (declared in include/gbfft.h).
//
// Mirrors the reference's GpuFft (larsjoost/wgls-rs-fft src/lib.rs:75-950):
//   GpuFft::new                  -> gbfft_create        (src/lib.rs:285-330)
//   GpuFft::is_gpu_available     -> gbfft_is_available  (src/lib.rs:381-389)
//   GpuFft::fft / ifft           -> gbfft_c2c_host(_rows) (src/lib.rs:433-568)
//   SizeCache / build_size_cache -> Plan / plan_for     (src/lib.rs:230-259, 709-943)
//   benchmark_gpu_only           -> gbfft_bench_device  (src/lib.rs:673-707)
// plus the device-resident entry gbfft_c2c_device.
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <memory>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "gbfft_internal.h"
#include "gbfft_plan.h"
#include "gbfft_ragged.h"
#include "host_pages.h"

using namespace gbfft;

struct gbfft_ragged_plan {
    gbfft_ctx *ctx;
    RaggedPlanImpl *impl;
};

// Host threads that copy a batch between caller memory and pinned staging:
// started on first use, kept for the context's life.  run(f) calls f(k, n)
// on the calling thread (k = 0) and every worker (k = 1 .. n-1) and returns
// when all have finished.
class CopyPool {
   public:
    explicit CopyPool(unsigned n) : n_(n) {
        for (unsigned k = 1; k < n_; ++k) workers_.emplace_back([this, k] { loop(k); });
    }
    ~CopyPool() {
        {
            std::lock_guard<std::mutex> g(m_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto &t : workers_) t.join();
    }
    unsigned size() const { return n_; }
    void run(const std::function<void(unsigned, unsigned)> &f) {
        {
            std::lock_guard<std::mutex> g(m_);
            job_ = &f;
            pending_ = n_ - 1;
            ++gen_;
        }
        cv_.notify_all();
        f(0, n_);
        std::unique_lock<std::mutex> l(m_);
        done_.wait(l, [this] { return pending_ == 0; });
        job_ = nullptr;
    }

   private:
    void loop(unsigned k) {
        unsigned seen = 0;
        for (;;) {
            const std::function<void(unsigned, unsigned)> *job;
            {
                std::unique_lock<std::mutex> l(m_);
                cv_.wait(l, [&] { return stop_ || gen_ != seen; });
                if (stop_) return;
                seen = gen_;
                job = job_;
            }
            (*job)(k, n_);
            std::lock_guard<std::mutex> g(m_);
            if (--pending_ == 0) done_.notify_one();
        }
    }
    unsigned n_;
    std::vector<std::thread> workers_;
    std::mutex m_;
    std::condition_variable cv_, done_;
    const std::function<void(unsigned, unsigned)> *job_ = nullptr;
    unsigned pending_ = 0, gen_ = 0;
    bool stop_ = false;
};

struct gbfft_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t xfer[3] = {nullptr, nullptr, nullptr};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::string err;
    // plans by (logn, precision, variant); tuned variant by (logn, precision, direction, log2 batch)
    std::map<std::tuple<int, int, PlanVariant>, std::unique_ptr<Plan>> plans;
    std::map<std::tuple<int, int, int, int>, PlanVariant> tuned;
    int window = GBFFT_WINDOW_NONE;
    uint32_t noise_seed = 0;
    float noise_sigma = 0.f;  // 0: no noise added on load
    std::map<int, std::unique_ptr<DeviceBuffer>> windows;  // Hann tables by log2 N
    bool auto_tune = false;
    bool tune_verbose = false;  // GBFFT_AUTOTUNE_VERBOSE=1: per-variant timings on stderr
    std::string tune_cache;
    DeviceBuffer tune_a, tune_b;  // scratch for the autotuner
    DeviceBuffer dbuf;    // device copy of a host batch
    DeviceBuffer dbuf_out;  // its transform (out of place: fused pairs, no shared workspace)
    std::unique_ptr<CopyPool> copy_pool;  // staging copies of pageable host batches
    DeviceBuffer ws;      // multi-pass workspace
    // counter blocks of the fused two-pass form, one per stream so that calls
    // on different streams never share one
    std::map<cudaStream_t, std::unique_ptr<DeviceBuffer>> fused_ctr;
    uint32_t *d_err = nullptr;  // raised by tensor-core and fused kernels when a bounded wait gives up
    bool err_armed = false;     // a kernel that can raise d_err was enqueued since it was last read
    void *hstage = nullptr;
    size_t hstage_bytes = 0;
    uint64_t launches = 0;
    int precision = GBFFT_PREC_FP32;
    size_t host_chunk = (size_t)32 << 20;  // bytes of a host batch per pipelined copy (GBFFT_HOST_CHUNK_BYTES)
    // Pageable host batches and separate rows are moved by the GPU itself through
    // the host's page tables when the device can (cudaDevAttrPageableMemoryAccess;
    // GBFFT_HOST_PATH=staged turns it off): no host memcpy, no pinned staging.
    bool host_direct = false;
    bool host_gather = false;  // GBFFT_HOST_PATH=gather: copy kernels around every transform
    bool prefault = true;      // GBFFT_PREFAULT=0: let the GPU fault the caller's output pages in itself
    int sms = 0;
    DeviceBuffer dtable;          // device copy of the caller's row pointers (in, then out)
    uint64_t *htable = nullptr;   // its pinned source
    size_t htable_bytes = 0;
    cudaEvent_t ev_table = nullptr;
};

namespace {

const char *kMsgInvalidSize = "Transform length must be a non-zero power of two";
const char *kMsgLengthMismatch = "All input vectors in a batch must have the same length";

int fail(gbfft_ctx *ctx, int status, const char *fmt, ...) {
    if (ctx) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        ctx->err = buf;
    }
    return status;
}

int cuda_fail(gbfft_ctx *ctx, cudaError_t e, const char *what) {
    if (e == cudaErrorMemoryAllocation)
        return fail(ctx, GBFFT_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
    return fail(ctx, GBFFT_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define GB_CUDA(ctx, call)                                   \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

bool is_pow2(uint64_t n) { return n != 0 && (n & (n - 1)) == 0; }
int log2u(uint64_t n) {
    int l = 0;
    while ((1ull << l) < n) ++l;
    return l;
}

bool device_supported(int dev) {
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, dev) != cudaSuccess) return false;
    return p.major == 10 && p.minor == 3;  // kernels are built for sm_103a only
}

int host_is_pinned(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return a.type == cudaMemoryTypeHost;
}

int ensure_hstage(gbfft_ctx *ctx, size_t bytes) {
    if (ctx->hstage_bytes >= bytes) return GBFFT_OK;
    if (ctx->hstage) cudaFreeHost(ctx->hstage);
    ctx->hstage = nullptr;
    ctx->hstage_bytes = 0;
    cudaError_t e = cudaHostAlloc(&ctx->hstage, bytes, cudaHostAllocDefault);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, GBFFT_ERR_OUT_OF_MEMORY, "pinned staging of %zu bytes: %s", bytes,
                    cudaGetErrorString(e));
    }
    ctx->hstage_bytes = bytes;
    return GBFFT_OK;
}

int get_plan(gbfft_ctx *ctx, int logn, const PlanVariant &v, Plan **out) {
    const auto key = std::make_tuple(logn, ctx->precision, v);
    auto it = ctx->plans.find(key);
    if (it != ctx->plans.end()) {
        *out = it->second.get();
        return GBFFT_OK;
    }
    std::unique_ptr<Plan> p(new Plan());
    std::string why;
    int st = plan_build(*p, logn, ctx->precision, v, ctx->stream, why);
    if (st != GBFFT_OK) return fail(ctx, st, "plan for N=2^%d: %s", logn, why.c_str());
    // Tables are filled on the context's stream; transforms may run on any
    // stream, so finish the fill before the plan is used (once per size).
    GB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *out = p.get();
    ctx->plans[key] = std::move(p);
    return GBFFT_OK;
}

// After a synchronisation: report (and clear) a device-side wait that gave up.
int check_device_flag(gbfft_ctx *ctx) {
    if (!ctx->err_armed) return GBFFT_OK;  // only FP32 kernels without waits ran: nothing can be raised
    ctx->err_armed = false;
    uint32_t v = 0;
    GB_CUDA(ctx, cudaMemcpy(&v, ctx->d_err, sizeof v, cudaMemcpyDeviceToHost));
    if (v != 0) {
        GB_CUDA(ctx, cudaMemset(ctx->d_err, 0, sizeof v));
        return fail(ctx, GBFFT_ERR_TIMEOUT,
                    "a bounded device wait gave up (tensor-core completion or fused-pass dependency)");
    }
    return GBFFT_OK;
}

int validate_common(gbfft_ctx *ctx, uint64_t n, int direction) {
    if (!ctx) return GBFFT_ERR_INVALID_ARGUMENT;
    if (direction != GBFFT_FORWARD && direction != GBFFT_INVERSE)
        return fail(ctx, GBFFT_ERR_INVALID_ARGUMENT, "direction must be -1 (forward) or +1 (inverse)");
    if (!is_pow2(n)) return fail(ctx, GBFFT_ERR_INVALID_SIZE, "%s", kMsgInvalidSize);
    if (log2u(n) > kMaxLogN)
        return fail(ctx, GBFFT_ERR_UNSUPPORTED, "transform length 2^%d exceeds 2^%d", log2u(n), kMaxLogN);
    if (ctx->window != GBFFT_WINDOW_NONE && log2u(n) > kWindowMaxLogN)
        return fail(ctx, GBFFT_ERR_UNSUPPORTED, "windows are provided for N <= 2^%d", kWindowMaxLogN);
    return GBFFT_OK;
}

int log2floor(uint64_t b) {
    int l = 0;
    while (b > 1) {
        b >>= 1;
        ++l;
    }
    return l;
}

std::tuple<int, int, int, int> tune_key(gbfft_ctx *ctx, int logn, uint64_t batch, int direction) {
    return std::make_tuple(logn, ctx->precision, direction, log2floor(batch));
}

int autotune(gbfft_ctx *ctx, uint64_t n, uint64_t batch, int direction, double *best_seconds);

PlanVariant choose_variant(gbfft_ctx *ctx, int logn, uint64_t batch, int direction, int &st) {
    st = GBFFT_OK;
    auto it = ctx->tuned.find(tune_key(ctx, logn, batch, direction));
    if (it != ctx->tuned.end()) return it->second;
    if (ctx->auto_tune) {
        double s = 0;
        st = autotune(ctx, 1ull << logn, batch, direction, &s);
        it = ctx->tuned.find(tune_key(ctx, logn, batch, direction));
        if (st == GBFFT_OK && it != ctx->tuned.end()) return it->second;
    }
    return plan_candidates(logn, ctx->precision).front();
}

// The window table for 2^logn samples when a window is selected, else nullptr.
int window_table(gbfft_ctx *ctx, int logn, const float **out) {
    *out = nullptr;
    if (ctx->window == GBFFT_WINDOW_NONE) return GBFFT_OK;
    if (logn > kWindowMaxLogN)
        return fail(ctx, GBFFT_ERR_UNSUPPORTED, "windows are provided for N <= 2^%d", kWindowMaxLogN);
    auto it = ctx->windows.find(logn);
    if (it == ctx->windows.end()) {
        std::unique_ptr<DeviceBuffer> b(new DeviceBuffer());
        int st = b->ensure(sizeof(float) << logn, ctx->err);
        if (st != GBFFT_OK) return fail(ctx, st, "%s", ctx->err.c_str());
        GB_CUDA(ctx, hann_fill((float *)b->ptr, 1ull << logn, ctx->stream));
        GB_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        it = ctx->windows.emplace(logn, std::move(b)).first;
    }
    *out = (const float *)it->second->ptr;
    return GBFFT_OK;
}

// Enqueue one transform of the whole device batch on `stream` with variant v.
int run_variant(gbfft_ctx *ctx, const float2 *in, float2 *out, uint64_t n, uint64_t batch, int direction,
                const PlanVariant &v, cudaStream_t stream, uint64_t row_base = 0) {
    Plan *plan = nullptr;
    int st = get_plan(ctx, log2u(n), v, &plan);
    if (st != GBFFT_OK) return st;
    const float *win = nullptr;
    st = window_table(ctx, log2u(n), &win);
    if (st != GBFFT_OK) return st;
    uint64_t launches = 0;
    std::string why;
    const LoadOps ops{win, ctx->noise_seed, ctx->noise_sigma, (uint32_t)row_base};
    DeviceBuffer *ctr = nullptr;
    if (plan->has_fused) {
        std::unique_ptr<DeviceBuffer> &b = ctx->fused_ctr[stream];
        if (!b) b.reset(new DeviceBuffer());
        ctr = b.get();
    }
    if (plan->has_fused || ctx->precision != GBFFT_PREC_FP32) ctx->err_armed = true;
    st = plan_execute(*plan, in, out, batch, direction, ctx->ws, ctx->d_err, stream, launches, why, ops, ctr);
    ctx->launches += launches;
    if (st != GBFFT_OK) return fail(ctx, st, "execute N=%llu batch=%llu: %s", (unsigned long long)n,
                                    (unsigned long long)batch, why.c_str());
    return GBFFT_OK;
}

// Time every candidate variant on scratch buffers; remember (and persist) the fastest.
int autotune(gbfft_ctx *ctx, uint64_t n, uint64_t batch, int direction, double *best_seconds) {
    const int logn = log2u(n);
    const size_t bytes = (size_t)n * batch * sizeof(float2);
    int st = ctx->tune_a.ensure(bytes, ctx->err);
    if (st == GBFFT_OK) st = ctx->tune_b.ensure(bytes, ctx->err);
    if (st != GBFFT_OK) return fail(ctx, st, "%s", ctx->err.c_str());
    float2 *a = (float2 *)ctx->tune_a.ptr, *b = (float2 *)ctx->tune_b.ptr;
    GB_CUDA(ctx, cudaMemsetAsync(a, 0, bytes, ctx->stream));
    const int reps = bytes >= ((size_t)256 << 20) ? 3 : 10;
    double best = 1e30;
    PlanVariant best_v = plan_candidates(logn, ctx->precision).front();
    for (const PlanVariant &v : plan_candidates(logn, ctx->precision)) {
        for (int w = 0; w < 2; ++w) {
            st = run_variant(ctx, a, b, n, batch, direction, v, ctx->stream);
            if (st != GBFFT_OK) break;
        }
        if (st != GBFFT_OK) {
            st = GBFFT_OK;  // a variant that cannot run is skipped
            continue;
        }
        GB_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
        for (int r = 0; r < reps; ++r) {
            st = run_variant(ctx, a, b, n, batch, direction, v, ctx->stream);
            if (st != GBFFT_OK) return st;
        }
        GB_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
        GB_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
        float ms = 0.f;
        GB_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
        const double s = (double)ms * 1e-3 / reps;
        if (ctx->tune_verbose)
            fprintf(stderr,
                    "gbfft autotune N=2^%d batch=%llu dir=%d prec=%d max_logr=%d persistent=%d fused=%d "
                    "tile=%d loge=%d tma=%d: %.3f us\n",
                    logn, (unsigned long long)batch, direction, ctx->precision, v.max_logr, v.persistent ? 1 : 0,
                    v.fused ? 1 : 0, v.tile, v.loge, v.tma ? 1 : 0,
                    s * 1e6);
        if (s < best) {
            best = s;
            best_v = v;
        }
    }
    st = check_device_flag(ctx);
    if (st != GBFFT_OK) return st;
    ctx->tuned[tune_key(ctx, logn, batch, direction)] = best_v;
    if (best_seconds) *best_seconds = best;
    if (!ctx->tune_cache.empty()) {
        FILE *f = fopen(ctx->tune_cache.c_str(), "a");
        if (f) {
            fprintf(f,
                    "{\"arch\": \"sm_103\", \"logn\": %d, \"precision\": %d, \"direction\": %d, \"batch_log2\": %d, "
                    "\"max_logr\": %d, \"persistent\": %d, \"fused\": %d, \"tile\": %d, \"loge\": %d, "
                    "\"tma\": %d, \"seconds\": %.9g}\n",
                    logn, ctx->precision, direction, log2floor(batch), best_v.max_logr, best_v.persistent ? 1 : 0,
                    best_v.fused ? 1 : 0, best_v.tile, best_v.loge, best_v.tma ? 1 : 0,
                    best);
            fclose(f);
        }
    }
    return GBFFT_OK;
}

void load_tune_cache(gbfft_ctx *ctx) {
    FILE *f = fopen(ctx->tune_cache.c_str(), "r");
    if (!f) return;
    char line[512];
    while (fgets(line, sizeof line, f)) {
        int logn, prec, dir, blog, mlr, pers, fused, tile, loge = 4, tma = 0;
        double sec;
        // lines written before the "loge" / "tma" keys existed read as loge 4 / tma 0
        const char *head =
            "{\"arch\": \"sm_103\", \"logn\": %d, \"precision\": %d, \"direction\": %d, \"batch_log2\": %d, "
            "\"max_logr\": %d, \"persistent\": %d, \"fused\": %d, \"tile\": %d, ";
        const std::string with_tma = std::string(head) + "\"loge\": %d, \"tma\": %d, \"seconds\": %lf}";
        const std::string with_loge = std::string(head) + "\"loge\": %d, \"seconds\": %lf}";
        const std::string without = std::string(head) + "\"seconds\": %lf}";
        const bool ok = sscanf(line, with_tma.c_str(), &logn, &prec, &dir, &blog, &mlr, &pers, &fused, &tile, &loge,
                               &tma, &sec) == 11 ||
                        (tma = 0, sscanf(line, with_loge.c_str(), &logn, &prec, &dir, &blog, &mlr, &pers, &fused,
                                         &tile, &loge, &sec) == 10) ||
                        (loge = 4, sscanf(line, without.c_str(), &logn, &prec, &dir, &blog, &mlr, &pers, &fused, &tile,
                                          &sec) == 9);
        if (ok)
            ctx->tuned[std::make_tuple(logn, prec, dir, blog)] =
                PlanVariant{mlr, pers != 0, fused != 0, tile, loge, tma != 0};
    }
    fclose(f);
}

// Enqueue one transform of the whole device batch on `stream`.
// row_base: batch index of in[0] within the caller's batch (keeps the fused
// noise stream continuous when a host batch is processed in chunks).
int run_device(gbfft_ctx *ctx, const float2 *in, float2 *out, uint64_t n, uint64_t batch, int direction,
               cudaStream_t stream, uint64_t row_base = 0) {
    int st = GBFFT_OK;
    const PlanVariant v = choose_variant(ctx, log2u(n), batch, direction, st);
    if (st != GBFFT_OK) return st;
    return run_variant(ctx, in, out, n, batch, direction, v, stream, row_base);
}

// Copy rows [r0, r1) between caller memory and the pinned stage (rows back to
// back), split by stage byte ranges over the context's copy threads (one
// thread below 1 MB), so even a single large row is copied in parallel.
constexpr unsigned kCopyThreads = 8;
template <class RowPtr>
static void copy_rows(gbfft_ctx *ctx, char *stage, RowPtr row, uint64_t r0, uint64_t r1, size_t row_bytes,
                      bool to_stage) {
    auto work = [&](size_t a, size_t b) {
        while (a < b) {
            const uint64_t r = a / row_bytes;
            const size_t off = a - r * row_bytes;
            const size_t len = std::min(b - a, row_bytes - off);
            char *caller = (char *)row(r) + off;
            if (to_stage) memcpy(stage + a, caller, len);
            else memcpy(caller, stage + a, len);
            a += len;
        }
    };
    const size_t a0 = (size_t)r0 * row_bytes, a1 = (size_t)r1 * row_bytes;
    if (a1 - a0 < ((size_t)1 << 20)) {
        work(a0, a1);
        return;
    }
    if (!ctx->copy_pool) {
        const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        ctx->copy_pool.reset(new CopyPool(std::min(kCopyThreads, hw)));
    }
    const unsigned nt = ctx->copy_pool->size();
    const size_t piece = (((a1 - a0) / nt) + 4095) & ~(size_t)4095;
    ctx->copy_pool->run([&](unsigned k, unsigned) {
        const size_t a = a0 + k * piece;
        if (a < a1) work(a, std::min(a1, a + piece));
    });
}

// Host batch: split into chunks of whole transforms and pipeline
// H2D -> transform -> D2H over three streams, so the two copy directions and
// the kernels overlap.  Pinned contiguous buffers are used as they are;
// otherwise (pageable buffers or separate rows, row(r) giving transform r's
// host address) each chunk is copied into pinned staging just before its
// H2D, and out of it once its D2H is done -- two chunks later, while the
// device works on the chunks in between.
template <class InRow, class OutRow>
static int host_pipeline(gbfft_ctx *ctx, uint64_t n, uint64_t batch, int direction, const float *pin_in,
                         float *pin_out, InRow in_row, OutRow out_row) {
    const size_t row_bytes = (size_t)n * sizeof(float2);
    const size_t bytes = row_bytes * batch;
    int st = ctx->dbuf.ensure(bytes, ctx->err);
    if (st == GBFFT_OK) st = ctx->dbuf_out.ensure(bytes, ctx->err);
    if (st != GBFFT_OK) return st;
    float2 *d = (float2 *)ctx->dbuf.ptr;
    float2 *dy = (float2 *)ctx->dbuf_out.ptr;
    const bool staged = !(pin_in && pin_out);
    if (staged) {
        st = ensure_hstage(ctx, bytes);
        if (st != GBFFT_OK) return st;
    }
    char *stage = (char *)ctx->hstage;
    const char *src = staged ? stage : (const char *)pin_in;
    char *dst = staged ? stage : (char *)pin_out;
    uint64_t rows_per_chunk = row_bytes >= ctx->host_chunk ? 1 : ctx->host_chunk / row_bytes;
    if (log2u(n) > kRowsMaxLogN && rows_per_chunk < batch) {
        // plans of three or more passes share the context's workspace: one chunk
        const PlanVariant v = choose_variant(ctx, log2u(n), rows_per_chunk, direction, st);
        Plan *plan = nullptr;
        if (st == GBFFT_OK) st = get_plan(ctx, log2u(n), v, &plan);
        if (st != GBFFT_OK) return st;
        if (plan->passes.size() >= 3) rows_per_chunk = batch;
    }
    std::vector<std::pair<uint64_t, uint64_t>> chunks;
    for (uint64_t r = 0; r < batch; r += rows_per_chunk) chunks.emplace_back(r, std::min(batch, r + rows_per_chunk));
    auto drain = [&](size_t c) -> int {  // chunk c's D2H is done: copy it out
        GB_CUDA(ctx, cudaStreamSynchronize(ctx->xfer[c % 3]));
        if (staged) copy_rows(ctx, stage, out_row, chunks[c].first, chunks[c].second, row_bytes, false);
        return GBFFT_OK;
    };
    for (size_t c = 0; c < chunks.size(); ++c) {
        const uint64_t r0 = chunks[c].first, rows = chunks[c].second - chunks[c].first;
        const size_t off = (size_t)r0 * row_bytes, len = (size_t)rows * row_bytes;
        if (c >= 3) {  // chunk c reuses the stream of chunk c - 3
            st = drain(c - 3);
            if (st != GBFFT_OK) return st;
        }
        if (staged) copy_rows(ctx, stage, in_row, r0, r0 + rows, row_bytes, true);
        cudaStream_t s = ctx->xfer[c % 3];
        GB_CUDA(ctx, cudaMemcpyAsync((char *)d + off, src + off, len, cudaMemcpyHostToDevice, s));
        st = run_device(ctx, (const float2 *)((char *)d + off), (float2 *)((char *)dy + off), n, rows, direction, s,
                        r0);
        if (st != GBFFT_OK) return st;
        GB_CUDA(ctx, cudaMemcpyAsync(dst + off, (char *)dy + off, len, cudaMemcpyDeviceToHost, s));
    }
    for (size_t c = chunks.size() >= 3 ? chunks.size() - 3 : 0; c < chunks.size(); ++c) {
        st = drain(c);
        if (st != GBFFT_OK) return st;
    }
    return check_device_flag(ctx);
}

// Populating means the kernel zeroing every absent page (~5 ms for 128 MB on
// one thread); runs of 8 MB and more are split over the context's copy
// threads (6.3 -> 5.2 ms for 128 MB).  See host_pages.h for when and why.
static void populate_run(gbfft_ctx *ctx, uintptr_t lo, uintptr_t hi) {
    const size_t len = hi - lo;
    if (len < ((size_t)8 << 20)) {
        populate_pages(lo, hi);
        return;
    }
    if (!ctx->copy_pool) {
        const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        ctx->copy_pool.reset(new CopyPool(std::min(kCopyThreads, hw)));
    }
    const uintptr_t page = host_page_size();
    const size_t piece = ((len / ctx->copy_pool->size()) + page - 1) & ~(page - 1);
    ctx->copy_pool->run([&](unsigned k, unsigned) {
        const uintptr_t a = lo + k * piece;
        if (a < hi) populate_pages(a, a + std::min<size_t>(piece, hi - a));
    });
}

// Host batch in pageable memory (contiguous at in_base/out_base, or separate
// rows in_rows[r] / out_rows[r]) moved by the GPU through the host's page
// tables.  Single-pass sizes (FP32): one launch of the transform reads the
// caller's rows and writes the caller's output rows directly.  Larger sizes
// and the split forms: per chunk of whole transforms, one kernel gathers the
// chunk's rows into HBM, the transform runs, one kernel scatters the result
// into the caller's rows; chunks alternate over three streams so one chunk's
// gather, another's transform and a third's scatter overlap.  Nothing runs on
// the host but the launches; the call returns when the results are in place.
// kNotDirect: returned (before any work) when allow_gather is false and the
// shape would need the gather / scatter route, so the caller takes its own.
constexpr int kNotDirect = -1;
// Row batches up to this size pass their row-address table to the kernels in
// pinned host memory instead of uploading it.
constexpr uint64_t kHostTableRows = 64;
static int host_pipeline_direct(gbfft_ctx *ctx, uint64_t n, uint64_t batch, int direction, const char *in_base,
                                char *out_base, const float *const *in_rows, float *const *out_rows,
                                bool allow_gather = true) {
    const size_t row_bytes = (size_t)n * sizeof(float2);
    const size_t bytes = row_bytes * batch;
    const int logn = log2u(n);
    int st = GBFFT_OK;
    // the plan the device entry would run for this shape decides the route
    const PlanVariant v0 = choose_variant(ctx, logn, batch, direction, st);
    Plan *plan = nullptr;
    if (st == GBFFT_OK) st = get_plan(ctx, logn, v0, &plan);
    if (st != GBFFT_OK) return st;
    // single-pass FP32: the transform kernel reads and writes the caller's rows;
    // a fused two-pass plan: its first pass reads them, its second writes them
    const bool single = !ctx->host_gather && !plan->multipass && ctx->precision == GBFFT_PREC_FP32;
    const bool pair = !ctx->host_gather && plan->has_fused && plan->passes.size() == 2 &&
                      batch * plan->fused.groups_per_transform <= 0x7fffffffull;
    if (!allow_gather && !(single && !in_rows) && !pair) return kNotDirect;
    // (allow_gather is false only for pinned batches, whose pages are present)
    if (ctx->prefault && allow_gather && batch > 0)
        prefault_output(out_base, bytes, in_rows ? out_rows : nullptr, batch, row_bytes,
                        [ctx](uintptr_t lo, uintptr_t hi) { populate_run(ctx, lo, hi); });
    if (in_rows && batch == 1 && !pair) {  // one row: its own address is the base, no pointer table
        in_base = (const char *)in_rows[0];
        out_base = (char *)out_rows[0];
        in_rows = nullptr;
    }
    const uint64_t *tin = nullptr, *tout = nullptr;
    uintptr_t align_bits = 0;
    if (in_rows || pair) {  // row addresses as tables the kernels read (the fused pair reads rows through them only)
        const size_t tbytes = 2 * batch * sizeof(uint64_t);
        if (ctx->htable_bytes < tbytes) {
            if (ctx->htable) cudaFreeHost(ctx->htable);
            ctx->htable = nullptr;
            ctx->htable_bytes = 0;
            cudaError_t e = cudaHostAlloc((void **)&ctx->htable, tbytes, cudaHostAllocDefault);
            if (e != cudaSuccess) {
                cudaGetLastError();
                return fail(ctx, GBFFT_ERR_OUT_OF_MEMORY, "pinned row table of %zu bytes: %s", tbytes,
                            cudaGetErrorString(e));
            }
            ctx->htable_bytes = tbytes;
        }
        // A small batch's kernels read the table straight from its pinned
        // host copy (this path runs only where the GPU reaches host memory):
        // no upload to wait for.  Larger batches upload it once, since every
        // CTA would otherwise start with a read across the host link.
        const bool host_table = batch <= kHostTableRows;
        if (!host_table) {
            st = ctx->dtable.ensure(tbytes, ctx->err);
            if (st != GBFFT_OK) return st;
        }
        for (uint64_t r = 0; r < batch; ++r) {
            const uintptr_t a = in_rows ? (uintptr_t)in_rows[r] : (uintptr_t)(in_base + r * row_bytes);
            const uintptr_t b = in_rows ? (uintptr_t)out_rows[r] : (uintptr_t)(out_base + r * row_bytes);
            ctx->htable[r] = (uint64_t)a;
            ctx->htable[batch + r] = (uint64_t)b;
            align_bits |= a | b;
        }
        if (host_table) {
            tin = ctx->htable;
        } else {
            GB_CUDA(ctx,
                    cudaMemcpyAsync(ctx->dtable.ptr, ctx->htable, tbytes, cudaMemcpyHostToDevice, ctx->xfer[0]));
            tin = (const uint64_t *)ctx->dtable.ptr;
        }
        tout = tin + batch;
    } else {
        align_bits = (uintptr_t)in_base | (uintptr_t)out_base;
    }
    if (single && (!tin || plan->rows.fn_tab)) {
        // one launch for the whole batch, no copy through HBM; the plan's own
        // per-row layout, so the same bits as the other paths
        const float *win = nullptr;
        st = window_table(ctx, logn, &win);
        if (st != GBFFT_OK) return st;
        const LoadOps ops{win, ctx->noise_seed, ctx->noise_sigma, 0u};
        GB_CUDA(ctx, rows_launch(plan->rows, (const float2 *)in_base, (float2 *)out_base, batch, plan->tw,
                                 direction, logn, false, ctx->sms, ctx->xfer[0], ops, tin, tout));
        ctx->launches += 1;
        GB_CUDA(ctx, cudaStreamSynchronize(ctx->xfer[0]));
        return check_device_flag(ctx);
    }
    if (pair) {
        // one launch of the fused pair: pass A reads the caller's rows, the
        // intermediate stays in device memory (mostly L2), pass B writes the
        // caller's output rows
        st = ctx->dbuf_out.ensure(bytes, ctx->err);
        if (st != GBFFT_OK) return st;
        const float *win = nullptr;
        st = window_table(ctx, logn, &win);
        if (st != GBFFT_OK) return st;
        const LoadOps ops{win, ctx->noise_seed, ctx->noise_sigma, 0u};
        std::unique_ptr<DeviceBuffer> &cb = ctx->fused_ctr[ctx->xfer[0]];
        if (!cb) cb.reset(new DeviceBuffer());
        ctx->err_armed = true;
        uint64_t launches = 0;
        std::string why;
        st = plan_execute_tables(*plan, tin, tout, (float2 *)ctx->dbuf_out.ptr, batch, direction, ctx->d_err,
                                 ctx->xfer[0], launches, why, ops, cb.get());
        ctx->launches += launches;
        if (st != GBFFT_OK)
            return fail(ctx, st, "execute N=%llu batch=%llu: %s", (unsigned long long)n, (unsigned long long)batch,
                        why.c_str());
        GB_CUDA(ctx, cudaStreamSynchronize(ctx->xfer[0]));
        return check_device_flag(ctx);
    }
    st = ctx->dbuf.ensure(bytes, ctx->err);
    if (st == GBFFT_OK) st = ctx->dbuf_out.ensure(bytes, ctx->err);
    if (st != GBFFT_OK) return st;
    char *d = (char *)ctx->dbuf.ptr;
    char *dy = (char *)ctx->dbuf_out.ptr;
    const bool vec16 = logn >= 1 && (align_bits & 15) == 0;
    uint64_t rows_per_chunk = row_bytes >= ctx->host_chunk ? 1 : ctx->host_chunk / row_bytes;
    if (logn > kRowsMaxLogN && rows_per_chunk < batch) {
        // plans of three or more passes share the context's workspace: one chunk
        const PlanVariant v = choose_variant(ctx, logn, rows_per_chunk, direction, st);
        Plan *plan = nullptr;
        if (st == GBFFT_OK) st = get_plan(ctx, logn, v, &plan);
        if (st != GBFFT_OK) return st;
        if (plan->passes.size() >= 3) rows_per_chunk = batch;
    }
    const size_t nchunks = (batch + rows_per_chunk - 1) / rows_per_chunk;
    if (tin && tin != ctx->htable) {  // the other two streams read the table that xfer[0] uploads
        GB_CUDA(ctx, cudaEventRecord(ctx->ev_table, ctx->xfer[0]));
        GB_CUDA(ctx, cudaStreamWaitEvent(ctx->xfer[1], ctx->ev_table, 0));
        GB_CUDA(ctx, cudaStreamWaitEvent(ctx->xfer[2], ctx->ev_table, 0));
    }
    size_t c = 0;
    for (uint64_t r0 = 0; r0 < batch; r0 += rows_per_chunk, ++c) {
        const uint64_t rows = std::min(batch - r0, rows_per_chunk);
        const size_t off = (size_t)r0 * row_bytes;
        cudaStream_t s = ctx->xfer[c % 3];
        GB_CUDA(ctx, host_rows_copy(tin ? tin + r0 : nullptr, (void *)(in_base ? in_base + off : nullptr), rows, logn,
                                    d + off, true, vec16, ctx->sms, s));
        st = run_device(ctx, (const float2 *)(d + off), (float2 *)(dy + off), n, rows, direction, s, r0);
        if (st != GBFFT_OK) return st;
        GB_CUDA(ctx, host_rows_copy(tout ? tout + r0 : nullptr, (void *)(out_base ? out_base + off : nullptr), rows,
                                    logn, dy + off, false, vec16, ctx->sms, s));
        ctx->launches += 2;
    }
    for (size_t k = 0; k < std::min<size_t>(nchunks, 3); ++k) GB_CUDA(ctx, cudaStreamSynchronize(ctx->xfer[k]));
    return check_device_flag(ctx);
}

}  // namespace

extern "C" {

const char *gbfft_version(void) { return "gbfft 0.1 (sm_103a)"; }

const char *gbfft_status_string(int s) {
    switch (s) {
        case GBFFT_OK: return "ok";
        case GBFFT_ERR_INVALID_SIZE: return kMsgInvalidSize;
        case GBFFT_ERR_LENGTH_MISMATCH: return kMsgLengthMismatch;
        case GBFFT_ERR_INVALID_ARGUMENT: return "invalid argument";
        case GBFFT_ERR_NO_DEVICE: return "no usable sm_103 GPU";
        case GBFFT_ERR_OUT_OF_MEMORY: return "out of memory";
        case GBFFT_ERR_CUDA: return "CUDA error";
        case GBFFT_ERR_TIMEOUT: return "device-side wait timed out";
        case GBFFT_ERR_UNSUPPORTED: return "unsupported size or precision";
        default: return "unknown status";
    }
}

int gbfft_is_available(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    for (int d = 0; d < n; ++d)
        if (device_supported(d)) return 1;
    return 0;
}

int gbfft_create(int device, gbfft_ctx **out_ctx) {
    if (!out_ctx) return GBFFT_ERR_INVALID_ARGUMENT;
    *out_ctx = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
        cudaGetLastError();
        return GBFFT_ERR_NO_DEVICE;
    }
    if (!device_supported(device)) return GBFFT_ERR_NO_DEVICE;
    if (cudaSetDevice(device) != cudaSuccess) return GBFFT_ERR_CUDA;
    std::unique_ptr<gbfft_ctx> ctx(new gbfft_ctx());
    ctx->device = device;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) return GBFFT_ERR_CUDA;
    for (auto &s : ctx->xfer)
        if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return GBFFT_ERR_CUDA;
    if (cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess)
        return GBFFT_ERR_CUDA;
    if (cudaMalloc(&ctx->d_err, sizeof(uint32_t)) != cudaSuccess) return GBFFT_ERR_OUT_OF_MEMORY;
    if (cudaMemset(ctx->d_err, 0, sizeof(uint32_t)) != cudaSuccess) return GBFFT_ERR_CUDA;
    if (const char *c = getenv("GBFFT_PRECISION")) {  // default precision of new contexts
        if (!strcmp(c, "tc_fp16")) ctx->precision = GBFFT_PREC_TC_FP16;
        else if (!strcmp(c, "tc_bf16x3")) ctx->precision = GBFFT_PREC_TC_BF16X3;
        else if (!strcmp(c, "tc_tf32")) ctx->precision = GBFFT_PREC_TC_TF32;
        else if (!strcmp(c, "tc_bf16x6")) ctx->precision = GBFFT_PREC_TC_BF16X6;
    }
    if (const char *c = getenv("GBFFT_HOST_CHUNK_BYTES")) {
        const long long v = atoll(c);
        if (v >= (1 << 16)) ctx->host_chunk = (size_t)v;
    }
    if (const char *c = getenv("GBFFT_AUTOTUNE_CACHE")) {
        ctx->tune_cache = c;
        load_tune_cache(ctx.get());
    }
    if (cudaEventCreateWithFlags(&ctx->ev_table, cudaEventDisableTiming) != cudaSuccess) return GBFFT_ERR_CUDA;
    cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device);
    int pageable = 0;
    if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device) != cudaSuccess) {
        cudaGetLastError();
        pageable = 0;
    }
    const char *hp = getenv("GBFFT_HOST_PATH");
    ctx->host_direct = pageable == 1 && !(hp && !strcmp(hp, "staged"));
    ctx->host_gather = hp && !strcmp(hp, "gather");
    if (const char *pf = getenv("GBFFT_PREFAULT")) ctx->prefault = pf[0] != '0';
    if (const char *a = getenv("GBFFT_AUTOTUNE")) ctx->auto_tune = a[0] == '1';
    if (const char *a = getenv("GBFFT_AUTOTUNE_VERBOSE")) ctx->tune_verbose = a[0] == '1';
    *out_ctx = ctx.release();
    return GBFFT_OK;
}

void gbfft_destroy(gbfft_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (auto &s : ctx->xfer)
        if (s) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    ctx->plans.clear();
    ctx->dbuf.release();
    ctx->dbuf_out.release();
    ctx->ws.release();
    if (ctx->d_err) cudaFree(ctx->d_err);
    if (ctx->hstage) cudaFreeHost(ctx->hstage);
    if (ctx->htable) cudaFreeHost(ctx->htable);
    ctx->dtable.release();
    if (ctx->ev_table) cudaEventDestroy(ctx->ev_table);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char *gbfft_last_error(const gbfft_ctx *ctx) { return ctx ? ctx->err.c_str() : ""; }

uint64_t gbfft_launch_count(const gbfft_ctx *ctx) { return ctx ? ctx->launches : 0; }

int gbfft_autotune(gbfft_ctx *ctx, uint64_t n, uint64_t batch, int direction, double *best_seconds) {
    int st = validate_common(ctx, n, direction);
    if (st != GBFFT_OK) return st;
    if (batch == 0) return fail(ctx, GBFFT_ERR_INVALID_ARGUMENT, "batch must be positive");
    GB_CUDA(ctx, cudaSetDevice(ctx->device));
    return autotune(ctx, n, batch, direction, best_seconds);
}

int gbfft_set_window(gbfft_ctx *ctx, int window) {
    if (!ctx) return GBFFT_ERR_INVALID_ARGUMENT;
    if (window != GBFFT_WINDOW_NONE && window != GBFFT_WINDOW_HANN)
        return fail(ctx, GBFFT_ERR_INVALID_ARGUMENT, "window %d is not provided", window);
    ctx->window = window;
    return GBFFT_OK;
}

int gbfft_set_noise(gbfft_ctx *ctx, uint32_t seed, float sigma) {
    if (!ctx) return GBFFT_ERR_INVALID_ARGUMENT;
    if (!(sigma >= 0.f) || sigma == INFINITY)
        return fail(ctx, GBFFT_ERR_INVALID_ARGUMENT, "noise sigma must be finite and >= 0");
    ctx->noise_seed = seed;
    ctx->noise_sigma = sigma;
    return GBFFT_OK;
}

int gbfft_set_precision(gbfft_ctx *ctx, int precision) {
    if (!ctx) return GBFFT_ERR_INVALID_ARGUMENT;
    if (precision != GBFFT_PREC_FP32 && precision != GBFFT_PREC_TC_FP16 && precision != GBFFT_PREC_TC_BF16X3 &&
        precision != GBFFT_PREC_TC_TF32 && precision != GBFFT_PREC_TC_BF16X6)
        return fail(ctx, GBFFT_ERR_INVALID_ARGUMENT, "precision %d is not a gbfft_precision", precision);
    ctx->precision = precision;
    return GBFFT_OK;
}

int gbfft_c2c_device(gbfft_ctx *ctx, const void *d_in, void *d_out, uint64_t n, uint64_t batch, int direction,
                     void *stream) {
    int st = validate_common(ctx, n, direction);
    if (st != GBFFT_OK) return st;
    if (batch == 0) return GBFFT_OK;
    if (!d_in || !d_out) return fail(ctx, GBFFT_ERR_INVALID_ARGUMENT, "null device pointer");
    GB_CUDA(ctx, cudaSetDevice(ctx->device));
    return run_device(ctx, (const float2 *)d_in, (float2 *)d_out, n, batch, direction, (cudaStream_t)stream);
}

// Host batch already contiguous in `in` (pinned or pageable).
static int host_contiguous(gbfft_ctx *ctx, const float *in, float *out, uint64_t n, uint64_t batch,
                           int direction) {
    const size_t row_bytes = (size_t)n * sizeof(float2);
    const bool pinned = host_is_pinned(in) && host_is_pinned(out);
    if (ctx->host_direct) {
        // pinned batches too go straight through the transform kernels where
        // those read and write host memory themselves; otherwise the copy
        // engines move them (faster than copy kernels for pinned memory)
        const int st = host_pipeline_direct(ctx, n, batch, direction, (const char *)in, (char *)out, nullptr,
                                            nullptr, !pinned);
        if (st != kNotDirect) return st;
    }
    auto in_row = [&](uint64_t r) { return (const char *)in + r * row_bytes; };
    auto out_row = [&](uint64_t r) { return (char *)out + r * row_bytes; };
    return host_pipeline(ctx, n, batch, direction, pinned ? in : nullptr, pinned ? out : nullptr, in_row, out_row);
}

int gbfft_c2c_host(gbfft_ctx *ctx, const float *in, float *out, uint64_t n, uint64_t batch, int direction) {
    if (!ctx) return GBFFT_ERR_INVALID_ARGUMENT;
    if (batch == 0) return GBFFT_OK;  // src/lib.rs:522-524
    int st = validate_common(ctx, n, direction);
    if (st != GBFFT_OK) return st;
    if (!in || !out) return fail(ctx, GBFFT_ERR_INVALID_ARGUMENT, "null host pointer");
    GB_CUDA(ctx, cudaSetDevice(ctx->device));
    return host_contiguous(ctx, in, out, n, batch, direction);
}

int gbfft_c2c_host_rows(gbfft_ctx *ctx, const float *const *in_rows, const uint64_t *row_lengths,
                        float *const *out_rows, uint64_t batch, int direction) {
    if (!ctx) return GBFFT_ERR_INVALID_ARGUMENT;
    if (batch == 0) return GBFFT_OK;  // src/lib.rs:522-524
    if (!in_rows || !row_lengths || !out_rows)
        return fail(ctx, GBFFT_ERR_INVALID_ARGUMENT, "null row array");
    // src/lib.rs:526-533: equal lengths, then power of two, row by row.
    const uint64_t n = row_lengths[0];
    for (uint64_t i = 0; i < batch; ++i) {
        if (row_lengths[i] != n) return fail(ctx, GBFFT_ERR_LENGTH_MISMATCH, "%s", kMsgLengthMismatch);
        if (!is_pow2(row_lengths[i])) return fail(ctx, GBFFT_ERR_INVALID_SIZE, "%s", kMsgInvalidSize);
    }
    int st = validate_common(ctx, n, direction);
    if (st != GBFFT_OK) return st;
    for (uint64_t i = 0; i < batch; ++i)
        if (!in_rows[i] || !out_rows[i]) return fail(ctx, GBFFT_ERR_INVALID_ARGUMENT, "null row pointer");
    GB_CUDA(ctx, cudaSetDevice(ctx->device));
    if (ctx->host_direct) return host_pipeline_direct(ctx, n, batch, direction, nullptr, nullptr, in_rows, out_rows);
    auto in_row = [&](uint64_t r) { return (const char *)in_rows[r]; };
    auto out_row = [&](uint64_t r) { return (char *)out_rows[r]; };
    return host_pipeline(ctx, n, batch, direction, nullptr, nullptr, in_row, out_row);
}

int gbfft_ragged_plan_create(gbfft_ctx *ctx, const gbfft_ragged_desc *descs, uint32_t count,
                             gbfft_ragged_plan **out_plan) {
    if (!ctx) return GBFFT_ERR_INVALID_ARGUMENT;
    if (!out_plan || (count > 0 && !descs)) return fail(ctx, GBFFT_ERR_INVALID_ARGUMENT, "null argument");
    *out_plan = nullptr;
    GB_CUDA(ctx, cudaSetDevice(ctx->device));
    RaggedPlanImpl *impl = nullptr;
    std::string why;
    int st = ragged_plan_build(impl, ctx->device, descs, count, ctx->precision, why);
    if (st != GBFFT_OK) return fail(ctx, st, "%s", why.c_str());
    *out_plan = new gbfft_ragged_plan{ctx, impl};
    return GBFFT_OK;
}

int gbfft_ragged_plan_set(gbfft_ragged_plan *plan, int option, uint64_t value) {
    if (!plan) return GBFFT_ERR_INVALID_ARGUMENT;
    std::string why;
    int st = ragged_plan_set(*plan->impl, option, value, why);
    return st == GBFFT_OK ? st : fail(plan->ctx, st, "%s", why.c_str());
}

int gbfft_ragged_execute(gbfft_ragged_plan *plan, const void *d_in, void *d_out, uint64_t capacity, int use_graph,
                         void *stream) {
    if (!plan) return GBFFT_ERR_INVALID_ARGUMENT;
    gbfft_ctx *ctx = plan->ctx;
    if (ragged_plan_items(*plan->impl) > 0 && (!d_in || !d_out))
        return fail(ctx, GBFFT_ERR_INVALID_ARGUMENT, "null device pointer");
    if (ragged_plan_extent(*plan->impl) > capacity)
        return fail(ctx, GBFFT_ERR_INVALID_ARGUMENT, "descriptors reach sample %llu, past the buffer capacity %llu",
                    (unsigned long long)ragged_plan_extent(*plan->impl), (unsigned long long)capacity);
    GB_CUDA(ctx, cudaSetDevice(ctx->device));
    std::string why;
    const uint64_t before = ragged_plan_launches(*plan->impl);
    int st = ragged_plan_execute(*plan->impl, d_in, d_out, (cudaStream_t)stream, use_graph != 0, why);
    ctx->launches += ragged_plan_launches(*plan->impl) - before;
    return st == GBFFT_OK ? st : fail(ctx, st, "ragged execute: %s", why.c_str());
}

int gbfft_ragged_wait(gbfft_ragged_plan *plan, void *stream) {
    if (!plan) return GBFFT_ERR_INVALID_ARGUMENT;
    GB_CUDA(plan->ctx, cudaSetDevice(plan->ctx->device));
    std::string why;
    int st = ragged_plan_wait(*plan->impl, (cudaStream_t)stream, why);
    return st == GBFFT_OK ? st : fail(plan->ctx, st, "%s", why.c_str());
}

uint64_t gbfft_ragged_launch_count(const gbfft_ragged_plan *plan) {
    return plan ? ragged_plan_launches(*plan->impl) : 0;
}

void gbfft_ragged_plan_destroy(gbfft_ragged_plan *plan) {
    if (!plan) return;
    cudaSetDevice(plan->ctx->device);
    ragged_plan_free(plan->impl);
    delete plan;
}

int gbfft_ragged_device(gbfft_ctx *ctx, const void *d_in, void *d_out, uint64_t capacity,
                        const gbfft_ragged_desc *descs, uint32_t count, void *stream) {
    gbfft_ragged_plan *plan = nullptr;
    int st = gbfft_ragged_plan_create(ctx, descs, count, &plan);
    if (st != GBFFT_OK) return st;
    st = gbfft_ragged_execute(plan, d_in, d_out, capacity, 0, stream);
    if (st == GBFFT_OK) st = gbfft_ragged_wait(plan, stream);
    gbfft_ragged_plan_destroy(plan);
    return st;
}

int gbfft_bench_device(gbfft_ctx *ctx, uint64_t n, uint64_t batch, int direction, int warmup, int iters,
                       double *seconds_per_iter) {
    int st = validate_common(ctx, n, direction);
    if (st != GBFFT_OK) return st;
    if (!seconds_per_iter || iters <= 0 || warmup < 0 || batch == 0)
        return fail(ctx, GBFFT_ERR_INVALID_ARGUMENT, "bad benchmark arguments");
    GB_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t bytes = (size_t)n * batch * sizeof(float2);
    st = ctx->dbuf.ensure(bytes, ctx->err);
    if (st != GBFFT_OK) return st;
    float2 *d = (float2 *)ctx->dbuf.ptr;
    GB_CUDA(ctx, cudaMemsetAsync(d, 0, bytes, ctx->stream));
    for (int i = 0; i < warmup; ++i) {
        st = run_device(ctx, d, d, n, batch, direction, ctx->stream);
        if (st != GBFFT_OK) return st;
    }
    GB_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
    for (int i = 0; i < iters; ++i) {
        st = run_device(ctx, d, d, n, batch, direction, ctx->stream);
        if (st != GBFFT_OK) return st;
    }
    GB_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
    GB_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
    st = check_device_flag(ctx);
    if (st != GBFFT_OK) return st;
    float ms = 0.f;
    GB_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    *seconds_per_iter = (double)ms * 1e-3 / iters;
    return GBFFT_OK;
}

}  // extern "C"
