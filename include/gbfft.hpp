// C++ mirror of larsjoost/wgls-rs-fft's executor interface over the C ABI in
// gbfft.h -- header-only, no CUDA headers needed.
//
//   trait FftExecutor { name, fft, ifft, as_any }        src/lib.rs:32-45
//   GpuFft::new / fft / ifft / is_gpu_available / Default src/lib.rs:285-489, 946-950
//
// Batches are std::vector<std::vector<std::complex<float>>> (the reference's
// &[Vec<Complex<f32>>]); failures throw gbfft::Error carrying the status and
// the library's message -- including the reference's own two messages for a
// non-power-of-two length and for rows of different lengths.  An empty batch
// returns an empty batch.
#pragma once
#include <complex>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "gbfft.h"

namespace gbfft {

using Complex = std::complex<float>;
using Batch = std::vector<std::vector<Complex>>;

class Error : public std::runtime_error {
   public:
    Error(int status, const std::string &msg) : std::runtime_error(msg), status_(status) {}
    int status() const { return status_; }

   private:
    int status_;
};

class FftExecutor {
   public:
    virtual ~FftExecutor() = default;
    virtual std::string name() const = 0;
    virtual Batch fft(const Batch &inputs) = 0;
    virtual Batch ifft(const Batch &inputs) = 0;
};

class GpuFft : public FftExecutor {
   public:
    // GpuFft::new (src/lib.rs:285-330): throws when no usable GB300 exists.
    explicit GpuFft(int device = 0) {
        const int st = gbfft_create(device, &ctx_);
        if (st != GBFFT_OK) throw Error(st, gbfft_status_string(st));
    }
    ~GpuFft() override { gbfft_destroy(ctx_); }
    GpuFft(const GpuFft &) = delete;
    GpuFft &operator=(const GpuFft &) = delete;
    GpuFft(GpuFft &&o) noexcept : ctx_(std::exchange(o.ctx_, nullptr)) {}
    GpuFft &operator=(GpuFft &&o) noexcept {
        if (this != &o) {
            gbfft_destroy(ctx_);
            ctx_ = std::exchange(o.ctx_, nullptr);
        }
        return *this;
    }

    // GpuFft::is_gpu_available (src/lib.rs:381-389)
    static bool is_gpu_available() { return gbfft_is_available() != 0; }

    std::string name() const override { return "GB300 (sm_103a Stockham radix-16)"; }

    // GpuFft::fft (src/lib.rs:433-438): forward, unscaled.
    Batch fft(const Batch &inputs) override { return run(inputs, GBFFT_FORWARD); }
    // GpuFft::ifft (src/lib.rs:483-488): inverse scaled by 1/N.
    Batch ifft(const Batch &inputs) override { return run(inputs, GBFFT_INVERSE); }

    // fft / ifft into caller-kept output rows of the inputs' lengths (no
    // reference counterpart): reused rows stay resident, so the GPU writes
    // them at the host link's rate.
    void transform_into(const Batch &inputs, Batch &outputs, bool inverse = false) {
        bool same = outputs.size() == inputs.size();
        for (size_t i = 0; same && i < inputs.size(); ++i) same = outputs[i].size() == inputs[i].size();
        if (!same) throw Error(GBFFT_ERR_INVALID_ARGUMENT, "output rows must have the input rows' lengths");
        if (inputs.empty()) return;
        const size_t b = inputs.size();
        std::vector<const float *> in(b);
        std::vector<uint64_t> len(b);
        std::vector<float *> outp(b);
        for (size_t i = 0; i < b; ++i) {
            in[i] = reinterpret_cast<const float *>(inputs[i].data());
            len[i] = inputs[i].size();
            outp[i] = reinterpret_cast<float *>(outputs[i].data());
        }
        check(gbfft_c2c_host_rows(ctx_, in.data(), len.data(), outp.data(), b, inverse ? GBFFT_INVERSE : GBFFT_FORWARD));
    }

    // Device-resident transform (no reference counterpart): interleaved
    // complex<float> device buffers, enqueued on `stream` (a cudaStream_t).
    void fft_device(const void *d_in, void *d_out, uint64_t n, uint64_t batch, int direction,
                    void *stream = nullptr) {
        check(gbfft_c2c_device(ctx_, d_in, d_out, n, batch, direction, stream));
    }

    // GpuFftTrait::benchmark_gpu_only (src/lib.rs:673-707): seconds per transform.
    double benchmark_gpu_only(uint64_t n, uint64_t batch, int warmup, int iters) {
        double s = 0.0;
        check(gbfft_bench_device(ctx_, n, batch, GBFFT_FORWARD, warmup, iters, &s));
        return s;
    }

    void set_precision(int precision) { check(gbfft_set_precision(ctx_, precision)); }
    // Hann window (GBFFT_WINDOW_HANN) or none applied to every loaded sample.
    void set_window(int window) { check(gbfft_set_window(ctx_, window)); }
    // The reference pipeline's noise added to every loaded sample (sigma 0: off).
    void set_noise(uint32_t seed, float sigma) { check(gbfft_set_noise(ctx_, seed, sigma)); }
    // Times every plan variant for a shape and keeps the fastest; seconds per transform.
    double autotune(uint64_t n, uint64_t batch, int direction = GBFFT_FORWARD) {
        double s = 0.0;
        check(gbfft_autotune(ctx_, n, batch, direction, &s));
        return s;
    }
    gbfft_ctx *context() { return ctx_; }

   private:
    void check(int st) {
        if (st != GBFFT_OK) {
            const char *m = gbfft_last_error(ctx_);
            throw Error(st, (m && *m) ? m : gbfft_status_string(st));
        }
    }

    Batch run(const Batch &inputs, int direction) {
        if (inputs.empty()) return {};  // src/lib.rs:522-524
        const size_t b = inputs.size();
        std::vector<const float *> in(b);
        std::vector<uint64_t> len(b);
        Batch out(b);
        std::vector<float *> outp(b);
        for (size_t i = 0; i < b; ++i) {
            in[i] = reinterpret_cast<const float *>(inputs[i].data());
            len[i] = inputs[i].size();
            out[i].resize(inputs[i].size());
            outp[i] = reinterpret_cast<float *>(out[i].data());
        }
        check(gbfft_c2c_host_rows(ctx_, in.data(), len.data(), outp.data(), b, direction));
        return out;
    }

    gbfft_ctx *ctx_ = nullptr;
};

// Ragged batch (no reference counterpart): mixed sizes and directions in one
// persistent launch over device buffers.
class RaggedPlan {
   public:
    RaggedPlan(GpuFft &fft, const std::vector<gbfft_ragged_desc> &descs) : ctx_(fft.context()) {
        const int st = gbfft_ragged_plan_create(ctx_, descs.data(), (uint32_t)descs.size(), &plan_);
        if (st != GBFFT_OK) throw Error(st, gbfft_last_error(ctx_));
    }
    ~RaggedPlan() { gbfft_ragged_plan_destroy(plan_); }
    RaggedPlan(const RaggedPlan &) = delete;
    RaggedPlan &operator=(const RaggedPlan &) = delete;
    void execute(const void *d_in, void *d_out, uint64_t capacity, bool use_graph = true, void *stream = nullptr) {
        check(gbfft_ragged_execute(plan_, d_in, d_out, capacity, use_graph ? 1 : 0, stream));
    }
    void wait(void *stream = nullptr) { check(gbfft_ragged_wait(plan_, stream)); }

   private:
    void check(int st) {
        if (st != GBFFT_OK) throw Error(st, gbfft_last_error(ctx_));
    }
    gbfft_ctx *ctx_ = nullptr;
    gbfft_ragged_plan *plan_ = nullptr;
};

}  // namespace gbfft
