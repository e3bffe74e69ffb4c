// Plan = everything size-specific the transform needs, built once per log2 N
// and cached by the context.  Replaces the reference's SizeCache
// (larsjoost/wgls-rs-fft src/lib.rs:230-259, 709-943): instead of wgpu buffers,
// bind groups and per-stage uniforms it holds device twiddle tables and the
// kernel schedule (single pass, or a list of global passes for N > 2^14).
#pragma once
#include <string>
#include <vector>

#include "gbfft_internal.h"

namespace gbfft {

struct DeviceBuffer {
    void *ptr = nullptr;
    size_t bytes = 0;
    int ensure(size_t want, std::string &err);
    void release();
    ~DeviceBuffer() { release(); }
};

// One global Stockham pass of the multi-pass form (fft_passes.cu).
struct PassDesc {
    const void *fn = nullptr;
    const void *fn_persistent = nullptr;  // tile loop with L2 prefetch of the next tile (FP32 form)
    int persist_ctas_per_sm = 0;
    int logr = 0;        // transform size handled in shared memory: R = 2^logr
    int logp = 0;        // product of the radices of earlier global passes
    int cols = 0;        // columns (independent length-R DFTs) per CTA
    int threads = 0;
    size_t smem = 0;
    uint64_t sub_tw_offset = 0;         // where this pass's sub-pass tables start
    TwiddleSegment segs[kMaxSub] = {};  // its in-SMEM sub-pass tables, offsets from 0
    int nseg = 0;
    int tw_entries = 0;
    bool tc = false;                    // radix-16 butterflies on the tensor cores
    const void *fn_tma = nullptr;       // first pass with its input tile brought in by the TMA
    const void *fn_tma_persistent = nullptr;  // the same as a tile loop prefetching the next tile into L2
    int tma_ctas_per_sm = 0;
    size_t smem_tma = 0;
};

// Two consecutive passes in one persistent launch whose queue alternates the
// first pass's tiles of group x with the second pass's tiles of group x - LAG,
// so that the intermediate is read back from L2 (fft_fused.cuh): both passes
// of a two-pass transform, or the last two of a three-pass one.
struct FusedDesc {
    const void *fn = nullptr;
    int threads = 0;
    size_t smem = 0;
    int logra = 0, logrb = 0;  // radices of the two passes
    int logpa = 0;             // product of the radices before them (0: the pair starts the transform)
    int logn = 0;
    uint32_t groups_per_transform = 1;
    uint32_t tiles_per_group = 0;  // of each pass
    uint64_t group_samples = 0;
    int ctas_per_sm = 0;
    int tmem_cols = 0;  // split forms: TMEM columns a CTA holds (bounds the CTAs per SM)
    int loge = 4;       // log2 of the samples a thread holds
    // 32 samples a thread: the pair's own sub-pass tables (offsets into the
    // plan's twiddle table; -1: the passes' tables are used)
    int64_t sub_off_a = -1, sub_off_b = -1;
};
// Upper bound on the intermediates in flight between the two passes (bytes).
constexpr uint64_t kFusedWindowBytes = 48ull << 20;

// The tunable choices of a plan: largest global-pass radix (multi-pass split),
// whether kernels run as persistent tile loops with L2 prefetch, whether pass
// pairs run as one launch with an L2-resident intermediate, and (single pass)
// how many transforms a CTA takes.
struct PlanVariant {
    int max_logr = 10;
    bool persistent = false;
    bool fused = false;
    int tile = 0;  // single pass: log2 of the samples a CTA moves (0: 2^12), i.e. transforms per CTA;
                   // three passes: log2 of the columns a first-pass CTA takes (0: 16)
    int loge = 4;  // single pass: log2 of the samples a thread holds (5: radix-32 sub-passes, N = 2^13, 2^14)
    bool tma = false;  // three passes, 8-column first pass: input tile brought in by the TMA
    bool operator<(const PlanVariant &o) const {
        if (max_logr != o.max_logr) return max_logr < o.max_logr;
        if (persistent != o.persistent) return persistent < o.persistent;
        if (fused != o.fused) return fused < o.fused;
        if (tile != o.tile) return tile < o.tile;
        if (loge != o.loge) return loge < o.loge;
        return tma < o.tma;
    }
    bool operator==(const PlanVariant &o) const {
        return max_logr == o.max_logr && persistent == o.persistent && fused == o.fused && tile == o.tile &&
               loge == o.loge && tma == o.tma;
    }
};

struct Plan {
    int logn = 0;
    PlanVariant variant;
    int sms = 0;
    int precision = GBFFT_PREC_FP32;
    void *gtab = nullptr;  // tensor-core forms: the 32 x 32 DFT operand parts
    bool multipass = false;
    bool needs_workspace = false;
    RowsKernelInfo rows;
    std::vector<PassDesc> passes;
    bool has_fused = false;  // variant.fused and a kernel exists for the split
    FusedDesc fused;
    // twiddle table (device): rows sub-pass tables, or for multi-pass the
    // per-pass sub-pass tables followed by the two-level W_N table.
    float2 *tw = nullptr;
    uint64_t tw_entries = 0;
    uint64_t tw_lo_offset = 0, tw_hi_offset = 0;  // W_N^i (i < 2^s), W_N^{i 2^s}
    int tw_split = 0;                             // s
    ~Plan();
};

// fft_passes.cu
// loge 5: 32 samples a thread, for the first pass of radix 2^9 / 2^10 only
bool pass_kernel_info(int logr, bool first, PassDesc &d, int loge = 4, int cols_log = 4, bool tma = false);
cudaError_t pass_prepare(PassDesc &d);
cudaError_t pass_launch(const PassDesc &d, const float2 *in, float2 *out, uint64_t batch, int logn,
                        const float2 *tw_sub, const float2 *tw_lo, const float2 *tw_hi, int tw_split,
                        float in_im_sign, float out_re_scale, float out_im_scale, cudaStream_t stream,
                        bool persistent = false, int sms = 0, LoadOps ops = LoadOps{nullptr, 0u, 0.f, 0u},
                        uint32_t *err = nullptr);

// fft_passes_tc.cu (split-precision tensor-core form)
bool pass_tc_kernel_info(int logr, bool first, int precision, PassDesc &d);
// both passes of a two-pass transform in one persistent launch (radices 2^8/2^7 .. 2^9/2^9)
// loge 5: 32-sample tiles with radix-32 tensor-core sub-DFTs (16-bit kinds)
bool fused_tc_kernel_info(int logr1, int logr2, int precision, FusedDesc &d, int loge = 4);
cudaError_t pass_tc_launch(const PassDesc &d, const float2 *in, float2 *out, uint64_t batch, int logn,
                           const float2 *tw_sub, const float2 *tw_lo, const float2 *tw_hi, int tw_split,
                           float in_im_sign, float out_re_scale, float out_im_scale, const void *gtab,
                           uint32_t *err, cudaStream_t stream, LoadOps ops = LoadOps{nullptr, 0u, 0.f, 0u});
cudaError_t tc_gtab_fill(void *out, cudaStream_t stream);

// fft_rows_tc.cu (split form of the single-pass transform, N = 2^4 .. 2^14; TF32 up to 2^13)
bool rows_tc_kernel_info(int logn, int precision, RowsKernelInfo &k);
cudaError_t rows_tc_prepare(RowsKernelInfo &k);
cudaError_t rows_tc_launch(const RowsKernelInfo &k, const float2 *in, float2 *out, uint64_t batch,
                           const float2 *tw, int direction, int logn, const void *gtab, uint32_t *err,
                           cudaStream_t stream, LoadOps ops);
// G table: radix 16: [FP16 hi | FP16 lo | BF16 hi | BF16 lo] (2 KB each), [TF32 hi | TF32 lo]
// (4 KB each); radix 32: [FP16 hi | FP16 lo | BF16 hi | BF16 lo] (8 KB each)
constexpr size_t kTcGtabBytes = 4 * 2048 + 2 * 4096 + 4 * 8192 + 3 * 2048;  // ... + BF16 x 6 parts

// fft_fused2.cu, fft_fused3.cu
// loge 5: tiles of 32 samples a thread (radix-32 sub-passes), pairs with a radix-2^9/2^10 pass
bool fused2_kernel_info(int logr1, int logr2, FusedDesc &d, int loge = 4);
// Sub-pass table segments of a radix-2^logr pass tile with 2^loge samples a
// thread, offsets from `base`; sets `entries`.  Returns the segment count.
int pass_sub_segments(int logr, int loge, TwiddleSegment *out, uint64_t base, int &entries);
bool fused3_kernel_info(int logn, FusedDesc &d);  // passes 2-3 of (logn - 16, 8, 8)
cudaError_t fused_prepare(FusedDesc &d);
uint32_t fused_lag(const FusedDesc &d, uint64_t ngroups, int sms);
cudaError_t fused_launch(const FusedDesc &d, const float2 *in, float2 *out, uint64_t batch, const float2 *tw_a,
                         const float2 *tw_b, const float2 *tw_lo, const float2 *tw_hi, float in_im, float out_re,
                         float out_im, LoadOps ops, uint32_t *ctr, uint32_t *err, int sms, cudaStream_t stream,
                         const void *gtab = nullptr, const uint64_t *tab_in = nullptr,
                         const uint64_t *tab_out = nullptr);

// log2 radices (each <= max_logr) of the global passes for a multi-pass
// transform of 2^logn.
std::vector<int> split_passes(int logn, int max_logr = 10);

// Append the twiddle segments of a multi-pass schedule (per-pass sub-pass
// tables, then the two-level W_N table) starting at `offset`; fills the pass
// descriptors' table offsets and the plan-level two-level table fields.
// Returns the offset one past the last entry.
uint64_t multipass_segments(int logn, std::vector<PassDesc> &passes, uint64_t offset,
                            std::vector<TwiddleSegment> &segs, uint64_t &lo_off, uint64_t &hi_off, int &split);

// Candidate variants the tuner tries for a size and precision, the first being
// the default used before any tuning.
std::vector<PlanVariant> plan_candidates(int logn, int precision);

int plan_build(Plan &p, int logn, int precision, const PlanVariant &v, cudaStream_t stream, std::string &why);
// `err` is a device flag the tensor-core and fused kernels raise when a bounded
// wait gives up.  `ops`: noise / window applied to every loaded input sample.
// `ctr`: counter block of the fused two-pass form (grown and zeroed here; the
// kernel leaves it zeroed); without it, or in place, the form falls back to
// two launches.
int plan_execute(const Plan &p, const float2 *in, float2 *out, uint64_t batch, int direction,
                 DeviceBuffer &ws, uint32_t *err, cudaStream_t stream, uint64_t &launches, std::string &why,
                 LoadOps ops = LoadOps{nullptr, 0u, 0.f, 0u}, DeviceBuffer *ctr = nullptr);

// A two-pass fused plan (has_fused, two passes) over the caller's rows: pass
// A reads transform b from tab_in[b] and pass B writes it to tab_out[b]
// (device arrays of row addresses the GPU reaches through the host's page
// tables); `work` (batch << logn samples of device memory) holds the
// intermediate.  One launch.
int plan_execute_tables(const Plan &p, const uint64_t *tab_in, const uint64_t *tab_out, float2 *work,
                        uint64_t batch, int direction, uint32_t *err, cudaStream_t stream, uint64_t &launches,
                        std::string &why, LoadOps ops, DeviceBuffer *ctr);

}  // namespace gbfft
