// Internal interfaces between the C ABI (gbfft_api.cu) and the kernel files.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/gbfft.h"
#include "fft_core.cuh"

namespace gbfft {

constexpr int kMaxLogN = 30;          // largest supported transform: 2^30 samples
constexpr int kRowsMaxLogN = 14;      // single-pass (in shared memory) limit
constexpr int kMaxSub = 16;

// ---- twiddle generation (twiddle.cu) -------------------------------------
// A segment fills `count` complex entries at `offset` of a table with
// W_M^{e(i)} = exp(-2 pi i e(i) / M), M = 2^logm, computed in FP64 and
// rounded to FP32.
//   kind 0 (sub-pass table): i = (m-1)*P + k, e = m*k, P = 2^logp
//   kind 1 (linear table):   e = i << logstride
struct TwiddleSegment {
    uint64_t offset;
    uint64_t count;
    int kind;
    int logm;
    int logp;
    int logstride;
};
cudaError_t twiddle_fill(float2 *table, const TwiddleSegment *segs, int nseg, cudaStream_t stream);
// Hann window table of n floats (FP64-computed).
cudaError_t hann_fill(float *w, uint64_t n, cudaStream_t stream);
constexpr int kWindowMaxLogN = 24;

// ---- single-pass kernel (fft_rows.cu) ------------------------------------
struct RowsKernelInfo {
    const void *fn = nullptr;             // forward
    const void *fn_persistent = nullptr;  // forward, tile loop with L2 prefetch of the next tile
    const void *fn_inv = nullptr;         // the same two for the inverse
    const void *fn_persistent_inv = nullptr;
    const void *fn_tab = nullptr;         // forward / inverse over per-row address tables
    const void *fn_tab_inv = nullptr;
    int persist_ctas_per_sm = 0;          // resident CTAs of fn_persistent (set by rows_prepare)
    int threads = 0;
    int transforms_per_cta = 0;
    size_t smem = 0;
    TwiddleSegment segs[kMaxSub] = {};  // sub-pass tables, offsets from 0
    int nseg = 0;
    int tw_entries = 0;
};
// logs: log2 of the samples a CTA moves (12; 11 or 13 for N = 2^6 .. 2^11);
// loge: log2 of the samples a thread holds (4; 5 for N = 2^13, 2^14)
bool rows_kernel_info(int logn, RowsKernelInfo &k, int logs = 12, int loge = 4);
cudaError_t rows_prepare(RowsKernelInfo &k);
// Sets fn_tab / fn_tab_inv for the tile (null where no table form is built).
void rows_tab_describe(int logn, int logs, int loge, RowsKernelInfo &k);
// persistent: use fn_persistent with at most persist_ctas_per_sm * sms CTAs.
// tab_in / tab_out: arrays of per-row addresses the device can read (row r
// read from tab_in[r], written to tab_out[r]; in / out ignored); never
// persistent.
cudaError_t rows_launch(const RowsKernelInfo &k, const float2 *in, float2 *out, uint64_t batch,
                        const float2 *tw, int direction, int logn, bool persistent, int sms, cudaStream_t stream,
                        LoadOps ops = LoadOps{nullptr, 0u, 0.f, 0u}, const uint64_t *tab_in = nullptr,
                        const uint64_t *tab_out = nullptr);

// ---- host rows <-> device batch, copied by the GPU (host_rows.cu) ---------
// Moves `rows` rows of 2^logn complex<f32> between caller host memory, reached
// through the host's page tables, and `dev` (the rows back to back).  Row r's
// host address is table[r] (a device array) or, with table == nullptr,
// base + r * 2^logn samples.  vec16: every host row address is 16-byte aligned
// and logn >= 1.  Needs cudaDevAttrPageableMemoryAccess.
cudaError_t host_rows_copy(const uint64_t *table, void *base, uint64_t rows, int logn, void *dev, bool to_device,
                           bool vec16, int sms, cudaStream_t stream);

}  // namespace gbfft
