// Single-pass tile configuration and kernel (shared by fft_rows.cu and
// fft_rows_tab.cu, which instantiates the table-addressed form).
#pragma once
#include "gbfft_internal.h"
#include "fft_tiles.cuh"

namespace gbfft {

// LOGS: log2 of the samples one CTA moves (2^12 by default; 2^11 and 2^13 are
// the autotuner's "transforms per CTA" alternatives for N <= 2^11).
// LE: log2 of the samples a thread holds: 4, or 5 for N = 2^13 / 2^14, whose
// radix-32 sub-passes (32 x 32 x 8, 32 x 32 x 16) need two exchanges instead
// of three (16 x 16 x 16 x 2, 16 x 16 x 16 x 4) at 128 registers a thread.
template <int LOGN, int LOGS = 12, int LE = 4>
struct RowsCfg : SubCfg<LOGN, LE> {
    using S = SubCfg<LOGN, LE>;
    static constexpr int TILE = 1 << LOGS;
    static constexpr int G_BY_SAMPLES = S::N >= TILE ? 1 : TILE / S::N;
    static constexpr int G_BY_THREADS = S::T >= TILE / 16 ? 1 : (TILE / 16) / S::T;
    static constexpr int G = G_BY_SAMPLES < G_BY_THREADS ? G_BY_SAMPLES : G_BY_THREADS;
    static constexpr int THREADS = G * S::T;
    static constexpr int REGS = LE == 4 ? 64 : 128;  // registers a thread
    static constexpr int MINB = THREADS * REGS >= 65536 ? 1 : 65536 / (THREADS * REGS);
    static constexpr size_t SMEM = S::NSUB > 1 ? (size_t)G * rows_buf_stride<LOGN, LE>() * sizeof(float2) : 0;
};

// DIRC: -1 forward, +1 inverse (a launch has one direction, so the sign and
// scale work is resolved at compile time).
// TAB: rows addressed through tables instead of in / out: row r is read from
// tab_in[r] and written to tab_out[r] (arrays of the rows' own addresses, in
// device memory or, for small batches, pinned host memory).  The host entries pass the caller's separate host rows this
// way; the GPU reads and writes them through the host's page tables, so a
// host batch needs no copy in HBM.  A separate instantiation, so the
// contiguous kernels are unchanged.
template <int LOGN, int LOGS, int DIRC, int LE, bool TAB = false>
__global__ void __launch_bounds__(RowsCfg<LOGN, LOGS, LE>::THREADS, RowsCfg<LOGN, LOGS, LE>::MINB)
fft_rows_kernel(const float2 *in, float2 *out, uint64_t batch, const float2 *__restrict__ tw,
                float in_im_sign, float out_re_scale, float out_im_scale, LoadOps ops,
                const uint64_t *__restrict__ tab_in, const uint64_t *__restrict__ tab_out) {
    using C = RowsCfg<LOGN, LOGS, LE>;
    extern __shared__ float2 smem_rows[];
    auto ref = [&](int g) {
        const uint64_t row = (uint64_t)blockIdx.x * C::G + g;
        if constexpr (TAB) {
            const bool act = row < batch;
            return RowRef{act ? (const float2 *)tab_in[row] : nullptr, act ? (float2 *)tab_out[row] : nullptr, act,
                          in_im_sign, out_re_scale, out_im_scale, (uint32_t)row};
        } else {
            return RowRef{in + row * C::N, out + row * C::N, row < batch, in_im_sign, out_re_scale, out_im_scale,
                          (uint32_t)row};
        }
    };
    // packed FP32 butterflies and twiddles from N = 2^8 (N = 4096: 401 -> 419
    // GSa/s); scalar below, where several transforms share a warp (2^6: 406
    // scalar against 399 packed)
    using Eng = std::conditional_t<(LOGN >= 8), DftRegsX2, DftRegsScalar>;
    rows_tile<LOGN, C::G, DIRC, LE>(ref, tw, smem_rows, ops, Eng{});
}

}  // namespace gbfft
