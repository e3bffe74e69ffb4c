// Single-pass batched FFT for N = 2^0 .. 2^14: one HBM read and one HBM write
// per sample.  Replaces the reference's floor(log4 N) radix-4 global passes
// plus optional radix-2 pass (larsjoost/wgls-rs-fft src/shaders.rs:8-106,
// dispatched by src/lib.rs:582-628), each of which round-trips all 8*N*B bytes
// through memory.
//
// One CTA transforms G whole rows (G*N = 4096 samples for N <= 4096 -- or
// 2048 / 8192, the tuner's alternatives for N = 2^6 .. 2^11 -- one row above):
//   * each thread owns E = 16 samples of one row (T = N/E threads per row) and
//     loads them straight from HBM into registers -- sample t + T*e, so a warp
//     reads 256 contiguous bytes per load instruction;
//   * radix-16 Stockham sub-passes (one radix 2/4/8 remainder sub-pass last)
//     run in registers; samples are exchanged through shared memory between
//     sub-passes;
//   * the last sub-pass writes natural-order results straight to HBM.
// Buffers written by a sub-pass with stride p < 16 are XOR swizzled
// (a ^ ((a >> 4) * p & 15)); with that every exchange is free of bank
// conflicts for N >= 256.
#include <algorithm>

#include "gbfft_internal.h"
#include "fft_rows.cuh"
#include "fft_tiles.cuh"

namespace gbfft {

// Persistent variant for the sizes whose per-transform footprint allows only
// one or two CTAs per SM (N = 2^12 .. 2^14): each CTA walks tiles
// blockIdx.x, +gridDim.x, ... and, before computing a tile, asks L2 for the
// next one (one 128-byte line per thread), so the HBM fetch of tile i+1
// overlaps the shared-memory sub-passes of tile i.
template <int LOGN, int LOGS, int DIRC, int LE>
__global__ void __launch_bounds__(RowsCfg<LOGN, LOGS, LE>::THREADS, RowsCfg<LOGN, LOGS, LE>::MINB)
fft_rows_persistent_kernel(const float2 *in, float2 *out, uint64_t batch, const float2 *__restrict__ tw,
                           float in_im_sign, float out_re_scale, float out_im_scale, LoadOps ops,
                           const uint64_t *, const uint64_t *) {  // (no row tables: the host never passes them)
    using C = RowsCfg<LOGN, LOGS, LE>;
    extern __shared__ float2 smem_rows[];
    constexpr uint32_t kTileSamples = C::G * C::N;
    constexpr uint32_t kLines = kTileSamples * sizeof(float2) / 128;
    const uint64_t ntiles = (batch + C::G - 1) / C::G;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint64_t next = tile + gridDim.x;
        if (next < ntiles) {
            const char *p = (const char *)(in + next * kTileSamples);
            const uint64_t avail = (batch - next * C::G) * C::N * sizeof(float2) / 128;  // lines inside the batch
            for (uint32_t l = threadIdx.x; l < kLines && l < avail; l += C::THREADS) prefetch_l2(p + (uint64_t)l * 128);
        }
        auto ref = [&](int g) {
            const uint64_t row = tile * C::G + g;
            return RowRef{in + row * C::N, out + row * C::N, row < batch, in_im_sign, out_re_scale, out_im_scale,
                      (uint32_t)row};
        };
        // scalar butterflies: this loop serves N = 2^14, one transform per SM,
        // where the packed ones measured slower (276 against 259 GSa/s)
        rows_tile<LOGN, C::G, DIRC, LE>(ref, tw, smem_rows, ops, DftRegsScalar{});
        __syncthreads();  // shared memory is reused by the next tile
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

template <int LOGN, int LOGS = 12, int LE = 4>
static void rows_describe(RowsKernelInfo &k) {
    using C = RowsCfg<LOGN, LOGS, LE>;
    k.fn = (const void *)fft_rows_kernel<LOGN, LOGS, -1, LE>;
    k.fn_persistent = (const void *)fft_rows_persistent_kernel<LOGN, LOGS, -1, LE>;
    k.fn_inv = (const void *)fft_rows_kernel<LOGN, LOGS, 1, LE>;
    k.fn_persistent_inv = (const void *)fft_rows_persistent_kernel<LOGN, LOGS, 1, LE>;
    rows_tab_describe(LOGN, LOGS, LE, k);
    k.threads = C::THREADS;
    k.transforms_per_cta = C::G;
    k.smem = C::SMEM;
    k.nseg = subcfg_segments<LOGN, LE>(k.segs, 0);
    k.tw_entries = C::tw_entries();
}

bool rows_kernel_info(int logn, RowsKernelInfo &k, int logs, int loge) {
    if (loge == 5) {  // 32 samples a thread: N = 2^13, 2^14 (one transform a CTA)
        if (logs != 12) return false;
        switch (logn) {
            case 13: rows_describe<13, 12, 5>(k); return true;
            case 14: rows_describe<14, 12, 5>(k); return true;
            default: return false;
        }
    }
    if (loge != 4) return false;
    if (logs == 11 || logs == 13) {  // other tile sizes for the sizes that batch transforms in a CTA
        switch (logn) {
#define GBFFT_ROWS_TILE(L)                                              \
    case L:                                                            \
        if (logs == 11) rows_describe<L, 11>(k); else rows_describe<L, 13>(k); \
        return true;
            GBFFT_ROWS_TILE(6) GBFFT_ROWS_TILE(7) GBFFT_ROWS_TILE(8) GBFFT_ROWS_TILE(9)
            GBFFT_ROWS_TILE(10) GBFFT_ROWS_TILE(11)
#undef GBFFT_ROWS_TILE
            default: return false;
        }
    }
    if (logs != 12) return false;
    switch (logn) {
#define GBFFT_ROWS_CASE(L) \
    case L: rows_describe<L>(k); return true;
        GBFFT_ROWS_CASE(0) GBFFT_ROWS_CASE(1) GBFFT_ROWS_CASE(2) GBFFT_ROWS_CASE(3)
        GBFFT_ROWS_CASE(4) GBFFT_ROWS_CASE(5) GBFFT_ROWS_CASE(6) GBFFT_ROWS_CASE(7)
        GBFFT_ROWS_CASE(8) GBFFT_ROWS_CASE(9) GBFFT_ROWS_CASE(10) GBFFT_ROWS_CASE(11)
        GBFFT_ROWS_CASE(12) GBFFT_ROWS_CASE(13) GBFFT_ROWS_CASE(14)
#undef GBFFT_ROWS_CASE
        default: return false;
    }
}

cudaError_t rows_prepare(RowsKernelInfo &k) {
    cudaError_t e = cudaSuccess;
    if (k.smem > 48 * 1024) {
        for (const void *fn : {k.fn, k.fn_persistent, k.fn_inv, k.fn_persistent_inv, k.fn_tab, k.fn_tab_inv}) {
            if (!fn) continue;
            e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k.smem);
            if (e != cudaSuccess) return e;
        }
    }
    int inv_ctas = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k.persist_ctas_per_sm, k.fn_persistent, k.threads, k.smem);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&inv_ctas, k.fn_persistent_inv, k.threads, k.smem);
    k.persist_ctas_per_sm = std::min(k.persist_ctas_per_sm, inv_ctas);
    return e;
}

cudaError_t rows_launch(const RowsKernelInfo &k, const float2 *in, float2 *out, uint64_t batch,
                        const float2 *tw, int direction, int logn, bool persistent, int sms, cudaStream_t stream,
                        LoadOps ops, const uint64_t *tab_in, const uint64_t *tab_out) {
    if (batch == 0) return cudaSuccess;
    uint64_t ctas = (batch + k.transforms_per_cta - 1) / k.transforms_per_cta;
    const bool inv = direction == GBFFT_INVERSE;
    const void *fn = tab_in ? (inv ? k.fn_tab_inv : k.fn_tab) : (inv ? k.fn_inv : k.fn);
    if (tab_in && !fn) return cudaErrorInvalidDeviceFunction;
    if (persistent && k.persist_ctas_per_sm > 0 && sms > 0 && !tab_in) {
        fn = inv ? k.fn_persistent_inv : k.fn_persistent;
        ctas = std::min<uint64_t>(ctas, (uint64_t)k.persist_ctas_per_sm * (uint64_t)sms);
    }
    if (ctas > 0x7fffffffull) return cudaErrorInvalidConfiguration;
    const float scale = inv ? ldexpf(1.0f, -logn) : 1.0f;
    float in_im = inv ? -1.0f : 1.0f;
    float out_re = scale, out_im = inv ? -scale : 1.0f;
    void *args[] = {(void *)&in,     (void *)&out,    (void *)&batch, (void *)&tw,     (void *)&in_im,
                    (void *)&out_re, (void *)&out_im, (void *)&ops,   (void *)&tab_in, (void *)&tab_out};
    return cudaLaunchKernel(fn, dim3((unsigned)ctas), dim3(k.threads), args, k.smem, stream);
}

}  // namespace gbfft
