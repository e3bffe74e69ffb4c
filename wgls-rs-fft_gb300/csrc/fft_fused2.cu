// Fused pass pairs (fft_fused.cuh): the two-pass instantiations
// (N = 2^15 .. 2^20, both passes in one launch) and the host side shared with
// the three-pass pairs (fft_fused3.cu).
#include <algorithm>

#include "gbfft_internal.h"
#include "gbfft_plan.h"
#include "fft_fused.cuh"

namespace gbfft {

bool fused2_kernel_info(int logr1, int logr2, FusedDesc &d, int loge) {
    if (loge == 5) {
#define GBFFT_F2E(A, B, T) \
    if (logr1 == A && logr2 == B) { fused_describe<A, B, T, A + B, 0, 5>(d); return true; }
        GBFFT_F2E(8, 7, 128)
        GBFFT_F2E(8, 8, 128)
        GBFFT_F2E(9, 8, 256)
        GBFFT_F2E(9, 9, 256)
        GBFFT_F2E(10, 9, 512)
        GBFFT_F2E(10, 10, 512)
#undef GBFFT_F2E
        return false;
    }
    if (loge != 4) return false;
#define GBFFT_F2(A, B, T) \
    if (logr1 == A && logr2 == B) { fused_describe<A, B, T, A + B, 0>(d); return true; }
    GBFFT_F2(7, 6, 128)
    GBFFT_F2(7, 7, 128)
    GBFFT_F2(8, 7, 256)
    GBFFT_F2(8, 8, 256)
    GBFFT_F2(9, 8, 512)
    GBFFT_F2(9, 9, 512)
    GBFFT_F2(10, 9, 1024)
    GBFFT_F2(10, 10, 1024)
#undef GBFFT_F2
    return false;
}

int pass_sub_segments(int logr, int loge, TwiddleSegment *out, uint64_t base, int &entries) {
    switch (loge * 16 + logr) {
#define GBFFT_SEG(E, R) \
    case E * 16 + R: entries = SubCfg<R, E>::tw_entries(); return subcfg_segments<R, E>(out, base);
        GBFFT_SEG(5, 7) GBFFT_SEG(5, 8) GBFFT_SEG(5, 9) GBFFT_SEG(5, 10)
        GBFFT_SEG(4, 5) GBFFT_SEG(4, 6) GBFFT_SEG(4, 7) GBFFT_SEG(4, 8) GBFFT_SEG(4, 9) GBFFT_SEG(4, 10)
#undef GBFFT_SEG
        default: entries = 0; return -1;
    }
}

cudaError_t fused_prepare(FusedDesc &d) {
    cudaError_t e = cudaSuccess;
    if (d.smem > 48 * 1024) {
        e = cudaFuncSetAttribute(d.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)d.smem);
        if (e != cudaSuccess) return e;
    }
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&d.ctas_per_sm, d.fn, d.threads, d.smem);
    if (e != cudaSuccess || d.tmem_cols <= 0) return e;
    // Split forms: the occupancy query answers 1 for kernels that allocate
    // tensor memory, although the SM runs as many such CTAs as registers and
    // shared memory allow (tcgen05.alloc only waits while the SM's 512 TMEM
    // columns are taken, and each CTA allocates before it claims any work, so
    // such a wait never holds up a dependency).  Count them from the kernel's
    // resources, bounded by the columns each CTA holds for its whole run.
    cudaFuncAttributes fa;
    int dev = 0, smem_sm = 0, regs_sm = 0, threads_sm = 0;
    if ((e = cudaFuncGetAttributes(&fa, d.fn)) != cudaSuccess) return e;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&threads_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev)) != cudaSuccess) return e;
    const int warps = (d.threads + 31) / 32;
    const int regs_cta = ((fa.numRegs + 7) / 8) * 8 * 32 * warps;  // allocated per warp in units of 8 per thread
    const size_t smem_cta = d.smem + fa.sharedSizeBytes + 1024;      // 1 KB reserved per CTA
    int fit = std::min(regs_sm / std::max(1, regs_cta), threads_sm / std::max(1, d.threads));
    fit = std::min<int>(fit, (int)(smem_sm / smem_cta));
    d.ctas_per_sm = std::max(1, std::min(std::max(d.ctas_per_sm, fit), 512 / d.tmem_cols));
    return cudaSuccess;
}

uint32_t fused_lag(const FusedDesc &d, uint64_t ngroups, int sms) {
    const uint64_t grid = (uint64_t)std::max(1, d.ctas_per_sm) * (uint64_t)std::max(1, sms);
    const uint64_t per = 2ull * d.tiles_per_group;
    // enough queue between producer and consumer that consumers rarely wait
    uint64_t lag = (2 * grid + per - 1) / per;
    // ... but a window of intermediates that stays well inside L2
    const uint64_t cap = std::max<uint64_t>(1, kFusedWindowBytes / (8ull * d.group_samples));
    lag = std::min(std::max<uint64_t>(lag, 1), cap);
    return (uint32_t)std::min<uint64_t>(lag, ngroups);
}

cudaError_t fused_launch(const FusedDesc &d, const float2 *in, float2 *out, uint64_t batch, const float2 *tw_a,
                         const float2 *tw_b, const float2 *tw_lo, const float2 *tw_hi, float in_im, float out_re,
                         float out_im, LoadOps ops, uint32_t *ctr, uint32_t *err, int sms, cudaStream_t stream,
                         const void *gtab, const uint64_t *tab_in, const uint64_t *tab_out) {
    FusedParams P;
    P.tab_in = tab_in;
    P.tab_out = tab_out;
    P.in = in;
    P.out = out;
    P.batch = (uint32_t)batch;
    P.ngroups = (uint32_t)(batch * d.groups_per_transform);
    P.lag = fused_lag(d, P.ngroups, sms);
    P.nitems = 2u * d.tiles_per_group * P.ngroups;
    P.tw_a = tw_a;
    P.tw_b = tw_b;
    P.tw_lo = tw_lo;
    P.tw_hi = tw_hi;
    P.in_im = in_im;
    P.out_re = out_re;
    P.out_im = out_im;
    P.ops = ops;
    P.ctr = ctr;
    P.err = err;
    P.spin_limit = 1u << 22;  // ~0.5 s of 128 ns polls; a healthy wait is a few microseconds
    P.gtab = (const uint4 *)gtab;
    const uint64_t grid = std::min<uint64_t>((uint64_t)P.nitems,
                                             (uint64_t)std::max(1, d.ctas_per_sm) * (uint64_t)std::max(1, sms));
    void *args[] = {(void *)&P};
    return cudaLaunchKernel(d.fn, dim3((unsigned)grid), dim3(d.threads), args, d.smem, stream);
}

}  // namespace gbfft
