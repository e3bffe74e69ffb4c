// Multi-pass form for N > 2^14: the transform is split into P global Stockham
// passes of large radix R_i = 2^5 .. 2^10 (N = R_1 ... R_P, P = 2 up to
// N = 2^20, 3 up to 2^30).  Global pass i, with p = R_1 ... R_{i-1}, is the
// reference's stage rule (larsjoost/wgls-rs-fft src/shaders.rs:20-62) at radix
// R_i: column j < N/R reads j + m N/R, is multiplied by W_{R p}^{m k}
// (k = j mod p), goes through a length-R DFT and lands at
// (j/p) R p + k + q p.  The length-R DFT itself runs in shared memory/registers
// with the same radix-16 sub-pass machinery as the single-pass kernel, so each
// global pass costs exactly one HBM read and one HBM write per sample.
//
// One CTA takes 16 adjacent columns of one transform: lanes are mapped column
// fastest, so every global load and store moves 16 x 8 = 128 contiguous bytes
// per half-warp, and the shared-memory tile [row][16 columns] is free of bank
// conflicts for every access pattern.  The first pass (p = 1) writes each
// column's R outputs contiguously; it stages them through shared memory
// (XOR-swizzled [column][row]) so that its HBM stores are fully coalesced too.
//
// Pre-twiddle: thread t of column j holds rows m = t + T e, and
//   W_{R p}^{m k} = W_{R p}^{t k} * W_{E p}^{e k}.
// The first factor is one lookup per thread; the second depends only on the
// column and e, so the CTA builds it once into a padded 16 x 17 shared table.
// Both come from two FP64-built tables (W_N^i for i < 2^s and W_N^{i 2^s}).
#include <algorithm>

#include "gbfft_internal.h"
#include "gbfft_plan.h"
#include "fft_tiles.cuh"

namespace gbfft {

// LE: log2 of the samples a thread holds (4: 64 registers; 5: radix-32
// sub-passes at 128 registers, one exchange fewer for radix 2^9 / 2^10).
template <int LOGR, int LE = 4>
struct PassCfg : PassTileCfg<LOGR, 1, LE> {
    using K = PassTileCfg<LOGR, 1, LE>;
    static constexpr int REGS = LE == 4 ? 64 : 128;
    static constexpr int MINB = K::THREADS * REGS >= 65536 ? 1 : 65536 / (K::THREADS * REGS);
    static constexpr size_t SMEM = K::SMEM_ELEMS * sizeof(float2);
};

template <int LOGR, bool FIRST, int LE = 4>
__global__ void __launch_bounds__(PassCfg<LOGR, LE>::THREADS, PassCfg<LOGR, LE>::MINB)
fft_pass_kernel(const float2 *in, float2 *out, int logn, int logp, const float2 *__restrict__ tw,
                const float2 *__restrict__ tw_lo, const float2 *__restrict__ tw_hi, int tw_split,
                float in_im_sign, float out_re_scale, float out_im_scale, LoadOps ops) {
    extern __shared__ float2 smem_pass[];
    const int lognc = logn - LOGR;                     // log2 (columns per transform)
    const uint64_t tile = blockIdx.x;
    const uint64_t b = tile >> (lognc - kColsLog);
    PassArgs a;
    a.src = in + (b << logn);
    a.dst = out + (b << logn);
    a.logn = logn;
    a.logp = logp;
    a.col0 = (uint32_t)(tile & ((1ull << (lognc - kColsLog)) - 1)) << kColsLog;
    a.tw_sub = tw;
    a.tw_lo = tw_lo;
    a.tw_hi = tw_hi;
    a.tw_split = tw_split;
    a.in_im = in_im_sign;
    a.out_re = out_re_scale;
    a.out_im = out_im_scale;
    a.coherent_load = false;
    a.row = (uint32_t)b;
    a.ops = ops;
    pass_tile<LOGR, 1, FIRST, DftRegs, 0, -1, LE>(a, smem_pass);
}

// Persistent variant: each CTA walks tiles blockIdx.x, +gridDim.x, ... and asks
// L2 for the next tile's R row segments (128 bytes each, one per thread)
// before computing the current one.
template <int LOGR, bool FIRST, int LE = 4>
__global__ void __launch_bounds__(PassCfg<LOGR, LE>::THREADS, PassCfg<LOGR, LE>::MINB)
fft_pass_persistent_kernel(const float2 *in, float2 *out, int logn, int logp, const float2 *__restrict__ tw,
                           const float2 *__restrict__ tw_lo, const float2 *__restrict__ tw_hi, int tw_split,
                           float in_im_sign, float out_re_scale, float out_im_scale, LoadOps ops,
                           uint64_t ntiles) {
    extern __shared__ float2 smem_pass[];
    constexpr int R = 1 << LOGR;
    const int lognc = logn - LOGR;
    const uint64_t tiles_per_row = 1ull << (lognc - kColsLog);
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint64_t next = tile + gridDim.x;
        if (next < ntiles) {
            const float2 *nb = in + ((next / tiles_per_row) << logn) + ((next % tiles_per_row) << kColsLog);
            for (int m = threadIdx.x; m < R; m += PassCfg<LOGR, LE>::THREADS) prefetch_l2(nb + ((uint64_t)m << lognc));
        }
        const uint64_t b = tile / tiles_per_row;
        PassArgs a;
        a.src = in + (b << logn);
        a.dst = out + (b << logn);
        a.logn = logn;
        a.logp = logp;
        a.col0 = (uint32_t)((tile % tiles_per_row) << kColsLog);
        a.tw_sub = tw;
        a.tw_lo = tw_lo;
        a.tw_hi = tw_hi;
        a.tw_split = tw_split;
        a.in_im = in_im_sign;
        a.out_re = out_re_scale;
        a.out_im = out_im_scale;
        a.coherent_load = false;
        a.row = (uint32_t)b;
        a.ops = ops;
        pass_tile<LOGR, 1, FIRST, DftRegs, 0, -1, LE>(a, smem_pass);
        __syncthreads();  // shared memory is reused by the next tile
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

template <int LOGR, int LE = 4>
static void pass_describe(PassDesc &d, bool first) {
    using C = PassCfg<LOGR, LE>;
    d.fn = first ? (const void *)fft_pass_kernel<LOGR, true, LE> : (const void *)fft_pass_kernel<LOGR, false, LE>;
    d.fn_persistent = first ? (const void *)fft_pass_persistent_kernel<LOGR, true, LE>
                            : (const void *)fft_pass_persistent_kernel<LOGR, false, LE>;
    d.threads = C::THREADS;
    d.smem = C::SMEM;
    d.cols = kCols;
    d.nseg = subcfg_segments<LOGR, LE>(d.segs, 0);
    d.tw_entries = SubCfg<LOGR, LE>::tw_entries();
}

bool pass_kernel_info(int logr, bool first, PassDesc &d, int loge) {
    d.logr = logr;
    if (loge == 5) {  // first passes of radix 2^9 / 2^10 (N = 2^25, 2^26 as (L-16, 8, 8))
        if (!first) return false;
        switch (logr) {
            case 9: pass_describe<9, 5>(d, true); return true;
            case 10: pass_describe<10, 5>(d, true); return true;
            default: return false;
        }
    }
    if (loge != 4) return false;
    switch (logr) {
#define GBFFT_PASS_CASE(L) \
    case L: pass_describe<L>(d, first); return true;
        GBFFT_PASS_CASE(5) GBFFT_PASS_CASE(6) GBFFT_PASS_CASE(7) GBFFT_PASS_CASE(8)
        GBFFT_PASS_CASE(9) GBFFT_PASS_CASE(10)
#undef GBFFT_PASS_CASE
        default: return false;
    }
}

cudaError_t pass_prepare(PassDesc &d) {
    cudaError_t e = cudaSuccess;
    if (d.smem > 48 * 1024) {
        e = cudaFuncSetAttribute(d.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)d.smem);
        if (e == cudaSuccess && d.fn_persistent)
            e = cudaFuncSetAttribute(d.fn_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)d.smem);
        if (e != cudaSuccess) return e;
    }
    if (!d.fn_persistent) return cudaSuccess;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&d.persist_ctas_per_sm, d.fn_persistent, d.threads, d.smem);
}

cudaError_t pass_launch(const PassDesc &d, const float2 *in, float2 *out, uint64_t batch, int logn,
                        const float2 *tw_sub, const float2 *tw_lo, const float2 *tw_hi, int tw_split,
                        float in_im_sign, float out_re_scale, float out_im_scale, cudaStream_t stream,
                        bool persistent, int sms, LoadOps ops) {
    uint64_t tiles = batch << (logn - d.logr - kColsLog);
    if (tiles == 0) return cudaSuccess;
    int logp = d.logp;
    if (persistent && d.fn_persistent && d.persist_ctas_per_sm > 0 && sms > 0) {
        const uint64_t grid = std::min<uint64_t>(tiles, (uint64_t)d.persist_ctas_per_sm * (uint64_t)sms);
        void *args[] = {(void *)&in,    (void *)&out,   (void *)&logn,     (void *)&logp,
                        (void *)&tw_sub, (void *)&tw_lo, (void *)&tw_hi,   (void *)&tw_split,
                        (void *)&in_im_sign, (void *)&out_re_scale, (void *)&out_im_scale, (void *)&ops,
                        (void *)&tiles};
        return cudaLaunchKernel(d.fn_persistent, dim3((unsigned)grid), dim3(d.threads), args, d.smem, stream);
    }
    if (tiles > 0x7fffffffull) return cudaErrorInvalidConfiguration;
    void *args[] = {(void *)&in,    (void *)&out,   (void *)&logn,     (void *)&logp,
                    (void *)&tw_sub, (void *)&tw_lo, (void *)&tw_hi,   (void *)&tw_split,
                    (void *)&in_im_sign, (void *)&out_re_scale, (void *)&out_im_scale, (void *)&ops};
    return cudaLaunchKernel(d.fn, dim3((unsigned)tiles), dim3(d.threads), args, d.smem, stream);
}

}  // namespace gbfft
