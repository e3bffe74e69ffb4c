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
#include "gbfft_internal.h"
#include "gbfft_plan.h"
#include "fft_smem.cuh"

namespace gbfft {

constexpr int kPassLogCols = 4;
constexpr int kPassCols = 1 << kPassLogCols;

template <int LOGR>
struct PassCfg : SubCfg<LOGR> {
    using S = SubCfg<LOGR>;
    static constexpr int THREADS = kPassCols * S::T;
    static constexpr int MINB = THREADS >= 1024 ? 1 : 1024 / THREADS;
    static constexpr int COLTW_STRIDE = S::E + 1;  // padded: conflict-free column reads
    static constexpr size_t SMEM = ((size_t)kPassCols * S::N + kPassCols * COLTW_STRIDE) * sizeof(float2);
};

template <int LOGR, int I, bool DONE = (I >= SubCfg<LOGR>::NSUB)>
struct PassChain {
    using C = SubCfg<LOGR>;
    __device__ __forceinline__ static void run(float2 (&v)[C::E], int t, int c, float2 *buf, const float2 *tw) {
        constexpr int PR = C::logr(I - 1), PP = C::logp(I - 1);
        if (I > 1) __syncthreads();
#pragma unroll
        for (int b = 0; b < (C::E >> PR); ++b)
#pragma unroll
            for (int q = 0; q < (1 << PR); ++q)
                buf[(subpass_out_pos<PR, PP, C::LOGT>(t, b, q) << kPassLogCols) + c] = v[b + q * (C::E >> PR)];
        __syncthreads();
#pragma unroll
        for (int e = 0; e < C::E; ++e) v[e] = buf[((t + C::T * e) << kPassLogCols) + c];
        subpass_run<LOGR, I>(v, t, tw);
        PassChain<LOGR, I + 1>::run(v, t, c, buf, tw);
    }
};
template <int LOGR, int I>
struct PassChain<LOGR, I, true> {
    __device__ __forceinline__ static void run(float2 (&)[SubCfg<LOGR>::E], int, int, float2 *, const float2 *) {}
};

__device__ __forceinline__ float2 twiddle_2level(const float2 *__restrict__ lo, const float2 *__restrict__ hi,
                                                 uint32_t ex, int split) {
    return cmul(ld_tw(hi + (ex >> split)), ld_tw(lo + (ex & ((1u << split) - 1))));
}

template <int LOGR, bool FIRST>
__global__ void __launch_bounds__(PassCfg<LOGR>::THREADS, PassCfg<LOGR>::MINB)
fft_pass_kernel(const float2 *in, float2 *out, int logn, int logp, const float2 *__restrict__ tw,
                const float2 *__restrict__ tw_lo, const float2 *__restrict__ tw_hi, int tw_split,
                float in_im_sign, float out_re_scale, float out_im_scale) {
    using C = PassCfg<LOGR>;
    constexpr int R = C::N, T = C::T, E = C::E;
    extern __shared__ float2 smem_pass[];
    float2 *coltw = smem_pass + kPassCols * R;
    const int tid = threadIdx.x;
    const int c = tid & (kPassCols - 1);
    const int t = tid >> kPassLogCols;
    const int lognc = logn - LOGR;                     // log2 (columns per transform)
    const uint64_t tile = blockIdx.x;
    const uint64_t b = tile >> (lognc - kPassLogCols);
    const uint32_t j0 = (uint32_t)(tile & ((1ull << (lognc - kPassLogCols)) - 1)) << kPassLogCols;
    const uint32_t j = j0 + c;
    const float2 *src = in + (b << logn);
    float2 *dst = out + (b << logn);

    float2 v[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const uint32_t m = t + T * e;
        float2 x = ld_stream(src + j + ((uint64_t)m << lognc));
        x.y *= in_im_sign;
        v[e] = x;
    }
    if (!FIRST) {
        const uint32_t pmask = (1u << logp) - 1;
        // per-column factors W_{E p}^{e k} = W_N^{(e k) << (logn - LOGE - logp)}
        const int sh_col = logn - C::LOGE - logp;
        for (int i = tid; i < kPassCols * E; i += C::THREADS) {
            const int cc = i >> C::LOGE, ee = i & (E - 1);
            const uint32_t kk = (j0 + cc) & pmask;
            coltw[cc * C::COLTW_STRIDE + ee] = twiddle_2level(tw_lo, tw_hi, (kk * ee) << sh_col, tw_split);
        }
        // per-thread factor W_{R p}^{t k}
        const uint32_t k = j & pmask;
        const float2 a = twiddle_2level(tw_lo, tw_hi, (t * k) << (logn - LOGR - logp), tw_split);
        __syncthreads();
#pragma unroll
        for (int e = 0; e < E; ++e) v[e] = cmul(v[e], cmul(a, coltw[c * C::COLTW_STRIDE + e]));
    }
    subpass_run<LOGR, 0>(v, t, tw);
    PassChain<LOGR, 1>::run(v, t, c, smem_pass, tw);

    constexpr int LR = C::logr(C::NSUB - 1), LP = C::logp(C::NSUB - 1);
    constexpr int NB = E >> LR;
    if (FIRST) {
        // Outputs of column j are contiguous at j R + q: stage them as
        // [column][q ^ column] and store the 16 R-sample block linearly.
        __syncthreads();
#pragma unroll
        for (int bb = 0; bb < NB; ++bb)
#pragma unroll
            for (int q = 0; q < (1 << LR); ++q) {
                const int pos = subpass_out_pos<LR, LP, C::LOGT>(t, bb, q);
                smem_pass[c * R + (pos ^ c)] = v[bb + q * NB];
            }
        __syncthreads();
        float2 *blk = dst + (uint64_t)j0 * R;
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const int lin = tid + C::THREADS * e;
            const int cc = lin >> LOGR, q = lin & (R - 1);
            const float2 y = smem_pass[cc * R + (q ^ cc)];
            st_stream(blk + lin, make_float2(y.x * out_re_scale, y.y * out_im_scale));
        }
    } else {
        const uint32_t pmask = (1u << logp) - 1;
        float2 *col = dst + ((uint64_t)(j >> logp) << (LOGR + logp)) + (j & pmask);
#pragma unroll
        for (int bb = 0; bb < NB; ++bb)
#pragma unroll
            for (int q = 0; q < (1 << LR); ++q) {
                const int pos = subpass_out_pos<LR, LP, C::LOGT>(t, bb, q);
                const float2 y = v[bb + q * NB];
                st_stream(col + ((uint64_t)pos << logp), make_float2(y.x * out_re_scale, y.y * out_im_scale));
            }
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

template <int LOGR>
static void pass_describe(PassDesc &d, bool first) {
    using C = PassCfg<LOGR>;
    d.fn = first ? (const void *)fft_pass_kernel<LOGR, true> : (const void *)fft_pass_kernel<LOGR, false>;
    d.threads = C::THREADS;
    d.smem = C::SMEM;
    d.cols = kPassCols;
    d.nseg = subcfg_segments<LOGR>(d.segs, 0);
    d.tw_entries = C::tw_entries();
}

bool pass_kernel_info(int logr, bool first, PassDesc &d) {
    d.logr = logr;
    switch (logr) {
#define GBFFT_PASS_CASE(L) \
    case L: pass_describe<L>(d, first); return true;
        GBFFT_PASS_CASE(5) GBFFT_PASS_CASE(6) GBFFT_PASS_CASE(7) GBFFT_PASS_CASE(8)
        GBFFT_PASS_CASE(9) GBFFT_PASS_CASE(10)
#undef GBFFT_PASS_CASE
        default: return false;
    }
}

cudaError_t pass_prepare(const PassDesc &d) {
    if (d.smem > 48 * 1024)
        return cudaFuncSetAttribute(d.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)d.smem);
    return cudaSuccess;
}

cudaError_t pass_launch(const PassDesc &d, const float2 *in, float2 *out, uint64_t batch, int logn,
                        const float2 *tw_sub, const float2 *tw_lo, const float2 *tw_hi, int tw_split,
                        float in_im_sign, float out_re_scale, float out_im_scale, cudaStream_t stream) {
    const uint64_t tiles = batch << (logn - d.logr - kPassLogCols);
    if (tiles == 0) return cudaSuccess;
    if (tiles > 0x7fffffffull) return cudaErrorInvalidConfiguration;
    int logp = d.logp;
    void *args[] = {(void *)&in,    (void *)&out,   (void *)&logn,     (void *)&logp,
                    (void *)&tw_sub, (void *)&tw_lo, (void *)&tw_hi,   (void *)&tw_split,
                    (void *)&in_im_sign, (void *)&out_re_scale, (void *)&out_im_scale};
    return cudaLaunchKernel(d.fn, dim3((unsigned)tiles), dim3(d.threads), args, d.smem, stream);
}

}  // namespace gbfft
