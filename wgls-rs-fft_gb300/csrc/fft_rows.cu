// Single-pass batched FFT for N = 2^0 .. 2^14: one HBM read and one HBM write
// per sample.  Replaces the reference's floor(log4 N) radix-4 global passes
// plus optional radix-2 pass (larsjoost/wgls-rs-fft src/shaders.rs:8-106,
// dispatched by src/lib.rs:582-628), each of which round-trips all 8*N*B bytes
// through memory.
//
// One CTA transforms G whole rows (G*N = 4096 samples for N <= 4096, one row
// above):
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
#include "gbfft_internal.h"
#include "fft_smem.cuh"

namespace gbfft {

template <int LOGN>
struct RowsCfg : SubCfg<LOGN> {
    using S = SubCfg<LOGN>;
    static constexpr int G_BY_SAMPLES = S::N >= 4096 ? 1 : 4096 / S::N;
    static constexpr int G_BY_THREADS = S::T >= 256 ? 1 : 256 / S::T;
    static constexpr int G = G_BY_SAMPLES < G_BY_THREADS ? G_BY_SAMPLES : G_BY_THREADS;
    static constexpr int THREADS = G * S::T;
    static constexpr int MINB = THREADS >= 1024 ? 1 : (THREADS >= 512 ? 2 : 4);
    static constexpr size_t SMEM = S::NSUB > 1 ? (size_t)G * S::N * sizeof(float2) : 0;
};

__device__ __forceinline__ int swz(int a, int logp) {
    return logp < 4 ? (a ^ (((a >> 4) << logp) & 15)) : a;
}

template <int LOGN, int I, bool DONE = (I >= SubCfg<LOGN>::NSUB)>
struct RowsChain {
    using C = SubCfg<LOGN>;
    __device__ __forceinline__ static void run(float2 (&v)[C::E], int t, float2 *buf, const float2 *tw) {
        constexpr int PR = C::logr(I - 1), PP = C::logp(I - 1);  // previous sub-pass
        if (I > 1) __syncthreads();  // readers of the previous exchange are done
#pragma unroll
        for (int b = 0; b < (C::E >> PR); ++b)
#pragma unroll
            for (int q = 0; q < (1 << PR); ++q)
                buf[swz(subpass_out_pos<PR, PP, C::LOGT>(t, b, q), PP)] = v[b + q * (C::E >> PR)];
        __syncthreads();
#pragma unroll
        for (int e = 0; e < C::E; ++e) v[e] = buf[swz(t + C::T * e, PP)];
        subpass_run<LOGN, I>(v, t, tw);
        RowsChain<LOGN, I + 1>::run(v, t, buf, tw);
    }
};
template <int LOGN, int I>
struct RowsChain<LOGN, I, true> {
    __device__ __forceinline__ static void run(float2 (&)[SubCfg<LOGN>::E], int, float2 *, const float2 *) {}
};

template <int LOGN>
__global__ void __launch_bounds__(RowsCfg<LOGN>::THREADS, RowsCfg<LOGN>::MINB)
fft_rows_kernel(const float2 *in, float2 *out, uint64_t batch, const float2 *__restrict__ tw,
                float in_im_sign, float out_re_scale, float out_im_scale) {
    using C = RowsCfg<LOGN>;
    extern __shared__ float2 smem_rows[];
    const int tid = threadIdx.x;
    const int g = tid >> C::LOGT;
    const int t = tid & (C::T - 1);
    const uint64_t row = (uint64_t)blockIdx.x * C::G + g;
    const bool active = row < batch;
    const float2 *src = in + row * C::N;
    float2 *dst = out + row * C::N;
    float2 *buf = smem_rows + g * C::N;

    float2 v[C::E];
#pragma unroll
    for (int e = 0; e < C::E; ++e) {
        float2 x = active ? ld_stream(src + t + C::T * e) : make_float2(0.f, 0.f);
        x.y *= in_im_sign;
        v[e] = x;
    }
    subpass_run<LOGN, 0>(v, t, tw);
    RowsChain<LOGN, 1>::run(v, t, buf, tw);

    // Last sub-pass (p * R = N): output q of butterfly j sits at j + q p.
    if (active) {
        constexpr int LR = C::logr(C::NSUB - 1), LP = C::logp(C::NSUB - 1);
        constexpr int NB = C::E >> LR;
#pragma unroll
        for (int b = 0; b < NB; ++b)
#pragma unroll
            for (int q = 0; q < (1 << LR); ++q) {
                const float2 y = v[b + q * NB];
                st_stream(dst + subpass_out_pos<LR, LP, C::LOGT>(t, b, q),
                          make_float2(y.x * out_re_scale, y.y * out_im_scale));
            }
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

template <int LOGN>
static void rows_describe(RowsKernelInfo &k) {
    using C = RowsCfg<LOGN>;
    k.fn = (const void *)fft_rows_kernel<LOGN>;
    k.threads = C::THREADS;
    k.transforms_per_cta = C::G;
    k.smem = C::SMEM;
    k.nseg = subcfg_segments<LOGN>(k.segs, 0);
    k.tw_entries = C::tw_entries();
}

bool rows_kernel_info(int logn, RowsKernelInfo &k) {
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

cudaError_t rows_prepare(const RowsKernelInfo &k) {
    if (k.smem > 48 * 1024)
        return cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k.smem);
    return cudaSuccess;
}

cudaError_t rows_launch(const RowsKernelInfo &k, const float2 *in, float2 *out, uint64_t batch,
                        const float2 *tw, int direction, int logn, cudaStream_t stream) {
    if (batch == 0) return cudaSuccess;
    const uint64_t ctas = (batch + k.transforms_per_cta - 1) / k.transforms_per_cta;
    if (ctas > 0x7fffffffull) return cudaErrorInvalidConfiguration;
    const bool inv = direction == GBFFT_INVERSE;
    const float scale = inv ? ldexpf(1.0f, -logn) : 1.0f;
    float in_im = inv ? -1.0f : 1.0f;
    float out_re = scale, out_im = inv ? -scale : 1.0f;
    void *args[] = {(void *)&in, (void *)&out, (void *)&batch, (void *)&tw,
                    (void *)&in_im, (void *)&out_re, (void *)&out_im};
    return cudaLaunchKernel(k.fn, dim3((unsigned)ctas), dim3(k.threads), args, k.smem, stream);
}

}  // namespace gbfft
