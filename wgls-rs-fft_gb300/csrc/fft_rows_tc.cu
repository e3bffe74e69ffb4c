// Split-precision tensor-core form of the single-pass transform (N = 2^4 .. 2^14),
// replacing, like fft_rows.cu, the reference's per-stage global passes
// (larsjoost/wgls-rs-fft src/shaders.rs:8-106, dispatched by src/lib.rs:582-628).
//
// The same tile as fft_rows.cu -- G whole transforms a CTA, 16 samples a
// thread, radix-16 sub-passes with shared-memory exchanges, one HBM read and
// one write per sample -- with every radix-16 butterfly set run on the tcgen05
// tensor cores (fft_tc.cuh; the radix 2/4/8 remainder stays on the FP32
// pipes).  One CTA per tile (4096 samples; one transform for N = 2^13, 2^14):
// TMEM, the mbarrier and the G parts are set up per CTA (as in
// fft_passes_tc.cu), and every completion wait is bounded.
// TF32 needs 256 B of operands per thread, so it stops at N = 2^13.
#include "gbfft_internal.h"
#include "gbfft_plan.h"
#include "fft_tc.cuh"
#include "fft_tiles.cuh"

namespace gbfft {

namespace {

__host__ __device__ constexpr uint32_t rtc_tmem_cols(int nmma) {
    return nmma * 32 <= 32 ? 32 : (nmma * 32 <= 64 ? 64 : (nmma * 32 <= 128 ? 128 : 256));
}

template <int LOGN, int KIND>
struct RowsTcCfg {
    using S = SubCfg<LOGN>;
    using Gm = TcGeom<KIND>;
    static_assert(LOGN >= 4, "a radix-16 sub-pass needs 16 samples a thread");
    // 4096 samples a CTA (one transform above that), as the FP32 tile
    static constexpr int G = S::N >= 4096 ? 1 : 4096 / S::N;
    static constexpr int THREADS = G * S::T;
    static_assert(THREADS % 128 == 0, "one M = 128 MMA per 128 threads");
    static constexpr int NMMA = THREADS / 128;
    static constexpr uint32_t TMEM_COLS = rtc_tmem_cols(NMMA);
    static constexpr size_t TILE_BYTES = (size_t)G * rows_buf_stride<LOGN>() * sizeof(float2);
    static constexpr size_t A_BYTES = (size_t)THREADS * Gm::ROW_BYTES;
    static constexpr size_t A_ALL = Gm::PARTS * A_BYTES;
    // the A operand parts alias the exchange tile (tc_dft16 waits for its readers)
    static constexpr size_t REGION = ((A_ALL > TILE_BYTES ? A_ALL : TILE_BYTES) + 1023) & ~(size_t)1023;
    static constexpr size_t OFF_G = REGION;
    static constexpr size_t OFF_MISC = OFF_G + Gm::PARTS * (size_t)Gm::G_BYTES;
    static constexpr size_t SMEM = OFF_MISC + 64;
    static constexpr int MINB = THREADS >= 1024 ? 1 : (THREADS >= 512 ? 2 : 4);
};

template <int LOGN, int DIRC, int KIND>
__global__ void __launch_bounds__(RowsTcCfg<LOGN, KIND>::THREADS, RowsTcCfg<LOGN, KIND>::MINB)
fft_rows_tc_kernel(const float2 *in, float2 *out, uint64_t batch, const float2 *__restrict__ tw,
                   float in_im_sign, float out_re_scale, float out_im_scale, LoadOps ops,
                   const uint4 *__restrict__ gtab, uint32_t *err) {
    using C = RowsTcCfg<LOGN, KIND>;
    using Gm = TcGeom<KIND>;
    extern __shared__ __align__(1024) uint8_t smem_rtc[];
    uint64_t *bar = (uint64_t *)(smem_rtc + C::OFF_MISC);
    uint32_t *s_taddr = (uint32_t *)(smem_rtc + C::OFF_MISC + 8);
    int *s_abort = (int *)(smem_rtc + C::OFF_MISC + 12);
    const int tid = threadIdx.x;
    const uint4 *gsrc = gtab + Gm::GTAB_OFF / 16;
    uint4 *gdst = (uint4 *)(smem_rtc + C::OFF_G);
    for (int i = tid; i < Gm::PARTS * Gm::G_BYTES / 16; i += C::THREADS) gdst[i] = gsrc[i];
    if (tid < 32) tmem_alloc(s_taddr, C::TMEM_COLS);
    if (tid == 0) {
        mbar_init(bar, 1);
        *s_abort = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    TcState st;
    tc_state_parts<KIND>(st, smem_rtc, C::A_BYTES, smem_rtc + C::OFF_G);
    st.bar = bar;
    st.abort = s_abort;
    st.err = err;
    st.taddr = *s_taddr;
    st.parity = 0;
    st.nmma = C::NMMA;
    st.spin_limit = kTcSpinLimit;

    auto ref = [&](int g) {
        const uint64_t row = (uint64_t)blockIdx.x * C::G + g;
        return RowRef{in + row * C::S::N, out + row * C::S::N, row < batch, in_im_sign, out_re_scale, out_im_scale,
                      (uint32_t)row};
    };
    rows_tile<LOGN, C::G, DIRC, 4>(ref, tw, (float2 *)smem_rtc, ops, DftTc<KIND>{&st});

    tc_fence_before();
    __syncthreads();
    if (tid == 0 && *s_abort) {
        // a wait gave up: let the MMAs that were issued finish before freeing TMEM
        for (uint32_t polls = 0; polls < kTcSpinLimit && !mbar_try_wait(bar, st.parity ^ 1u); ++polls) {
        }
    }
    __syncthreads();
    tc_fence_after();
    if (tid < 32) tmem_dealloc(st.taddr, C::TMEM_COLS);
}

template <int LOGN, int KIND>
void rows_tc_describe(RowsKernelInfo &k) {
    using C = RowsTcCfg<LOGN, KIND>;
    k.fn = (const void *)fft_rows_tc_kernel<LOGN, -1, KIND>;
    k.fn_inv = (const void *)fft_rows_tc_kernel<LOGN, 1, KIND>;
    k.fn_persistent = nullptr;
    k.fn_persistent_inv = nullptr;
    k.persist_ctas_per_sm = 0;
    k.threads = C::THREADS;
    k.transforms_per_cta = C::G;
    k.smem = C::SMEM;
    k.nseg = subcfg_segments<LOGN>(k.segs, 0);
    k.tw_entries = SubCfg<LOGN>::tw_entries();
}

template <int KIND>
bool rows_tc_info_kind(int logn, RowsKernelInfo &k) {
    switch (logn) {
#define GBFFT_RTC(L) \
    case L: rows_tc_describe<L, KIND>(k); return true;
        GBFFT_RTC(4) GBFFT_RTC(5) GBFFT_RTC(6) GBFFT_RTC(7) GBFFT_RTC(8) GBFFT_RTC(9) GBFFT_RTC(10)
        GBFFT_RTC(11) GBFFT_RTC(12) GBFFT_RTC(13)
#undef GBFFT_RTC
        case 14:
            if constexpr (KIND == kTcTF32) return false;  // 256 KB of TF32 operands
            else {
                rows_tc_describe<14, KIND>(k);
                return true;
            }
        default: return false;
    }
}

}  // namespace

bool rows_tc_kernel_info(int logn, int precision, RowsKernelInfo &k) {
    switch (tc_kind_of_precision(precision)) {
        case kTcBF16: return rows_tc_info_kind<kTcBF16>(logn, k);
        case kTcBF16X6: return rows_tc_info_kind<kTcBF16X6>(logn, k);
        case kTcTF32: return rows_tc_info_kind<kTcTF32>(logn, k);
        default: return rows_tc_info_kind<kTcF16>(logn, k);
    }
}

cudaError_t rows_tc_prepare(RowsKernelInfo &k) {
    if (k.smem <= 48 * 1024) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k.smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k.fn_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k.smem);
    return e;
}

cudaError_t rows_tc_launch(const RowsKernelInfo &k, const float2 *in, float2 *out, uint64_t batch,
                           const float2 *tw, int direction, int logn, const void *gtab, uint32_t *err,
                           cudaStream_t stream, LoadOps ops) {
    if (batch == 0) return cudaSuccess;
    const uint64_t ctas = (batch + k.transforms_per_cta - 1) / k.transforms_per_cta;
    if (ctas > 0x7fffffffull) return cudaErrorInvalidConfiguration;
    const bool inv = direction == GBFFT_INVERSE;
    const float scale = inv ? ldexpf(1.0f, -logn) : 1.0f;
    float in_im = inv ? -1.0f : 1.0f;
    float out_re = scale, out_im = inv ? -scale : 1.0f;
    const uint4 *g = (const uint4 *)gtab;
    void *args[] = {(void *)&in,     (void *)&out,    (void *)&batch, (void *)&tw, (void *)&in_im,
                    (void *)&out_re, (void *)&out_im, (void *)&ops,   (void *)&g,  (void *)&err};
    return cudaLaunchKernel(inv ? k.fn_inv : k.fn, dim3((unsigned)ctas), dim3(k.threads), args, k.smem, stream);
}

}  // namespace gbfft
