// Split-precision tensor-core form of the multi-pass transform (N >= 2^15).
//
// Identical data flow to fft_passes.cu -- one HBM read and one HBM write per
// sample per global pass, FP32 twiddles, FP32 shared-memory exchanges -- but
// every radix-16 butterfly set of a sub-pass runs on the tcgen05 tensor cores
// as D = A.G with FP16 (or BF16) hi/lo operands and FP32 accumulation in
// tensor memory (fft_tc.cuh).  Radix 2/4/8 remainder sub-passes stay on the
// FP32 pipes.
//
// Per CTA: warp 0 allocates 32 TMEM columns per 128 threads (the D blocks),
// thread 0 initialises one mbarrier that tcgen05.commit arrives on, and the
// four 32 x 32 operand parts of G (hi/lo, FP16/BF16, precomputed in canonical
// layout) are copied into shared memory.  Every completion wait is bounded:
// on expiry the kernel raises an error flag, stops issuing MMAs, waits (again
// bounded) for the MMAs it issued, frees its TMEM and finishes.
#include "gbfft_internal.h"
#include "gbfft_plan.h"
#include "fft_tc.cuh"
#include "fft_tiles.cuh"

namespace gbfft {

// Column groups per CTA: enough threads (>= 128) to fill one M = 128 MMA.
template <int LOGR>
constexpr int tc_groups() {
    return (kCols << (LOGR - 4)) >= 128 ? 1 : 128 / (kCols << (LOGR - 4));
}

template <int LOGR>
struct PassTcCfg {
    static constexpr int NG = tc_groups<LOGR>();
    using K = PassTileCfg<LOGR, NG>;
    static constexpr int THREADS = K::THREADS;
    static constexpr int NMMA = THREADS / 128;
    static constexpr uint32_t TMEM_COLS = NMMA * 32 <= 32 ? 32 : (NMMA * 32 <= 64 ? 64 : (NMMA * 32 <= 128 ? 128 : 256));
    // The hi and lo A operands (THREADS rows x 64 bytes each) occupy exactly the
    // bytes of the FP32 exchange tile (16 NG columns x R rows x 8 bytes): the
    // tile is idle while a tensor-core DFT runs, so they share them.
    static constexpr size_t A_BYTES = (size_t)THREADS * kTcRowBytes;
    static constexpr size_t TILE_BYTES = K::SMEM_ELEMS * sizeof(float2);  // exchange tile + column twiddles
    static constexpr size_t OFF_TILE = 0;
    static constexpr size_t OFF_AHI = 0;
    static constexpr size_t OFF_ALO = A_BYTES;
    static constexpr size_t OFF_G = TILE_BYTES;                 // g_hi, g_lo (2 KB each)
    static constexpr size_t OFF_MISC = OFF_G + 2 * kTcGBytes;
    static constexpr size_t SMEM = OFF_MISC + 64;
    static_assert(2 * A_BYTES <= (size_t)NG * kCols * (1 << LOGR) * sizeof(float2),
                  "A operands must fit in the exchange tile (column twiddles follow it)");
    static constexpr int MINB = THREADS >= 1024 ? 1 : (THREADS >= 512 ? 2 : 4);
};

template <int LOGR, bool FIRST, bool BF16>
__global__ void __launch_bounds__(PassTcCfg<LOGR>::THREADS, PassTcCfg<LOGR>::MINB)
fft_pass_tc_kernel(const float2 *in, float2 *out, int logn, int logp, const float2 *__restrict__ tw,
                   const float2 *__restrict__ tw_lo, const float2 *__restrict__ tw_hi, int tw_split,
                   float in_im_sign, float out_re_scale, float out_im_scale, const uint4 *__restrict__ gtab,
                   uint32_t *err, LoadOps ops) {
    using C = PassTcCfg<LOGR>;
    extern __shared__ __align__(1024) uint8_t smem_tc[];
    uint64_t *bar = (uint64_t *)(smem_tc + C::OFF_MISC);
    uint32_t *s_taddr = (uint32_t *)(smem_tc + C::OFF_MISC + 8);
    int *s_abort = (int *)(smem_tc + C::OFF_MISC + 12);
    const int tid = threadIdx.x;

    // G operand parts: gtab holds [fp16 hi | fp16 lo | bf16 hi | bf16 lo], 2 KB each
    const uint4 *gsrc = gtab + (BF16 ? 2 : 0) * (kTcGBytes / 16);
    uint4 *gdst = (uint4 *)(smem_tc + C::OFF_G);
    for (int i = tid; i < 2 * kTcGBytes / 16; i += C::THREADS) gdst[i] = gsrc[i];
    if (tid < 32) tmem_alloc(s_taddr, C::TMEM_COLS);
    if (tid == 0) {
        mbar_init(bar, 1);
        *s_abort = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();

    TcState st;
    st.a_hi = smem_tc + C::OFF_AHI;
    st.a_lo = smem_tc + C::OFF_ALO;
    st.g_hi = smem_tc + C::OFF_G;
    st.g_lo = smem_tc + C::OFF_G + kTcGBytes;
    st.bar = bar;
    st.abort = s_abort;
    st.err = err;
    st.taddr = *s_taddr;
    st.parity = 0;
    st.nmma = C::NMMA;
    st.spin_limit = kTcSpinLimit;

    const int lognc = logn - LOGR;
    const uint64_t tile = blockIdx.x;
    const uint64_t tiles_per_row = (1ull << lognc) / (kCols * C::NG);
    const uint64_t b = tile / tiles_per_row;
    PassArgs a;
    a.src = in + (b << logn);
    a.dst = out + (b << logn);
    a.logn = logn;
    a.logp = logp;
    a.col0 = (uint32_t)((tile % tiles_per_row) * (kCols * C::NG));
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
    pass_tile<LOGR, C::NG, FIRST>(a, (float2 *)(smem_tc + C::OFF_TILE), DftTc<BF16>{&st});

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

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

template <int LOGR>
static void pass_tc_describe(PassDesc &d, bool first, bool bf16) {
    using C = PassTcCfg<LOGR>;
    if (first)
        d.fn = bf16 ? (const void *)fft_pass_tc_kernel<LOGR, true, true> : (const void *)fft_pass_tc_kernel<LOGR, true, false>;
    else
        d.fn = bf16 ? (const void *)fft_pass_tc_kernel<LOGR, false, true>
                    : (const void *)fft_pass_tc_kernel<LOGR, false, false>;
    d.threads = C::THREADS;
    d.smem = C::SMEM;
    d.cols = kCols * C::NG;
    d.nseg = subcfg_segments<LOGR>(d.segs, 0);
    d.tw_entries = SubCfg<LOGR>::tw_entries();
    d.tc = true;
}

bool pass_tc_kernel_info(int logr, bool first, bool bf16, PassDesc &d) {
    d.logr = logr;
    switch (logr) {
        case 5: pass_tc_describe<5>(d, first, bf16); return true;
        case 6: pass_tc_describe<6>(d, first, bf16); return true;
        case 7: pass_tc_describe<7>(d, first, bf16); return true;
        case 8: pass_tc_describe<8>(d, first, bf16); return true;
        case 9: pass_tc_describe<9>(d, first, bf16); return true;
        default: return false;
    }
}

cudaError_t pass_tc_launch(const PassDesc &d, const float2 *in, float2 *out, uint64_t batch, int logn,
                           const float2 *tw_sub, const float2 *tw_lo, const float2 *tw_hi, int tw_split,
                           float in_im_sign, float out_re_scale, float out_im_scale, const void *gtab,
                           uint32_t *err, cudaStream_t stream, LoadOps ops) {
    const uint64_t tiles = (batch << (logn - d.logr)) / (uint64_t)d.cols;
    if (tiles == 0) return cudaSuccess;
    if (tiles > 0x7fffffffull) return cudaErrorInvalidConfiguration;
    int logp = d.logp;
    void *args[] = {(void *)&in,     (void *)&out,   (void *)&logn,      (void *)&logp,
                    (void *)&tw_sub, (void *)&tw_lo, (void *)&tw_hi,     (void *)&tw_split,
                    (void *)&in_im_sign, (void *)&out_re_scale, (void *)&out_im_scale, (void *)&gtab,
                    (void *)&err, (void *)&ops};
    return cudaLaunchKernel(d.fn, dim3((unsigned)tiles), dim3(d.threads), args, d.smem, stream);
}

// G = [[cos, -sin], [sin, cos]] parts in canonical K-major layout:
// out = [fp16 hi | fp16 lo | bf16 hi | bf16 lo], 2048 bytes each.
__global__ void tc_gtab_kernel(uint8_t *out) {
    const int i = threadIdx.x + blockIdx.x * blockDim.x;
    if (i >= 32 * 32) return;
    const int n = i / 32, k = i % 32;  // operand B is K-major: row n (output column), element k
    const int q = n & 15, e = k & 15;
    double sn, cs;
    sincospi(2.0 * (double)((q * e) & 15) / 16.0, &sn, &cs);
    double g;
    if (n < 16) g = (k < 16) ? cs : sn;
    else g = (k < 16) ? -sn : cs;
    const float gf = (float)g;
    const uint32_t off = tc_elem_offset(n, k);
    const __half h = __float2half_rn(gf);
    const __half l = __float2half_rn(gf - __half2float(h));
    const __nv_bfloat16 bh = __float2bfloat16_rn(gf);
    const __nv_bfloat16 bl = __float2bfloat16_rn(gf - __bfloat162float(bh));
    *(uint16_t *)(out + 0 * kTcGBytes + off) = __half_as_ushort(h);
    *(uint16_t *)(out + 1 * kTcGBytes + off) = __half_as_ushort(l);
    *(uint16_t *)(out + 2 * kTcGBytes + off) = __bfloat16_as_ushort(bh);
    *(uint16_t *)(out + 3 * kTcGBytes + off) = __bfloat16_as_ushort(bl);
}

cudaError_t tc_gtab_fill(void *out, cudaStream_t stream) {
    tc_gtab_kernel<<<4, 256, 0, stream>>>((uint8_t *)out);
    return cudaGetLastError();
}

}  // namespace gbfft
