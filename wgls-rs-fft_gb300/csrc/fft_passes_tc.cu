// Split-precision tensor-core forms of the multi-pass transform (N >= 2^15).
//
// Identical data flow to fft_passes.cu / fft_fused.cuh -- FP32 twiddles,
// FP32 shared-memory exchanges -- but every radix-16 butterfly set of a
// sub-pass runs on the tcgen05 tensor cores as D = A.G with hi/lo operands
// (FP16, BF16 or TF32) and FP32 accumulation in tensor memory (fft_tc.cuh).
// Radix 2/4/8 remainder sub-passes stay on the FP32 pipes.
//
//   fft_pass_tc_kernel<LOGR, FIRST, KIND>    one global pass per launch
//   fft_fused_tc_kernel<RA, RB, T, L, KIND>  both passes of a two-pass
//       transform in one persistent launch, the intermediate kept in L2
//       (the queue of fft_fused.cuh), so each sample crosses DRAM once.
//
// Per CTA: warp 0 allocates 32 TMEM columns per 128 threads (the D blocks),
// thread 0 initialises one mbarrier that tcgen05.commit arrives on, and the
// two 32 x 32 operand parts of G (hi/lo, precomputed in canonical layout) are
// copied into shared memory.  The persistent form does this once per CTA for
// its whole run.  Every completion wait is bounded: on expiry the kernel
// raises an error flag, stops issuing MMAs, waits (again bounded) for the
// MMAs it issued, frees its TMEM and finishes.
#include <algorithm>

#include "gbfft_internal.h"
#include "gbfft_plan.h"
#include "fft_tc.cuh"
#include "fft_fused.cuh"

namespace gbfft {

__host__ __device__ constexpr uint32_t tc_tmem_cols(int nmma) {
    return nmma * 32 <= 32 ? 32 : (nmma * 32 <= 64 ? 64 : (nmma * 32 <= 128 ? 128 : 256));
}

// Column groups per CTA: enough threads (>= 128) to fill one M = 128 MMA.
template <int LOGR>
constexpr int tc_groups() {
    return (kCols << (LOGR - 4)) >= 128 ? 1 : 128 / (kCols << (LOGR - 4));
}

// Shared memory of a tensor-core tile kernel: the item region (FP32 exchange
// tile + column twiddles; the A operand parts alias it while a tensor-core
// DFT runs -- every tc_dft16 waits for the tile's readers before writing A),
// then the G parts (two, three for BF16 x 6), then the mbarrier, TMEM address
// and abort flag.
template <int KIND, int THREADS, size_t TILE_BYTES, int RADIX = 16>
struct TcSmem {
    using Gm = TcGeom<KIND, RADIX>;
    static constexpr int RADIX_ = RADIX;
    static constexpr int NMMA = THREADS / 128;
    static_assert(THREADS % 128 == 0, "one M = 128 MMA per 128 threads");
    static constexpr uint32_t TMEM_COLS = tc_tmem_cols(NMMA * RADIX / 16);  // 2 RADIX columns per block
    static constexpr size_t A_BYTES = (size_t)THREADS * Gm::ROW_BYTES;
    static constexpr size_t A_ALL = Gm::PARTS * A_BYTES;
    static constexpr size_t REGION = ((A_ALL > TILE_BYTES ? A_ALL : TILE_BYTES) + 1023) & ~(size_t)1023;
    static constexpr size_t OFF_G = REGION;
    static constexpr size_t OFF_MISC = OFF_G + Gm::PARTS * (size_t)Gm::G_BYTES;
    static constexpr size_t SMEM = OFF_MISC + 64;
    // CTAs per SM that shared memory allows (228 KB per SM, 1 KB reserved per CTA)
    static constexpr int FIT = (int)((228u * 1024u) / (SMEM + 1024u));
};

// Per-CTA set-up: G parts into shared memory, TMEM, mbarrier.
template <int KIND, class L>
__device__ __forceinline__ void tc_cta_setup(uint8_t *smem, const uint4 *__restrict__ gtab, uint32_t *err,
                                             TcState &st) {
    using Gm = typename L::Gm;
    uint64_t *bar = (uint64_t *)(smem + L::OFF_MISC);
    uint32_t *s_taddr = (uint32_t *)(smem + L::OFF_MISC + 8);
    int *s_abort = (int *)(smem + L::OFF_MISC + 12);
    const int tid = threadIdx.x;
    const uint4 *gsrc = gtab + Gm::GTAB_OFF / 16;
    uint4 *gdst = (uint4 *)(smem + L::OFF_G);
    for (int i = tid; i < Gm::PARTS * Gm::G_BYTES / 16; i += blockDim.x) gdst[i] = gsrc[i];
    if (tid < 32) tmem_alloc(s_taddr, L::TMEM_COLS);
    if (tid == 0) {
        mbar_init(bar, 1);
        *s_abort = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    tc_state_parts<KIND, L::RADIX_>(st, smem, L::A_BYTES, smem + L::OFF_G);
    st.bar = bar;
    st.abort = s_abort;
    st.err = err;
    st.taddr = *s_taddr;
    st.parity = 0;
    st.nmma = L::NMMA;
    st.spin_limit = kTcSpinLimit;
}

// Per-CTA tear-down: after an aborted wait let the issued MMAs finish, then
// free TMEM.
template <class L>
__device__ __forceinline__ void tc_cta_teardown(const TcState &st) {
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x == 0 && *st.abort) {
        for (uint32_t polls = 0; polls < kTcSpinLimit && !mbar_try_wait(st.bar, st.parity ^ 1u); ++polls) {
        }
    }
    __syncthreads();
    tc_fence_after();
    if (threadIdx.x < 32) tmem_dealloc(st.taddr, L::TMEM_COLS);
}

// ---------------------------------------------------------------------------
// one pass per launch
// ---------------------------------------------------------------------------

template <int LOGR, int KIND>
struct PassTcCfg {
    static constexpr int NG = tc_groups<LOGR>();
    using K = PassTileCfg<LOGR, NG>;
    static constexpr int THREADS = K::THREADS;
    using L = TcSmem<KIND, THREADS, K::SMEM_ELEMS * sizeof(float2)>;
    static constexpr int MINB0 = THREADS >= 1024 ? 1 : (THREADS >= 512 ? 2 : 4);
    static constexpr int MINB = L::FIT < MINB0 ? (L::FIT < 1 ? 1 : L::FIT) : MINB0;
};

template <int LOGR, bool FIRST, int KIND>
__global__ void __launch_bounds__(PassTcCfg<LOGR, KIND>::THREADS, PassTcCfg<LOGR, KIND>::MINB)
fft_pass_tc_kernel(const float2 *in, float2 *out, int logn, int logp, const float2 *__restrict__ tw,
                   const float2 *__restrict__ tw_lo, const float2 *__restrict__ tw_hi, int tw_split,
                   float in_im_sign, float out_re_scale, float out_im_scale, const uint4 *__restrict__ gtab,
                   uint32_t *err, LoadOps ops) {
    using C = PassTcCfg<LOGR, KIND>;
    extern __shared__ __align__(1024) uint8_t smem_tc[];
    TcState st;
    tc_cta_setup<KIND, typename C::L>(smem_tc, gtab, err, st);

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
    pass_tile<LOGR, C::NG, FIRST>(a, (float2 *)smem_tc, DftTc<KIND>{&st});

    tc_cta_teardown<typename C::L>(st);
}

// ---------------------------------------------------------------------------
// both passes of a two-pass transform in one persistent launch
// ---------------------------------------------------------------------------

// LE = 5: 32-sample tiles whose radix-32 sub-passes run on the tensor cores
// (radix-32 G, 64 TMEM columns per 128 threads); 16-bit kinds only.
template <int LOGRA, int LOGRB, int THREADS, int LOGN, int KIND, int LE = 4>
struct FusedTcCfg {
    using F = FusedCfg<LOGRA, LOGRB, THREADS, LOGN, 0, LE>;
    using L = TcSmem<KIND, THREADS, F::SMEM, LE == 5 ? 32 : 16>;
    static constexpr int MINB = L::FIT < F::MINB ? (L::FIT < 1 ? 1 : L::FIT) : F::MINB;
};

template <int LOGRA, int LOGRB, int THREADS, int LOGN, int KIND, int LE = 4>
__global__ void __launch_bounds__(THREADS, (FusedTcCfg<LOGRA, LOGRB, THREADS, LOGN, KIND, LE>::MINB))
fft_fused_tc_kernel(FusedParams P) {
    using C = FusedTcCfg<LOGRA, LOGRB, THREADS, LOGN, KIND, LE>;
    extern __shared__ __align__(1024) uint8_t smem_ftc[];
    TcState st;
    tc_cta_setup<KIND, typename C::L>(smem_ftc, P.gtab, P.err, st);
    if constexpr (LE == 5)
        fused_loop<LOGRA, LOGRB, THREADS, LOGN, 0, 5>(P, (float2 *)smem_ftc, DftTc32<KIND>{&st});
    else
        fused_loop<LOGRA, LOGRB, THREADS, LOGN, 0>(P, (float2 *)smem_ftc, DftTc<KIND>{&st});
    fused_finish<THREADS>(P);
    tc_cta_teardown<typename C::L>(st);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

template <int LOGR, int KIND>
static void pass_tc_describe(PassDesc &d, bool first) {
    using C = PassTcCfg<LOGR, KIND>;
    d.fn = first ? (const void *)fft_pass_tc_kernel<LOGR, true, KIND> : (const void *)fft_pass_tc_kernel<LOGR, false, KIND>;
    d.threads = C::THREADS;
    d.smem = C::L::SMEM;
    d.cols = kCols * C::NG;
    d.nseg = subcfg_segments<LOGR>(d.segs, 0);
    d.tw_entries = SubCfg<LOGR>::tw_entries();
    d.tc = true;
}

template <int KIND>
static bool pass_tc_info_kind(int logr, bool first, PassDesc &d) {
    switch (logr) {
        case 5: pass_tc_describe<5, KIND>(d, first); return true;
        case 6: pass_tc_describe<6, KIND>(d, first); return true;
        case 7: pass_tc_describe<7, KIND>(d, first); return true;
        case 8: pass_tc_describe<8, KIND>(d, first); return true;
        case 9: pass_tc_describe<9, KIND>(d, first); return true;
        default: return false;
    }
}

bool pass_tc_kernel_info(int logr, bool first, int precision, PassDesc &d) {
    d.logr = logr;
    switch (tc_kind_of_precision(precision)) {
        case kTcBF16: return pass_tc_info_kind<kTcBF16>(logr, first, d);
        case kTcBF16X6: return pass_tc_info_kind<kTcBF16X6>(logr, first, d);
        case kTcTF32: return pass_tc_info_kind<kTcTF32>(logr, first, d);
        default: return pass_tc_info_kind<kTcF16>(logr, first, d);
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

template <int LOGRA, int LOGRB, int THREADS, int KIND, int LE = 4>
static void fused_tc_describe(FusedDesc &d) {
    constexpr int LOGN = LOGRA + LOGRB;
    using C = FusedTcCfg<LOGRA, LOGRB, THREADS, LOGN, KIND, LE>;
    using F = typename C::F;
    d.fn = (const void *)fft_fused_tc_kernel<LOGRA, LOGRB, THREADS, LOGN, KIND, LE>;
    d.loge = LE;
    d.threads = THREADS;
    d.smem = C::L::SMEM;
    d.logra = LOGRA;
    d.logrb = LOGRB;
    d.logpa = 0;
    d.logn = LOGN;
    d.groups_per_transform = F::GPT;
    d.tiles_per_group = F::T;
    d.group_samples = F::GROUP_SAMPLES;
    d.tmem_cols = (int)C::L::TMEM_COLS;
}

template <int KIND>
static bool fused_tc_info_kind(int logr1, int logr2, FusedDesc &d, int loge) {
    if (loge == 5) {
        if constexpr (KIND == kTcTF32 || KIND == kTcBF16X6) {
            return false;
        } else {
#define GBFFT_FTC5(A, B) \
    if (logr1 == A && logr2 == B) { fused_tc_describe<A, B, 256, KIND, 5>(d); return true; }
            GBFFT_FTC5(8, 7)
            GBFFT_FTC5(8, 8)
            GBFFT_FTC5(9, 8)
            GBFFT_FTC5(9, 9)
#undef GBFFT_FTC5
            return false;
        }
    }
    if (loge != 4) return false;
#define GBFFT_FTC(A, B, T) \
    if (logr1 == A && logr2 == B) { fused_tc_describe<A, B, T, KIND>(d); return true; }
    GBFFT_FTC(8, 7, 256)
    GBFFT_FTC(8, 8, 256)
    GBFFT_FTC(9, 8, 512)
    GBFFT_FTC(9, 9, 512)
#undef GBFFT_FTC
    return false;
}

bool fused_tc_kernel_info(int logr1, int logr2, int precision, FusedDesc &d, int loge) {
    switch (tc_kind_of_precision(precision)) {
        case kTcBF16: return fused_tc_info_kind<kTcBF16>(logr1, logr2, d, loge);
        case kTcBF16X6: return fused_tc_info_kind<kTcBF16X6>(logr1, logr2, d, loge);
        case kTcTF32: return fused_tc_info_kind<kTcTF32>(logr1, logr2, d, loge);
        default: return fused_tc_info_kind<kTcF16>(logr1, logr2, d, loge);
    }
}

// G = [[cos, -sin], [sin, cos]] parts in canonical K-major layout:
// out = [fp16 hi | fp16 lo | bf16 hi | bf16 lo] (2048 bytes each), then
// [tf32 hi | tf32 lo] (4096 bytes each).  The TF32 parts come from the FP64
// value: hi = the FP32 value with its 13 low mantissa bits cleared, lo = the
// rest rounded to the nearest TF32 value.  The three BF16 parts of the BF16 x 6
// kind, [hi | lo | mid] (2048 bytes each), follow the radix-32 parts at byte
// 49152: hi = RN(g), mid = RN(g - hi), lo = RN(g - hi - mid), from the FP64 g.
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
    const uint32_t off = TcGeom<kTcF16>::elem_offset(n, k);
    const __half h = __float2half_rn(gf);
    const __half l = __float2half_rn(gf - __half2float(h));
    const __nv_bfloat16 bh = __float2bfloat16_rn(gf);
    const __nv_bfloat16 bl = __float2bfloat16_rn(gf - __bfloat162float(bh));
    *(uint16_t *)(out + 0 * 2048 + off) = __half_as_ushort(h);
    *(uint16_t *)(out + 1 * 2048 + off) = __half_as_ushort(l);
    *(uint16_t *)(out + 2 * 2048 + off) = __bfloat16_as_ushort(bh);
    *(uint16_t *)(out + 3 * 2048 + off) = __bfloat16_as_ushort(bl);
    const uint32_t th = __float_as_uint(gf) & 0xFFFFE000u;
    uint32_t tl = __float_as_uint((float)(g - (double)__uint_as_float(th)));
    tl = (tl + 0x1000u) & 0xFFFFE000u;  // to nearest TF32 (ties away from zero)
    const uint32_t off32 = TcGeom<kTcTF32>::elem_offset(n, k);
    *(uint32_t *)(out + 8192 + off32) = th;
    *(uint32_t *)(out + 8192 + 4096 + off32) = tl;
    const __nv_bfloat16 x6h = __double2bfloat16(g);
    const double r1 = g - (double)__bfloat162float(x6h);
    const __nv_bfloat16 x6m = __double2bfloat16(r1);
    const __nv_bfloat16 x6l = __double2bfloat16(r1 - (double)__bfloat162float(x6m));
    uint8_t *x6 = out + TcGeom<kTcBF16X6>::GTAB_OFF;
    *(uint16_t *)(x6 + 0 * 2048 + off) = __bfloat16_as_ushort(x6h);
    *(uint16_t *)(x6 + 1 * 2048 + off) = __bfloat16_as_ushort(x6l);
    *(uint16_t *)(x6 + 2 * 2048 + off) = __bfloat16_as_ushort(x6m);
}

// Radix-32 G (64 x 64) parts for the 32-sample tiles, after the radix-16 ones:
// [fp16 hi | fp16 lo | bf16 hi | bf16 lo], 8192 bytes each, from byte 16384.
__global__ void tc_gtab32_kernel(uint8_t *out) {
    const int i = threadIdx.x + blockIdx.x * blockDim.x;
    if (i >= 64 * 64) return;
    const int n = i / 64, k = i % 64;  // operand B is K-major: row n (output column), element k
    const int q = n & 31, e = k & 31;
    double sn, cs;
    sincospi(2.0 * (double)((q * e) & 31) / 32.0, &sn, &cs);
    double g;
    if (n < 32) g = (k < 32) ? cs : sn;
    else g = (k < 32) ? -sn : cs;
    const float gf = (float)g;
    const uint32_t off = TcGeom<kTcF16, 32>::elem_offset(n, k);
    const __half h = __float2half_rn(gf);
    const __half l = __float2half_rn(gf - __half2float(h));
    const __nv_bfloat16 bh = __float2bfloat16_rn(gf);
    const __nv_bfloat16 bl = __float2bfloat16_rn(gf - __bfloat162float(bh));
    uint8_t *base = out + TcGeom<kTcF16, 32>::GTAB_OFF;
    *(uint16_t *)(base + 0 * 8192 + off) = __half_as_ushort(h);
    *(uint16_t *)(base + 1 * 8192 + off) = __half_as_ushort(l);
    *(uint16_t *)(base + 2 * 8192 + off) = __bfloat16_as_ushort(bh);
    *(uint16_t *)(base + 3 * 8192 + off) = __bfloat16_as_ushort(bl);
}

cudaError_t tc_gtab_fill(void *out, cudaStream_t stream) {
    tc_gtab_kernel<<<4, 256, 0, stream>>>((uint8_t *)out);
    tc_gtab32_kernel<<<16, 256, 0, stream>>>((uint8_t *)out);
    return cudaGetLastError();
}

}  // namespace gbfft
