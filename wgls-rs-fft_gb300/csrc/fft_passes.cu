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
// conflicts for every access pattern.  First passes of radix 2^9 / 2^10 may
// take 8 columns instead (CL = 3: 64-byte row segments, half the tile, two
// CTAs per SM where 16 columns fit one).  The first pass (p = 1) writes each
// column's R outputs contiguously; it stages them through shared memory
// (XOR-swizzled [column][row]) so that its HBM stores are fully coalesced too.
//
// Pre-twiddle: thread t of column j holds rows m = t + T e, and
//   W_{R p}^{m k} = W_{R p}^{t k} * W_{E p}^{e k}.
// The first factor is one lookup per thread; the second depends only on the
// column and e, so the CTA builds it once into a padded 16 x 17 shared table.
// Both come from two FP64-built tables (W_N^i for i < 2^s and W_N^{i 2^s}).
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>

#include "gbfft_internal.h"
#include "gbfft_plan.h"
#include "fft_tc.cuh"
#include "fft_tiles.cuh"

namespace gbfft {

// LE: log2 of the samples a thread holds (4: 64 registers; 5: radix-32
// sub-passes at 128 registers, one exchange fewer for radix 2^9 / 2^10).
// CL: log2 of the columns a CTA takes.
template <int LOGR, int LE = 4, int CL = kColsLog>
struct PassCfg : PassTileCfg<LOGR, 1, LE, CL> {
    using K = PassTileCfg<LOGR, 1, LE, CL>;
    static constexpr int REGS = LE == 4 ? 64 : 128;
    static constexpr int MINB = K::THREADS * REGS >= 65536 ? 1 : 65536 / (K::THREADS * REGS);
    static constexpr size_t SMEM = K::SMEM_ELEMS * sizeof(float2);
};

template <int LOGR, bool FIRST, int LE = 4, int CL = kColsLog>
__global__ void __launch_bounds__(PassCfg<LOGR, LE, CL>::THREADS, PassCfg<LOGR, LE, CL>::MINB)
fft_pass_kernel(const float2 *in, float2 *out, int logn, int logp, const float2 *__restrict__ tw,
                const float2 *__restrict__ tw_lo, const float2 *__restrict__ tw_hi, int tw_split,
                float in_im_sign, float out_re_scale, float out_im_scale, LoadOps ops) {
    extern __shared__ __align__(16) float2 smem_pass[];
    const int lognc = logn - LOGR;                     // log2 (columns per transform)
    const uint64_t tile = blockIdx.x;
    const uint64_t b = tile >> (lognc - CL);
    PassArgs a;
    a.src = in + (b << logn);
    a.dst = out + (b << logn);
    a.logn = logn;
    a.logp = logp;
    a.col0 = (uint32_t)(tile & ((1ull << (lognc - CL)) - 1)) << CL;
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
    pass_tile<LOGR, 1, FIRST, DftRegs, 0, -1, LE, CL>(a, smem_pass);
}

// Persistent variant: each CTA walks tiles blockIdx.x, +gridDim.x, ... and asks
// L2 for the next tile's R row segments (2^CL x 8 bytes each, one per thread)
// before computing the current one.
template <int LOGR, bool FIRST, int LE = 4, int CL = kColsLog>
__global__ void __launch_bounds__(PassCfg<LOGR, LE, CL>::THREADS, PassCfg<LOGR, LE, CL>::MINB)
fft_pass_persistent_kernel(const float2 *in, float2 *out, int logn, int logp, const float2 *__restrict__ tw,
                           const float2 *__restrict__ tw_lo, const float2 *__restrict__ tw_hi, int tw_split,
                           float in_im_sign, float out_re_scale, float out_im_scale, LoadOps ops,
                           uint64_t ntiles) {
    extern __shared__ __align__(16) float2 smem_pass[];
    constexpr int R = 1 << LOGR;
    const int lognc = logn - LOGR;
    const uint64_t tiles_per_row = 1ull << (lognc - CL);
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint64_t next = tile + gridDim.x;
        if (next < ntiles) {
            const float2 *nb = in + ((next / tiles_per_row) << logn) + ((next % tiles_per_row) << CL);
            for (int m = threadIdx.x; m < R; m += PassCfg<LOGR, LE, CL>::THREADS) prefetch_l2(nb + ((uint64_t)m << lognc));
        }
        const uint64_t b = tile / tiles_per_row;
        PassArgs a;
        a.src = in + (b << logn);
        a.dst = out + (b << logn);
        a.logn = logn;
        a.logp = logp;
        a.col0 = (uint32_t)((tile % tiles_per_row) << CL);
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
        pass_tile<LOGR, 1, FIRST, DftRegs, 0, -1, LE, CL>(a, smem_pass);
        __syncthreads();  // shared memory is reused by the next tile
    }
}

// First pass of radix 2^9 / 2^10 (N = 2^25, 2^26) whose input tile -- 8
// adjacent columns x R rows, R row segments of 64 bytes 2^(logn - LOGR) * 8
// bytes apart -- is brought into shared memory by the tensor memory
// accelerator: R / 256 tiled copies of a [256 rows][8 columns] box of a 3-D
// tensor map over the input (float32 elements: 2 N / R x R x batch), issued
// by one thread and completing on one mbarrier.  The LDG form issues R * 8 / 8
// loads of 8 bytes a CTA (32 a thread) and is held back by the global-load
// queue; here the SM issues four instructions a tile and the copy engine of
// the TMA generates the strided addresses.  The wait is bounded: on expiry
// the launch raises the error flag (GBFFT_ERR_TIMEOUT on the host), waits
// once more, bounded, for its copies and skips the tile.
constexpr int kTmaBoxRows = 256;
constexpr uint32_t kTmaSpinLimit = 1u << 20;

template <int LOGR, int LE>
struct PassTmaCfg {
    using C = PassCfg<LOGR, LE, 3>;
    static constexpr size_t OFF_BAR = (C::SMEM + 15) & ~(size_t)15;
    static constexpr size_t SMEM = OFF_BAR + 16;
    static constexpr uint32_t TILE_BYTES = (1u << LOGR) * 8u * (uint32_t)sizeof(float2);
};

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, int x, int y, int z,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(dst),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

template <int LOGR, int LE>
__global__ void __launch_bounds__(PassCfg<LOGR, LE, 3>::THREADS, PassCfg<LOGR, LE, 3>::MINB)
fft_pass_first_tma_kernel(const __grid_constant__ CUtensorMap map, float2 *out, int logn,
                          const float2 *__restrict__ tw, const float2 *__restrict__ tw_lo,
                          const float2 *__restrict__ tw_hi, int tw_split, float in_im_sign, LoadOps ops,
                          uint32_t *err) {
    using T = PassTmaCfg<LOGR, LE>;
    constexpr int R = 1 << LOGR;
    extern __shared__ __align__(1024) float2 smem_tma[];
    uint64_t *bar = (uint64_t *)((char *)smem_tma + T::OFF_BAR);
    int *s_fail = (int *)((char *)smem_tma + T::OFF_BAR + 8);
    const int lognc = logn - LOGR;
    const uint64_t tile = blockIdx.x;
    const uint64_t b = tile >> (lognc - 3);
    const uint32_t col0 = (uint32_t)(tile & ((1ull << (lognc - 3)) - 1)) << 3;
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        *s_fail = 0;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                     "r"(T::TILE_BYTES)
                     : "memory");
#pragma unroll
        for (int k = 0; k < R / kTmaBoxRows; ++k)
            tma_load_3d(smem_u32(smem_tma + k * kTmaBoxRows * 8), &map, (int)(2 * col0), k * kTmaBoxRows, (int)b,
                        smem_u32(bar));
    }
    uint32_t polls = 0;
    bool done = mbar_try_wait(bar, 0);
    while (!done && ++polls < kTmaSpinLimit) done = mbar_try_wait(bar, 0);
    if (!done) *s_fail = 1;
    __syncthreads();
    if (*s_fail) {
        if (threadIdx.x == 0) {
            atomicExch(err, 4u);
            for (uint32_t n = 0; n < kTmaSpinLimit && !mbar_try_wait(bar, 0); ++n) {
            }
        }
        __syncthreads();
        return;
    }
    PassArgs a;
    a.src = nullptr;
    a.dst = out + (b << logn);
    a.logn = logn;
    a.logp = 0;
    a.col0 = col0;
    a.tw_sub = tw;
    a.tw_lo = tw_lo;
    a.tw_hi = tw_hi;
    a.tw_split = tw_split;
    a.in_im = in_im_sign;
    a.out_re = 1.0f;
    a.out_im = 1.0f;
    a.coherent_load = false;
    a.row = (uint32_t)b;
    a.ops = ops;
    pass_tile<LOGR, 1, true, DftRegs, 0, -1, LE, 3, true>(a, smem_tma);
}

__device__ __forceinline__ void tma_prefetch_3d(const CUtensorMap *map, int x, int y, int z) {
    asm volatile("cp.async.bulk.prefetch.tensor.3d.L2.global.tile [%0, {%1, %2, %3}];" ::"l"((uint64_t)map), "r"(x),
                 "r"(y), "r"(z)
                 : "memory");
}

// Persistent form: each CTA walks tiles blockIdx.x, +gridDim.x, ...; while a
// tile is computed, the next tile's boxes are already being fetched into L2
// (one TMA prefetch instruction a box), so its tiled copies find them there.
// The mbarrier is re-armed every tile (phase = tile count & 1) after the CTA
// barrier that ends the previous tile's reads of the shared tile.
template <int LOGR, int LE>
__global__ void __launch_bounds__(PassCfg<LOGR, LE, 3>::THREADS, PassCfg<LOGR, LE, 3>::MINB)
fft_pass_first_tma_persistent_kernel(const __grid_constant__ CUtensorMap map, float2 *out, int logn,
                                     const float2 *__restrict__ tw, const float2 *__restrict__ tw_lo,
                                     const float2 *__restrict__ tw_hi, int tw_split, float in_im_sign, LoadOps ops,
                                     uint32_t *err, uint64_t ntiles) {
    using T = PassTmaCfg<LOGR, LE>;
    constexpr int R = 1 << LOGR;
    extern __shared__ __align__(1024) float2 smem_tma[];
    uint64_t *bar = (uint64_t *)((char *)smem_tma + T::OFF_BAR);
    int *s_fail = (int *)((char *)smem_tma + T::OFF_BAR + 8);
    const int lognc = logn - LOGR;
    const uint64_t per_row = 1ull << (lognc - 3);  // tiles a transform
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        *s_fail = 0;
    }
    __syncthreads();
    uint32_t phase = 0;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, phase ^= 1u) {
        const uint64_t b = tile / per_row;
        const uint32_t col0 = (uint32_t)(tile % per_row) << 3;
        if (threadIdx.x == 0) {
            // the previous tile's shared-memory writes (exchanges, output staging)
            // are ordered before the copies that overwrite the tile
            fence_proxy_async_smem();
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                         "r"(T::TILE_BYTES)
                         : "memory");
#pragma unroll
            for (int k = 0; k < R / kTmaBoxRows; ++k)
                tma_load_3d(smem_u32(smem_tma + k * kTmaBoxRows * 8), &map, (int)(2 * col0), k * kTmaBoxRows,
                            (int)b, smem_u32(bar));
            const uint64_t next = tile + gridDim.x;
            if (next < ntiles) {
#pragma unroll
                for (int k = 0; k < R / kTmaBoxRows; ++k)
                    tma_prefetch_3d(&map, (int)(2 * ((uint32_t)(next % per_row) << 3)), k * kTmaBoxRows,
                                    (int)(next / per_row));
            }
        }
        uint32_t polls = 0;
        bool done = mbar_try_wait(bar, phase);
        while (!done && ++polls < kTmaSpinLimit) done = mbar_try_wait(bar, phase);
        if (!done) *s_fail = 1;
        __syncthreads();
        if (*s_fail) {
            if (threadIdx.x == 0) {
                atomicExch(err, 4u);
                for (uint32_t n = 0; n < kTmaSpinLimit && !mbar_try_wait(bar, phase); ++n) {
                }
            }
            __syncthreads();
            return;
        }
        PassArgs a;
        a.src = nullptr;
        a.dst = out + (b << logn);
        a.logn = logn;
        a.logp = 0;
        a.col0 = col0;
        a.tw_sub = tw;
        a.tw_lo = tw_lo;
        a.tw_hi = tw_hi;
        a.tw_split = tw_split;
        a.in_im = in_im_sign;
        a.out_re = 1.0f;
        a.out_im = 1.0f;
        a.coherent_load = false;
        a.row = (uint32_t)b;
        a.ops = ops;
        pass_tile<LOGR, 1, true, DftRegs, 0, -1, LE, 3, true>(a, smem_tma);
        __syncthreads();  // every read of the shared tile is done before the next tile's copies
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            p = nullptr;
        }
        return (PFN_cuTensorMapEncodeTiled_v12000)p;
    }();
    return fn;
}

template <int LOGR, int LE = 4>
static void pass_describe(PassDesc &d, bool first) {
    using C = PassCfg<LOGR, LE>;
    d.fn = first ? (const void *)fft_pass_kernel<LOGR, true, LE> : (const void *)fft_pass_kernel<LOGR, false, LE>;
    d.fn_persistent = first ? (const void *)fft_pass_persistent_kernel<LOGR, true, LE>
                            : (const void *)fft_pass_persistent_kernel<LOGR, false, LE>;
    d.threads = C::THREADS;
    d.smem = C::SMEM;
    d.cols = C::COLS;
    d.nseg = subcfg_segments<LOGR, LE>(d.segs, 0);
    d.tw_entries = SubCfg<LOGR, LE>::tw_entries();
}

// First pass of 8 columns a CTA; tma: its input tile comes by the tensor
// memory accelerator, the LDG kernel kept as the form for inputs that are not
// 16-byte aligned.
template <int LOGR, int LE>
static void pass_describe_first8(PassDesc &d, bool tma) {
    using C = PassCfg<LOGR, LE, 3>;
    d.fn = (const void *)fft_pass_kernel<LOGR, true, LE, 3>;
    d.fn_persistent = (const void *)fft_pass_persistent_kernel<LOGR, true, LE, 3>;
    d.threads = C::THREADS;
    d.smem = C::SMEM;
    d.cols = C::COLS;
    d.nseg = subcfg_segments<LOGR, LE>(d.segs, 0);
    d.tw_entries = SubCfg<LOGR, LE>::tw_entries();
    if (tma) {
        d.fn_tma = (const void *)fft_pass_first_tma_kernel<LOGR, LE>;
        d.fn_tma_persistent = (const void *)fft_pass_first_tma_persistent_kernel<LOGR, LE>;
        d.smem_tma = PassTmaCfg<LOGR, LE>::SMEM;
    }
}

bool pass_kernel_info(int logr, bool first, PassDesc &d, int loge, int cols_log, bool tma) {
    d.logr = logr;
    if (tma && !(first && cols_log == 3)) return false;
    if (cols_log == 3) {  // first passes of radix 2^9 / 2^10 only
        if (!first) return false;
        switch (logr * 10 + loge) {
            case 94: pass_describe_first8<9, 4>(d, tma); return true;
            case 95: pass_describe_first8<9, 5>(d, tma); return true;
            case 104: pass_describe_first8<10, 4>(d, tma); return true;
            case 105: pass_describe_first8<10, 5>(d, tma); return true;
            default: return false;
        }
    }
    if (cols_log != kColsLog) return false;
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
    if (d.fn_tma && d.smem_tma > 48 * 1024) {
        e = cudaFuncSetAttribute(d.fn_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)d.smem_tma);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(d.fn_tma_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)d.smem_tma);
        if (e != cudaSuccess) return e;
    }
    if (d.fn_tma_persistent) {
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&d.tma_ctas_per_sm, d.fn_tma_persistent, d.threads,
                                                          d.smem_tma);
        if (e != cudaSuccess) return e;
    }
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
                        bool persistent, int sms, LoadOps ops, uint32_t *err) {
    uint64_t tiles = (batch << (logn - d.logr)) / (uint64_t)d.cols;
    if (tiles == 0) return cudaSuccess;
    // the 8-column first pass stores 16-byte pairs
    if (d.cols < kCols && ((uintptr_t)out & 15u)) return cudaErrorMisalignedAddress;
    int logp = d.logp;
    // tensor-map first pass: needs a 16-byte aligned input (the map's base
    // address), an error flag for its bounded wait, and the CUDA driver's encoder;
    // otherwise the LDG kernel runs
    PFN_cuTensorMapEncodeTiled_v12000 encode = d.fn_tma ? tensor_map_encoder() : nullptr;
    if (d.fn_tma && encode && err && ((uintptr_t)in & 15u) == 0 && tiles <= 0x7fffffffull && batch <= 0xffffffffull) {
        const int lognc = logn - d.logr;
        // dims (innermost first): 2 N / R floats (the row), R rows, batch
        const cuuint64_t dims[3] = {2ull << lognc, 1ull << d.logr, batch};
        const cuuint64_t strides[2] = {(2ull << lognc) * sizeof(float), (1ull << logn) * sizeof(float2)};
        const cuuint32_t box[3] = {16, (cuuint32_t)std::min(1 << d.logr, kTmaBoxRows), 1};
        const cuuint32_t estr[3] = {1, 1, 1};
        alignas(64) CUtensorMap map;
        if (encode(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void *)in, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS) {
            if (persistent && d.fn_tma_persistent && d.tma_ctas_per_sm > 0 && sms > 0) {
                const uint64_t grid = std::min<uint64_t>(tiles, (uint64_t)d.tma_ctas_per_sm * (uint64_t)sms);
                void *pargs[] = {(void *)&map,   (void *)&out,      (void *)&logn,       (void *)&tw_sub,
                                 (void *)&tw_lo, (void *)&tw_hi,    (void *)&tw_split,   (void *)&in_im_sign,
                                 (void *)&ops,   (void *)&err,      (void *)&tiles};
                return cudaLaunchKernel(d.fn_tma_persistent, dim3((unsigned)grid), dim3(d.threads), pargs,
                                        d.smem_tma, stream);
            }
            void *args[] = {(void *)&map,  (void *)&out,   (void *)&logn,     (void *)&tw_sub,     (void *)&tw_lo,
                            (void *)&tw_hi, (void *)&tw_split, (void *)&in_im_sign, (void *)&ops, (void *)&err};
            return cudaLaunchKernel(d.fn_tma, dim3((unsigned)tiles), dim3(d.threads), args, d.smem_tma, stream);
        }
    }
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
