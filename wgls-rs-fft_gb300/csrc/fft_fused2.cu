// Two global passes in ONE persistent launch, with the intermediate kept in
// L2 (N = 2^15 .. 2^20, FP32 form, out of place).
//
// The two-launch form (fft_passes.cu) writes every sample to HBM after the
// first pass and reads it back in the second: 32 bytes of DRAM traffic per
// sample.  Here the first-pass tiles of transform b and the second-pass tiles
// of transform b - LAG alternate in one work queue, so a transform's
// intermediate (N x 8 bytes, written into the output buffer with normal L2
// priority) is read back by the second pass a few microseconds after it was
// written, while it is still in GB300's 129 MB L2.  The second pass then
// rewrites the same lines in place (each of its tiles reads and writes the
// same samples), and only the final values reach HBM: DRAM traffic falls
// towards the 16 bytes per sample of a single pass.  The window of transforms
// between producer and consumer (LAG x N x 8 bytes) is bounded by the host to
// a few tens of MB.
//
// Queue (one atomicAdd per item):  P1(0..L-1) | P1(L) P2(0) | P1(L+1) P2(1) |
// ... | P2(B-L..B-1), each P1(b)/P2(b) being the T tiles of one pass of
// transform b.  A second-pass tile waits until all T first-pass tiles of its
// transform have published; those tiles sit earlier in the queue and are
// owned by running CTAs that never wait, so every wait ends.  Each wait is
// still bounded (spin_limit polls with __nanosleep); on expiry the kernel
// raises the context's error flag, every CTA stops taking items and the host
// reports GBFFT_ERR_TIMEOUT.  The last CTA to leave resets the counters, so
// the kernel needs no memset node before the next launch.
//
// The stage rule of both passes is the reference's Stockham stage
// (larsjoost/wgls-rs-fft src/shaders.rs:20-62) at radices R1 and R2, exactly
// as in the two-launch form; only the scheduling differs.
#include <algorithm>

#include "gbfft_internal.h"
#include "gbfft_plan.h"
#include "fft_tiles.cuh"

namespace gbfft {

template <int LOGR1, int LOGR2, int THREADS>
struct Fused2Cfg {
    static constexpr int NG1 = THREADS >> LOGR1;
    static constexpr int NG2 = THREADS >> LOGR2;
    static_assert(NG1 >= 1 && NG2 >= 1, "CTA narrower than a radix");
    static_assert(PassTileCfg<LOGR1, NG1>::THREADS == THREADS && PassTileCfg<LOGR2, NG2>::THREADS == THREADS,
                  "both passes must use every thread");
    static constexpr size_t E1 = PassTileCfg<LOGR1, NG1>::SMEM_ELEMS, E2 = PassTileCfg<LOGR2, NG2>::SMEM_ELEMS;
    static constexpr size_t SMEM = (E1 > E2 ? E1 : E2) * sizeof(float2);
    static constexpr int MINB = THREADS >= 1024 ? 1 : 1024 / THREADS;
};

struct Fused2Params {
    const float2 *in;
    float2 *out;
    uint32_t batch;
    uint32_t lag;     // min(LAG, batch)
    uint32_t nitems;  // 2 x tiles x batch
    int logn;
    const float2 *tw1, *tw2;  // sub-pass tables of the two radices
    const float2 *tw_lo, *tw_hi;
    int tw_split;
    float in_im, out_re, out_im;
    LoadOps ops;
    uint32_t *ctr;  // [0] next item, [1] CTAs finished, [2 + b] first-pass tiles of b published
    uint32_t *err;
    uint32_t spin_limit;
};

__device__ __forceinline__ uint32_t f2_ld_acquire(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Queue position -> (pass, transform, tile); T tiles per pass per transform.
template <uint32_t T>
__device__ __forceinline__ void fused2_item(const Fused2Params &P, uint32_t idx, bool &first, uint32_t &b,
                                            uint32_t &tile) {
    const uint32_t L = P.lag;
    const uint32_t pro = L * T;
    if (idx < pro) {
        first = true;
        b = idx / T;
        tile = idx % T;
        return;
    }
    idx -= pro;
    const uint32_t steady = (P.batch - L) * 2u * T;
    if (idx < steady) {
        const uint32_t g = idx / (2u * T), r = idx % (2u * T);
        first = r < T;
        b = first ? L + g : g;
        tile = first ? r : r - T;
        return;
    }
    idx -= steady;
    first = false;
    b = P.batch - L + idx / T;
    tile = idx % T;
}

// Next queue position, or past the end once the error flag is up.
__device__ __forceinline__ uint32_t fused2_claim(const Fused2Params &P) {
    return *(volatile uint32_t *)P.err != 0u ? 0xffffffffu : atomicAdd(P.ctr, 1u);
}

template <int LOGR1, int LOGR2, int THREADS>
__global__ void __launch_bounds__(THREADS, Fused2Cfg<LOGR1, LOGR2, THREADS>::MINB)
fft_fused2_kernel(Fused2Params P) {
    using C = Fused2Cfg<LOGR1, LOGR2, THREADS>;
    constexpr int LOGN = LOGR1 + LOGR2;
    constexpr uint32_t T = (1u << LOGN) / (16u * THREADS);
    extern __shared__ float2 smem_f2[];
    // Claimed queue positions, double-buffered: slot `par` holds the current
    // item, slot par ^ 1 receives the next claim while the tile runs.
    __shared__ uint32_t s_item[2];
    __shared__ int s_abort;
    if (threadIdx.x == 0) s_item[0] = fused2_claim(P);
    __syncthreads();
    for (uint32_t par = 0;; par ^= 1u) {
        const uint32_t idx = s_item[par];
        if (idx >= P.nitems) break;
        // Claim the following item now: its index is needed only when this
        // one is done, so the atomic's round trip overlaps the tile.  Claims
        // stay in queue order, so the oldest unfinished item is always some
        // CTA's current item and can proceed: every wait still ends.  (Slot
        // par ^ 1 was last read before the previous item's final barrier.)
        if (threadIdx.x == 0) s_item[par ^ 1u] = fused2_claim(P);
        bool first;
        uint32_t b, tile;
        fused2_item<T>(P, idx, first, b, tile);
        const uint64_t base = (uint64_t)b << LOGN;
        PassArgs a;
        a.logn = LOGN;
        a.tw_lo = P.tw_lo;
        a.tw_hi = P.tw_hi;
        a.tw_split = P.tw_split;
        a.row = b;
        if (first) {
            a.src = P.in + base;
            a.dst = P.out + base;
            a.logp = 0;
            a.col0 = tile * (uint32_t)(kCols * C::NG1);
            a.tw_sub = P.tw1;
            a.in_im = P.in_im;
            a.out_re = 1.0f;
            a.out_im = 1.0f;
            a.coherent_load = false;
            a.keep_l2 = true;
            a.ops = P.ops;
            pass_tile<LOGR1, C::NG1, true, DftRegs, LOGR1 + LOGR2, 0>(a, smem_f2);
        } else {
            if (threadIdx.x == 0) {
                uint32_t polls = 0;
                int abort = 0;
                while (f2_ld_acquire(P.ctr + 2 + b) < T) {
                    if (++polls > P.spin_limit) {
                        atomicExch(P.err, 1u);
                        abort = 1;
                        break;
                    }
                    __nanosleep(128);
                }
                s_abort = abort;
            }
            __syncthreads();
            if (s_abort) break;
            a.src = P.out + base;
            a.dst = P.out + base;
            a.logp = LOGR1;
            a.col0 = tile * (uint32_t)(kCols * C::NG2);
            a.tw_sub = P.tw2;
            a.in_im = 1.0f;
            a.out_re = P.out_re;
            a.out_im = P.out_im;
            a.coherent_load = true;
            a.ops = LoadOps{nullptr, 0u, 0.f, 0u};
            pass_tile<LOGR2, C::NG2, false, DftRegs, LOGR1 + LOGR2, LOGR1>(a, smem_f2);
        }
        __syncthreads();  // the tile's stores are issued; shared memory is free
        if (threadIdx.x == 0) {
            fused2_item<T>(P, idx, first, b, tile);  // recomputed: nothing stays live across the tile
            if (first) {
                // publish: the barrier ordered the CTA's stores before this fence
                __threadfence();
                atomicAdd(P.ctr + 2 + b, 1u);
            }
        }
    }
    // The last CTA to finish clears the counters for the next launch; every
    // other CTA has published all its work before it counts itself out.
    __shared__ int s_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(P.ctr + 1, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (s_last) {
        __threadfence();
        for (uint32_t i = threadIdx.x; i < 2u + P.batch; i += THREADS) P.ctr[i] = 0u;
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

template <int LOGR1, int LOGR2, int THREADS>
static void fused2_describe(Fused2Desc &d) {
    using C = Fused2Cfg<LOGR1, LOGR2, THREADS>;
    d.fn = (const void *)fft_fused2_kernel<LOGR1, LOGR2, THREADS>;
    d.threads = THREADS;
    d.smem = C::SMEM;
    d.logr1 = LOGR1;
    d.logr2 = LOGR2;
}

bool fused2_kernel_info(int logr1, int logr2, Fused2Desc &d) {
#define GBFFT_F2(A, B, T) \
    if (logr1 == A && logr2 == B) { fused2_describe<A, B, T>(d); return true; }
    GBFFT_F2(8, 7, 256)
    GBFFT_F2(8, 8, 256)
    GBFFT_F2(9, 8, 512)
    GBFFT_F2(9, 9, 512)
    GBFFT_F2(10, 9, 1024)
    GBFFT_F2(10, 10, 1024)
#undef GBFFT_F2
    return false;
}

cudaError_t fused2_prepare(Fused2Desc &d) {
    cudaError_t e = cudaSuccess;
    if (d.smem > 48 * 1024) {
        e = cudaFuncSetAttribute(d.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)d.smem);
        if (e != cudaSuccess) return e;
    }
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&d.ctas_per_sm, d.fn, d.threads, d.smem);
}

uint32_t fused2_lag(const Fused2Desc &d, int logn, uint64_t batch, int sms) {
    const uint64_t tiles = (1ull << logn) / (16ull * (uint64_t)d.threads);
    const uint64_t grid = (uint64_t)std::max(1, d.ctas_per_sm) * (uint64_t)std::max(1, sms);
    // enough queue between producer and consumer that consumers rarely wait
    uint64_t lag = (2 * grid + 2 * tiles - 1) / (2 * tiles);
    // ... but a window of intermediates that stays well inside L2
    const uint64_t cap = std::max<uint64_t>(1, kFused2WindowBytes / ((8ull << logn)));
    lag = std::min(std::max<uint64_t>(lag, 1), cap);
    return (uint32_t)std::min<uint64_t>(lag, batch);
}

cudaError_t fused2_launch(const Fused2Desc &d, const float2 *in, float2 *out, uint64_t batch, int logn,
                          const float2 *tw1, const float2 *tw2, const float2 *tw_lo, const float2 *tw_hi,
                          int tw_split, float in_im, float out_re, float out_im, LoadOps ops, uint32_t *ctr,
                          uint32_t *err, int sms, cudaStream_t stream) {
    Fused2Params P;
    P.in = in;
    P.out = out;
    P.batch = (uint32_t)batch;
    const uint32_t tiles = (uint32_t)((1ull << logn) / (16ull * (uint64_t)d.threads));  // per pass per transform
    P.lag = fused2_lag(d, logn, batch, sms);
    P.nitems = 2u * tiles * P.batch;
    P.logn = logn;
    P.tw1 = tw1;
    P.tw2 = tw2;
    P.tw_lo = tw_lo;
    P.tw_hi = tw_hi;
    P.tw_split = tw_split;
    P.in_im = in_im;
    P.out_re = out_re;
    P.out_im = out_im;
    P.ops = ops;
    P.ctr = ctr;
    P.err = err;
    P.spin_limit = 1u << 22;  // ~0.5 s of 128 ns polls; a healthy wait is a few microseconds
    const uint64_t grid = std::min<uint64_t>((uint64_t)P.nitems,
                                             (uint64_t)std::max(1, d.ctas_per_sm) * (uint64_t)std::max(1, sms));
    void *args[] = {(void *)&P};
    return cudaLaunchKernel(d.fn, dim3((unsigned)grid), dim3(d.threads), args, d.smem, stream);
}

}  // namespace gbfft
