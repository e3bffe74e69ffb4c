// Two consecutive global passes (A, then B) in ONE persistent launch, with
// the intermediate kept in L2.
//
// Used for both passes of a two-pass transform (N = 2^15 .. 2^20, A = the
// first pass) and for the last two passes of a three-pass transform with
// radices (R1, R, R) (N = 2^21 .. 2^26, A = the second pass).  The passes
// split into independent GROUPS: a group's B tiles read only what its A tiles
// wrote.
//   * two passes: a group is one transform (T = N / (16 x THREADS) tiles each);
//   * last two of three: with W = 16 columns per tile, the B tiles of columns
//     {u R1 + g W + c} (u < R, c < W) read, by the Stockham stage rule
//     (larsjoost/wgls-rs-fft src/shaders.rs:20-62: pass p reads j + m N/R and
//     writes (j/p) R p + (j mod p) + q p), exactly what the A tiles of columns
//     {m R1 + g W + c} (m < R) wrote; R tiles of each pass and 16 R^2 samples
//     (8 MB at R = 256) per group, R1 / W groups per transform.
// The queue alternates the A tiles of group x with the B tiles of group
// x - LAG: P_A(0..L-1) | P_A(L) P_B(0) | P_A(L+1) P_B(1) | ... | P_B(G-L..G-1).
// A's output goes into the output buffer with normal L2 priority
// (st.global.cg); B reads it back with L1-bypassing loads a few microseconds
// later and rewrites the same samples in place (each B tile reads and writes
// the same samples), so the intermediate is served from GB300's 129 MB L2
// and only the final values reach HBM.  The host bounds LAG x (group bytes)
// to a few tens of MB.
//
// Every CTA claims queue positions with one atomicAdd (the next claim is made
// while the current tile runs).  A B tile waits until all T A tiles of its
// group have published; those sit earlier in the queue and claims are made in
// queue order, so the oldest unfinished tile is always some CTA's current tile
// and can proceed: every wait ends.  Each wait is still bounded (spin_limit
// polls with __nanosleep); on expiry the kernel raises the context's error
// flag, every CTA stops taking items and the host reports GBFFT_ERR_TIMEOUT.
// Producers publish after the CTA barrier with one thread's __threadfence +
// atomicAdd; the consumer polls with ld.acquire.gpu.  The last CTA to leave
// zeroes the counters, so no memset precedes a launch.
#pragma once
#include "fft_tiles.cuh"

namespace gbfft {

// LOGPA: log2 of the product of the radices before pass A (0: A is the first
// pass).  Both passes use every thread; for LOGPA > 0 both radices are equal.
// LE: log2 of the samples a thread holds (4: 64 registers a thread; 5: radix-32
// sub-passes, 128 registers a thread).
template <int LOGRA, int LOGRB, int THREADS, int LOGN, int LOGPA, int LE = 4>
struct FusedCfg {
    static constexpr int NGA = (THREADS << (LE - 4)) >> LOGRA;
    static constexpr int NGB = (THREADS << (LE - 4)) >> LOGRB;
    static_assert(NGA >= 1 && NGB >= 1, "CTA narrower than a radix");
    static_assert(PassTileCfg<LOGRA, NGA, LE>::THREADS == THREADS && PassTileCfg<LOGRB, NGB, LE>::THREADS == THREADS,
                  "both passes must use every thread");
    static_assert(LOGPA == 0 ? LOGN == LOGRA + LOGRB : (LOGRA == LOGRB && NGA == 1 && LOGPA >= 4),
                  "two-pass transform, or the last two passes (R1, R, R) of three with one column group a tile");
    static constexpr bool FIRST_A = LOGPA == 0;
    static constexpr int LOGPB = LOGPA + LOGRA;
    // groups per transform and tiles of each pass per group
    static constexpr uint32_t GPT = FIRST_A ? 1u : (1u << LOGPA) / kCols;
    static constexpr uint32_t T = FIRST_A ? (1u << LOGN) / ((1u << LE) * THREADS) : (1u << LOGRB);
    static constexpr uint64_t GROUP_SAMPLES = (uint64_t)T * (1u << LE) * THREADS;
    static constexpr size_t EA = PassTileCfg<LOGRA, NGA, LE>::SMEM_ELEMS, EB = PassTileCfg<LOGRB, NGB, LE>::SMEM_ELEMS;
    static constexpr size_t SMEM = (EA > EB ? EA : EB) * sizeof(float2);
    static constexpr int REGS = LE == 4 ? 64 : 128;
    static constexpr int MINB = THREADS * REGS >= 65536 ? 1 : 65536 / (THREADS * REGS);
};

struct FusedParams {
    const float2 *in;   // input of pass A (the caller's input, or the first pass's output)
    float2 *out;
    uint32_t batch;
    uint32_t ngroups;   // batch x groups per transform
    uint32_t lag;       // min(LAG, ngroups)
    uint32_t nitems;    // 2 x T x ngroups
    const float2 *tw_a, *tw_b;  // sub-pass tables of the two radices
    const float2 *tw_lo, *tw_hi;
    float in_im, out_re, out_im;
    LoadOps ops;        // applied by pass A when it is the first pass
    uint32_t *ctr;      // [0] next item, [1] CTAs finished, [2 + group] A tiles published
    uint32_t *err;
    uint32_t spin_limit;
    const uint4 *gtab;  // split forms: the G operand table (fft_passes_tc.cu)
    // Two-pass transforms only: when set, pass A reads transform b from
    // tab_in[b] and pass B writes it to tab_out[b] (the addresses of the
    // caller's host rows, which the GPU reaches through the host's page
    // tables); `out` then holds only the intermediate.  Null otherwise.
    const uint64_t *tab_in;
    const uint64_t *tab_out;
};

__device__ __forceinline__ uint32_t fused_ld_acquire(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Queue position -> (pass A?, group, tile within the group's pass).
template <uint32_t T>
__device__ __forceinline__ void fused_item(const FusedParams &P, uint32_t idx, bool &is_a, uint32_t &grp,
                                           uint32_t &tile) {
    const uint32_t L = P.lag;
    const uint32_t pro = L * T;
    if (idx < pro) {
        is_a = true;
        grp = idx / T;
        tile = idx % T;
        return;
    }
    idx -= pro;
    const uint32_t steady = (P.ngroups - L) * 2u * T;
    if (idx < steady) {
        const uint32_t g = idx / (2u * T), r = idx % (2u * T);
        is_a = r < T;
        grp = is_a ? L + g : g;
        tile = is_a ? r : r - T;
        return;
    }
    idx -= steady;
    is_a = false;
    grp = P.ngroups - L + idx / T;
    tile = idx % T;
}

// Next queue position, or past the end once the error flag is up.
__device__ __forceinline__ uint32_t fused_claim(const FusedParams &P) {
    return *(volatile uint32_t *)P.err != 0u ? 0xffffffffu : atomicAdd(P.ctr, 1u);
}

// The queue loop of one CTA: claims items until the queue (or the launch,
// after an error) is exhausted.  `Eng` runs the radix-16 butterflies (FP32
// registers, or the tensor cores for the split forms); every thread of the
// CTA takes part in every item.
template <int LOGRA, int LOGRB, int THREADS, int LOGN, int LOGPA, int LE = 4, class Eng>
__device__ __forceinline__ void fused_loop(const FusedParams &P, float2 *smem_f, Eng eng) {
    using C = FusedCfg<LOGRA, LOGRB, THREADS, LOGN, LOGPA, LE>;
    constexpr uint32_t T = C::T, GPT = C::GPT;
    // Claimed queue positions, double-buffered: slot `par` holds the current
    // item, slot par ^ 1 receives the next claim while the tile runs.
    __shared__ uint32_t s_item[2];
    __shared__ int s_abort;
    if (threadIdx.x == 0) s_item[0] = fused_claim(P);
    __syncthreads();
    for (uint32_t par = 0;; par ^= 1u) {
        const uint32_t idx = s_item[par];
        if (idx >= P.nitems) break;
        // Claim the following item now: its index is needed only when this
        // one is done, so the atomic's round trip overlaps the tile.  (Slot
        // par ^ 1 was last read before the previous item's final barrier.)
        if (threadIdx.x == 0) s_item[par ^ 1u] = fused_claim(P);
        bool is_a;
        uint32_t grp, tile;
        fused_item<T>(P, idx, is_a, grp, tile);
        const uint32_t b = grp / GPT, g = grp % GPT;
        const uint64_t base = (uint64_t)b << LOGN;
        PassArgs a;
        a.logn = LOGN;
        a.tw_lo = P.tw_lo;
        a.tw_hi = P.tw_hi;
        a.tw_split = (LOGN + 1) / 2;
        a.row = b;
        if (is_a) {
            a.src = (C::FIRST_A && P.tab_in) ? (const float2 *)P.tab_in[b] : P.in + base;
            a.dst = P.out + base;
            a.logp = LOGPA;
            // two passes: tiles in column order; last two of three: column
            // blocks m GPT + g of the group
            a.col0 = C::FIRST_A ? tile * (uint32_t)(kCols * C::NGA) : (tile * GPT + g) * (uint32_t)kCols;
            a.tw_sub = P.tw_a;
            a.in_im = C::FIRST_A ? P.in_im : 1.0f;
            a.out_re = 1.0f;
            a.out_im = 1.0f;
            a.coherent_load = false;
            a.keep_l2 = true;
            a.ops = C::FIRST_A ? P.ops : LoadOps{nullptr, 0u, 0.f, 0u};
            pass_tile<LOGRA, C::NGA, C::FIRST_A, Eng, LOGN, LOGPA, LE>(a, smem_f, eng);
        } else {
            if (threadIdx.x == 0) {
                uint32_t polls = 0;
                int abort = 0;
                while (fused_ld_acquire(P.ctr + 2 + grp) < T) {
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
            a.dst = (C::FIRST_A && P.tab_out) ? (float2 *)P.tab_out[b] : P.out + base;
            a.logp = C::LOGPB;
            a.col0 = C::FIRST_A ? tile * (uint32_t)(kCols * C::NGB) : (tile * GPT + g) * (uint32_t)kCols;
            a.tw_sub = P.tw_b;
            a.in_im = 1.0f;
            a.out_re = P.out_re;
            a.out_im = P.out_im;
            a.coherent_load = true;
            a.ops = LoadOps{nullptr, 0u, 0.f, 0u};
            pass_tile<LOGRB, C::NGB, false, Eng, LOGN, C::LOGPB, LE>(a, smem_f, eng);
        }
        __syncthreads();  // the tile's stores are issued; shared memory is free
        if (threadIdx.x == 0) {
            fused_item<T>(P, idx, is_a, grp, tile);  // recomputed: nothing stays live across the tile
            if (is_a) {
                // publish: the barrier ordered the CTA's stores before this fence
                __threadfence();
                atomicAdd(P.ctr + 2 + grp, 1u);
            }
        }
    }
}

// The last CTA to finish clears the counters for the next launch; every
// other CTA has published all its work before it counts itself out.
template <int THREADS>
__device__ __forceinline__ void fused_finish(const FusedParams &P) {
    __shared__ int s_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(P.ctr + 1, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (s_last) {
        __threadfence();
        for (uint32_t i = threadIdx.x; i < 2u + P.ngroups; i += THREADS) P.ctr[i] = 0u;
    }
}

template <int LOGRA, int LOGRB, int THREADS, int LOGN, int LOGPA, int LE = 4>
__global__ void __launch_bounds__(THREADS, (FusedCfg<LOGRA, LOGRB, THREADS, LOGN, LOGPA, LE>::MINB))
fft_fused_kernel(FusedParams P) {
    extern __shared__ float2 smem_f[];
    // packed FP32 butterflies (2^16: 226 -> 232 GSa/s), except for pairs with a
    // radix-2^10 pass (32 x 32 sub-passes at 128 registers), where the scalar
    // ones measured faster (2^19: 152.4 against 149.8 GSa/s)
    using Eng = std::conditional_t<(LOGRA >= 10 || LOGRB >= 10), DftRegsScalar, DftRegs>;
    fused_loop<LOGRA, LOGRB, THREADS, LOGN, LOGPA, LE>(P, smem_f, Eng{});
    fused_finish<THREADS>(P);
}

template <int LOGRA, int LOGRB, int THREADS, int LOGN, int LOGPA, int LE = 4>
inline void fused_describe(FusedDesc &d) {
    using C = FusedCfg<LOGRA, LOGRB, THREADS, LOGN, LOGPA, LE>;
    d.fn = (const void *)fft_fused_kernel<LOGRA, LOGRB, THREADS, LOGN, LOGPA, LE>;
    d.loge = LE;
    d.threads = THREADS;
    d.smem = C::SMEM;
    d.logra = LOGRA;
    d.logrb = LOGRB;
    d.logpa = LOGPA;
    d.logn = LOGN;
    d.groups_per_transform = C::GPT;
    d.tiles_per_group = C::T;
    d.group_samples = C::GROUP_SAMPLES;
}

}  // namespace gbfft
