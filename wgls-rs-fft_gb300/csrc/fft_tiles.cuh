// Tile bodies shared by the uniform kernels (fft_rows.cu, fft_passes.cu) and
// the ragged persistent kernel (fft_ragged.cu).
//
//   rows_tile<LOGN, G>  -- G whole transforms of length 2^LOGN, one HBM read and
//                          one HBM write per sample (the single-pass form).
//   pass_tile<LOGR, NG, FIRST>
//                       -- NG groups of 16 (or 2^CL) adjacent columns of one
//                          global Stockham pass of radix R = 2^LOGR (multi-pass form).
// Both use all G*T (resp. NG*2^CL*T) threads of the CTA and __syncthreads().
#pragma once
#include "fft_smem.cuh"

namespace gbfft {

constexpr int kColsLog = 4;
constexpr int kCols = 1 << kColsLog;

// Exchange-buffer position of element a after a sub-pass with p = 2^logp: for
// p < 2^LE the low LE bits are XORed with (a >> LE) << logp (a bijection), which
// spreads the stride-p writes over the banks.
template <int LE = 4>
GBFFT_HD int swz(int a, int logp) {
    return logp < LE ? (a ^ (((a >> LE) << logp) & ((1 << LE) - 1))) : a;
}

// Sub-passes 1..NSUB-1 of a row transform held as v[] by thread t, exchanged
// through buf (XOR-swizzled positions).
template <int LOGN, int I, int LE = 4, bool DONE = (I >= SubCfg<LOGN, LE>::NSUB)>
struct RowsChain {
    using C = SubCfg<LOGN, LE>;
    template <class Eng>
    __device__ __forceinline__ static void run(float2 (&v)[C::E], int t, float2 *buf, const float2 *tw, Eng &eng) {
        constexpr int PR = C::logr(I - 1), PP = C::logp(I - 1);  // previous sub-pass
        if (I > 1) __syncthreads();  // readers of the previous exchange are done
#pragma unroll
        for (int b = 0; b < (C::E >> PR); ++b)
#pragma unroll
            for (int q = 0; q < (1 << PR); ++q)
                buf[swz<C::LOGE>(subpass_out_pos<PR, PP, C::LOGT>(t, b, q), PP)] = v[b + q * (C::E >> PR)];
        __syncthreads();
#pragma unroll
        for (int e = 0; e < C::E; ++e) v[e] = buf[swz<C::LOGE>(t + C::T * e, PP)];
        subpass_run<LOGN, I, LE>(v, t, tw, eng);
        RowsChain<LOGN, I + 1, LE>::run(v, t, buf, tw, eng);
    }
};
template <int LOGN, int I, int LE>
struct RowsChain<LOGN, I, LE, true> {
    template <class Eng>
    __device__ __forceinline__ static void run(float2 (&)[SubCfg<LOGN, LE>::E], int, float2 *, const float2 *,
                                               Eng &) {}
};

// Samples between the exchange buffers of consecutive transforms of a rows
// tile: N, plus T (one sample a thread) when a warp spans more than two
// transforms (T < 16: N = 2^5 .. 2^7 with 16 samples a thread).  Unpadded, the
// 32 / T buffers a warp touches would start on the same banks (16-, 8- and
// 4-way conflicts); offset by 2T words each, one warp access covers 64
// consecutive words: two wavefronts, the minimum for 32 8-byte lanes.
template <int LOGN, int LE = 4>
GBFFT_HD constexpr int rows_buf_stride() {
    return SubCfg<LOGN, LE>::N + (SubCfg<LOGN, LE>::T < 16 ? SubCfg<LOGN, LE>::T : 0);
}

// Per-transform access for rows_tile: where transform g of the tile lives,
// whether it exists, and its direction.
struct RowRef {
    const float2 *src;
    float2 *dst;
    bool active;
    float in_im, out_re, out_im;
    uint32_t row;      // batch index (noise stream)
};

// G transforms of length 2^LOGN; thread tid = g*T + t.  `ref(g)` gives the
// transform's RowRef.  smem holds G * rows_buf_stride complex values (unused
// if NSUB == 1).
// DIRC: direction known at compile time (-1 forward: no sign or scale work at
// all; +1 inverse: conjugate on load, RowRef's scales on store), or 0 (taken
// from RowRef per transform, for launches that mix directions).
// LE: log2 of the samples a thread holds (SubCfg).
template <int LOGN, int G, int DIRC = 0, int LE = 4, class RefFn, class Eng = DftRegs>
__device__ __forceinline__ void rows_tile(RefFn ref, const float2 *__restrict__ tw, float2 *smem, const LoadOps &ops,
                                          Eng eng = Eng()) {
    using C = SubCfg<LOGN, LE>;
    const int tid = threadIdx.x;
    const int g = tid >> C::LOGT;
    const int t = tid & (C::T - 1);
    const RowRef r = ref(g);
    float2 v[C::E];
    // All E loads first, back to back (the branch on the noise stays outside
    // the load loop so nothing serialises them).
#pragma unroll
    for (int e = 0; e < C::E; ++e) v[e] = r.active ? ld_stream(r.src + t + C::T * e) : make_float2(0.f, 0.f);
    if (ops.noise_sigma != 0.f) {
#pragma unroll
        for (int e = 0; e < C::E; ++e) {
            const float2 z = pipeline_noise(t + C::T * e, ops.row_base + r.row, ops.noise_seed, ops.noise_sigma);
            v[e] = make_float2(v[e].x + z.x, v[e].y + z.y);
        }
    }
    if constexpr (DIRC == 0) {
#pragma unroll
        for (int e = 0; e < C::E; ++e) v[e].y *= r.in_im;
    } else if constexpr (DIRC > 0) {
#pragma unroll
        for (int e = 0; e < C::E; ++e) v[e].y = -v[e].y;
    }
    if (ops.win != nullptr) {
#pragma unroll
        for (int e = 0; e < C::E; ++e) {
            const float w = __ldg(ops.win + t + C::T * e);
            v[e] = make_float2(v[e].x * w, v[e].y * w);
        }
    }
    subpass_run<LOGN, 0, LE>(v, t, tw, eng);
    RowsChain<LOGN, 1, LE>::run(v, t, smem + g * rows_buf_stride<LOGN, LE>(), tw, eng);
    // last sub-pass (p R = N): output q of butterfly j sits at j + q p
    if (r.active) {
        constexpr int LR = C::logr(C::NSUB - 1), LP = C::logp(C::NSUB - 1);
        constexpr int NB = C::E >> LR;
#pragma unroll
        for (int b = 0; b < NB; ++b)
#pragma unroll
            for (int q = 0; q < (1 << LR); ++q) {
                const float2 y = v[b + q * NB];
                st_stream(r.dst + subpass_out_pos<LR, LP, C::LOGT>(t, b, q),
                          DIRC < 0 ? y : make_float2(y.x * r.out_re, y.y * r.out_im));
            }
    }
}

// ---- global-pass tiles -----------------------------------------------------

// Row of the [row][2^CL column] exchange tile.  With 16 columns a warp spans
// two rows, which fill the banks whatever their distance.  With 8 it spans four
// (t = 4w .. 4w+3); after a sub-pass with p = 1 they are 2^PR apart and would
// all share one half of the banks, so row bit 0 is flipped by row bit PR.  That
// permutes every aligned group of four rows within itself, so the reads of rows
// t + T e stay conflict-free.
template <int CL, int PP, int PR>
GBFFT_HD int xrow(int row) {
    if constexpr (CL < kColsLog && PP == 0) return row ^ ((row >> PR) & 1);
    else return row;
}
// Exchange-tile index of (row, column c) after a sub-pass (PR, PP).
template <int CL, int PP, int PR>
GBFFT_HD int xch_idx(int row, int c) {
    return (xrow<CL, PP, PR>(row) << CL) + c;
}
// A first pass stages output `pos` of column c at [column][pos ^ (column << (4 - CL))]:
// a warp's 32 / 2^CL rows of 2^CL columns then cover every bank pair twice, and
// with CL < 4 the XOR keeps bit 0, so samples pos, pos + 1 (pos even) stay adjacent.
template <int CL, int LOGR>
GBFFT_HD int stage_idx(int c, int pos) {
    return (c << LOGR) + (pos ^ (c << (kColsLog - CL)));
}

template <int LOGR, int I, int LE = 4, int CL = kColsLog, bool DONE = (I >= SubCfg<LOGR, LE>::NSUB)>
struct PassChain {
    using C = SubCfg<LOGR, LE>;
    template <class Eng>
    __device__ __forceinline__ static void run(float2 (&v)[C::E], int t, int c, float2 *buf, const float2 *tw,
                                               Eng &eng) {
        constexpr int PR = C::logr(I - 1), PP = C::logp(I - 1);
        if (I > 1) __syncthreads();
#pragma unroll
        for (int b = 0; b < (C::E >> PR); ++b)
#pragma unroll
            for (int q = 0; q < (1 << PR); ++q)
                buf[xch_idx<CL, PP, PR>(subpass_out_pos<PR, PP, C::LOGT>(t, b, q), c)] = v[b + q * (C::E >> PR)];
        __syncthreads();
#pragma unroll
        for (int e = 0; e < C::E; ++e) v[e] = buf[xch_idx<CL, PP, PR>(t + C::T * e, c)];
        subpass_run<LOGR, I, LE>(v, t, tw, eng);
        PassChain<LOGR, I + 1, LE, CL>::run(v, t, c, buf, tw, eng);
    }
};
template <int LOGR, int I, int LE, int CL>
struct PassChain<LOGR, I, LE, CL, true> {
    template <class Eng>
    __device__ __forceinline__ static void run(float2 (&)[SubCfg<LOGR, LE>::E], int, int, float2 *, const float2 *,
                                               Eng &) {}
};

__device__ __forceinline__ float2 twiddle_2level(const float2 *__restrict__ lo, const float2 *__restrict__ hi,
                                                 uint32_t ex, int split) {
    return cmul(ld_tw(hi + (ex >> split)), ld_tw(lo + (ex & ((1u << split) - 1))));
}

template <int LOGR, int NG, int LE = 4, int CL = kColsLog>
struct PassTileCfg {
    using S = SubCfg<LOGR, LE>;
    static constexpr int COLS = 1 << CL;
    static constexpr int THREADS = NG * COLS * S::T;
    static constexpr int COLTW_STRIDE = S::E + 1;  // padded: conflict-free column reads
    static constexpr size_t SMEM_ELEMS = (size_t)NG * COLS * S::N + (size_t)NG * COLS * COLTW_STRIDE;
};

// Arguments of one global pass over one transform (offsets already applied).
struct PassArgs {
    const float2 *src;  // transform base, input of this pass
    float2 *dst;        // transform base, output of this pass
    int logn, logp;
    uint32_t col0;      // first column of the tile (multiple of NG * 2^CL)
    const float2 *tw_sub, *tw_lo, *tw_hi;
    int tw_split;
    float in_im;          // -1: conjugate the input (first pass of an inverse)
    float out_re, out_im; // output scale; later passes only (a first pass never scales)
    bool coherent_load;  // input written earlier in the same kernel: bypass L1
    bool keep_l2 = false;  // output is read again soon (fused pairs): store it with normal L2 priority
    uint32_t row;        // batch index of the transform (noise stream)
    LoadOps ops;         // first pass: noise / window applied on load
};

// NG groups x 2^CL columns (16 by default) of one global Stockham pass of radix 2^LOGR.
// LOGN_CT / LOGP_CT: log2 N and log2 p when the caller knows them at compile
// time (0 / -1: taken from a.logn / a.logp).  Constant sizes turn every
// strided address and twiddle index into immediates.  LE: log2 of the
// samples a thread holds (SubCfg; the sub-pass tables in a.tw_sub follow it).
// CL: log2 of the columns a group takes; 8 columns still move 64 contiguous
// bytes per row and halve the tile, so a radix-2^9/2^10 tile fits twice per SM.
// PRE: the input tile is already in shared memory as [row][2^CL columns] at
// the group's exchange buffer (NG = 1; brought in by the tensor memory
// accelerator), so the samples are read from there instead of from a.src.
template <int LOGR, int NG, bool FIRST, class Eng = DftRegs, int LOGN_CT = 0, int LOGP_CT = -1, int LE = 4,
          int CL = kColsLog, bool PRE = false>
__device__ __forceinline__ void pass_tile(const PassArgs &a, float2 *smem, Eng eng = Eng()) {
    using C = SubCfg<LOGR, LE>;
    using K = PassTileCfg<LOGR, NG, LE, CL>;
    constexpr int R = C::N, T = C::T, E = C::E;
    constexpr int COLS = 1 << CL;
    const int tid = threadIdx.x;
    const int grp = tid / (COLS * T);
    const int lt = tid - grp * (COLS * T);
    const int c = lt & (COLS - 1);
    const int t = lt >> CL;
    float2 *buf = smem + grp * (COLS * R);
    float2 *coltw = smem + NG * COLS * R + grp * (COLS * K::COLTW_STRIDE);
    const int logn = LOGN_CT > 0 ? LOGN_CT : a.logn;
    const int logp = LOGP_CT >= 0 ? LOGP_CT : a.logp;
    const int tw_split = LOGN_CT > 0 ? (LOGN_CT + 1) / 2 : a.tw_split;
    const int lognc = logn - LOGR;
    const uint32_t j0 = a.col0 + grp * COLS;
    const uint32_t j = j0 + c;

    float2 v[E];
    // All E loads first, back to back; options are applied afterwards.
    if constexpr (PRE) {
        static_assert(NG == 1, "one column group per CTA");
#pragma unroll
        for (int e = 0; e < E; ++e) v[e] = buf[((t + T * e) << CL) + c];
        __syncthreads();  // the tile is the exchange buffer: every thread has its samples first
    } else if (a.coherent_load) {
#pragma unroll
        for (int e = 0; e < E; ++e) v[e] = __ldcg(a.src + j + ((uint64_t)(t + T * e) << lognc));
    } else {
#pragma unroll
        for (int e = 0; e < E; ++e) v[e] = ld_stream(a.src + j + ((uint64_t)(t + T * e) << lognc));
    }
    if (FIRST && a.ops.noise_sigma != 0.f) {
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const float2 z = pipeline_noise(j + ((uint32_t)(t + T * e) << lognc), a.ops.row_base + a.row,
                                           a.ops.noise_seed, a.ops.noise_sigma);
            v[e] = make_float2(v[e].x + z.x, v[e].y + z.y);
        }
    }
    if (a.in_im != 1.0f) {
#pragma unroll
        for (int e = 0; e < E; ++e) v[e].y *= a.in_im;
    }
    if (FIRST && a.ops.win != nullptr) {
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const float w = __ldg(a.ops.win + j + ((uint64_t)(t + T * e) << lognc));
            v[e] = make_float2(v[e].x * w, v[e].y * w);
        }
    }
    if (!FIRST) {
        const uint32_t pmask = (1u << logp) - 1;
        // per-column factors W_{E p}^{e k} = W_N^{(e k) << (logn - LOGE - logp)}
        const int sh_col = logn - C::LOGE - logp;
        for (int i = lt; i < COLS * E; i += COLS * T) {
            const int cc = i >> C::LOGE, ee = i & (E - 1);
            const uint32_t kk = (j0 + cc) & pmask;
            coltw[cc * K::COLTW_STRIDE + ee] = twiddle_2level(a.tw_lo, a.tw_hi, (kk * ee) << sh_col, tw_split);
        }
        // per-thread factor W_{R p}^{t k}
        const uint32_t k = j & pmask;
        const float2 w = twiddle_2level(a.tw_lo, a.tw_hi, (t * k) << (logn - LOGR - logp), tw_split);
        __syncthreads();
#pragma unroll
        for (int e = 0; e < E; ++e) v[e] = cmul(v[e], cmul(w, coltw[c * K::COLTW_STRIDE + e]));
    }
    subpass_run<LOGR, 0, LE>(v, t, a.tw_sub, eng);
    PassChain<LOGR, 1, LE, CL>::run(v, t, c, buf, a.tw_sub, eng);

    constexpr int LR = C::logr(C::NSUB - 1), LP = C::logp(C::NSUB - 1);
    constexpr int NB = E >> LR;
    if (FIRST) {
        // Outputs of column j are contiguous at j R + q: stage them (stage_idx)
        // and store each group's 2^CL R-sample block linearly.
        __syncthreads();
#pragma unroll
        for (int bb = 0; bb < NB; ++bb)
#pragma unroll
            for (int q = 0; q < (1 << LR); ++q) {
                const int pos = subpass_out_pos<LR, LP, C::LOGT>(t, bb, q);
                buf[stage_idx<CL, LOGR>(c, pos)] = v[bb + q * NB];
            }
        __syncthreads();
        float2 *blk = a.dst + (uint64_t)j0 * R;
        if constexpr (CL < kColsLog) {
            // samples q, q + 1 (q even) are adjacent in the staging buffer: 16-byte
            // loads and stores, half the store instructions (the caller's dst is
            // 16-byte aligned)
#pragma unroll
            for (int e = 0; e < E / 2; ++e) {
                const int lin = 2 * (lt + COLS * T * e);
                const int cc = lin >> LOGR, q = lin & (R - 1);
                const float4 w = *reinterpret_cast<const float4 *>(buf + stage_idx<CL, LOGR>(cc, q));
                if (a.keep_l2) __stcg(reinterpret_cast<float4 *>(blk + lin), w);
                else st_stream(reinterpret_cast<float4 *>(blk + lin), w);
            }
        } else if (a.keep_l2) {
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const int lin = lt + COLS * T * e;
                const int cc = lin >> LOGR, q = lin & (R - 1);
                __stcg(blk + lin, buf[stage_idx<CL, LOGR>(cc, q)]);
            }
        } else {
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const int lin = lt + COLS * T * e;
                const int cc = lin >> LOGR, q = lin & (R - 1);
                st_stream(blk + lin, buf[stage_idx<CL, LOGR>(cc, q)]);
            }
        }
    } else {
        const uint32_t pmask = (1u << logp) - 1;
        float2 *col = a.dst + ((uint64_t)(j >> logp) << (LOGR + logp)) + (j & pmask);
        if (a.out_re != 1.0f || a.out_im != 1.0f) {
#pragma unroll
            for (int e = 0; e < E; ++e) v[e] = make_float2(v[e].x * a.out_re, v[e].y * a.out_im);
        }
        if (a.keep_l2) {
#pragma unroll
            for (int bb = 0; bb < NB; ++bb)
#pragma unroll
                for (int q = 0; q < (1 << LR); ++q) {
                    const int pos = subpass_out_pos<LR, LP, C::LOGT>(t, bb, q);
                    __stcg(col + ((uint64_t)pos << logp), v[bb + q * NB]);
                }
        } else {
#pragma unroll
            for (int bb = 0; bb < NB; ++bb)
#pragma unroll
                for (int q = 0; q < (1 << LR); ++q) {
                    const int pos = subpass_out_pos<LR, LP, C::LOGT>(t, bb, q);
                    st_stream(col + ((uint64_t)pos << logp), v[bb + q * NB]);
                }
        }
    }
}

}  // namespace gbfft
