// Schedule and register-level sub-pass of an FFT of length 2^LOGN computed by
// 2^LOGT threads that each hold E = 16 samples (fewer when N < 16).
//
// The transform is a Stockham autosort -- the same family as the reference's
// radix-4 stages (larsjoost/wgls-rs-fft src/shaders.rs:8-63: butterfly j reads
// j + m N/R, twiddles by W_{Rp}^{m k} with k = j mod p, writes
// (j/p) R p + k + q p) -- but with radix 16 (plus one radix 2/4/8 remainder
// sub-pass last), executed in registers with shared-memory exchanges instead
// of one HBM round trip per stage.
//
// Thread t owns samples t + T e (e < E) at the start of every sub-pass; in a
// sub-pass of radix R it runs E/R butterflies j = t + T b, butterfly b using
// register slots b + m E/R.
#pragma once
#include "fft_core.cuh"

namespace gbfft {

template <int LOGN>
struct SubCfg {
    static constexpr int LOGE = LOGN < 4 ? LOGN : 4;
    static constexpr int N = 1 << LOGN;
    static constexpr int E = 1 << LOGE;
    static constexpr int LOGT = LOGN - LOGE;
    static constexpr int T = 1 << LOGT;
    static constexpr int NFULL = LOGE == 0 ? 1 : LOGN / LOGE;
    static constexpr int LREM = LOGE == 0 ? 0 : LOGN % LOGE;
    static constexpr int NSUB = NFULL + (LREM ? 1 : 0);

    // log2 radix of sub-pass i and log2 of p = product of earlier radices
    __host__ __device__ static constexpr int logr(int i) { return i < NFULL ? LOGE : LREM; }
    __host__ __device__ static constexpr int logp(int i) { return i * LOGE; }
    // Offset (complex entries) of sub-pass i's table in the concatenation of
    // the tables of sub-passes 1..NSUB-1.  Table of sub-pass i holds
    // W_{R p}^{m k} for m in [1, R), k in [0, p), laid out [m-1][k].
    __host__ __device__ static constexpr int tw_offset(int i) {
        int off = 0;
        for (int s = 1; s < i; ++s) off += ((1 << logr(s)) - 1) << logp(s);
        return off;
    }
    __host__ __device__ static constexpr int tw_entries() { return tw_offset(NSUB); }
};

// Butterflies of one sub-pass on the register array v.
template <int LOGE, int LOGR, int LOGP, int LOGT>
__device__ __forceinline__ void subpass_compute(float2 (&v)[1 << LOGE], int t, const float2 *tw) {
    constexpr int E = 1 << LOGE, R = 1 << LOGR, NB = E / R, P = 1 << LOGP, T = 1 << LOGT;
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        float2 x[R];
#pragma unroll
        for (int m = 0; m < R; ++m) x[m] = v[b + m * NB];
        if (LOGP > 0) {
            const int j = t + T * b;
            const int k = j & (P - 1);
#pragma unroll
            for (int m = 1; m < R; ++m) x[m] = cmul(x[m], ld_tw(tw + (m - 1) * P + k));
        }
        Dft<R>::run(x);
#pragma unroll
        for (int q = 0; q < R; ++q) v[b + q * NB] = x[q];
    }
}

// Position (within the transform) of output q of butterfly slot b after
// sub-pass (LOGR, LOGP): (j / p) R p + (j mod p) + q p.
template <int LOGR, int LOGP, int LOGT>
__device__ __forceinline__ int subpass_out_pos(int t, int b, int q) {
    const int j = t + (b << LOGT);
    return ((j >> LOGP) << (LOGR + LOGP)) + (j & ((1 << LOGP) - 1)) + (q << LOGP);
}

}  // namespace gbfft
