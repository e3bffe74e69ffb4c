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
#include <type_traits>
#include <utility>

#include "fft_core.cuh"
#include "gbfft_internal.h"

namespace gbfft {

// LE: log2 of the samples a thread holds (4, or 5 for the 32-sample tiles
// of N = 2^13 / 2^14, which need one exchange fewer).
template <int LOGN, int LE = 4>
struct SubCfg {
    static constexpr int LOGE = LOGN < LE ? LOGN : LE;
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
    // The last sub-pass with radix R < E runs E/R butterflies per thread with
    // k = j = t + T b; its twiddle W_N^{m (t + T b)} factors into a table entry
    // W_N^{m t} and the constant W_E^{m b}.
    __host__ __device__ static constexpr bool factored(int i) { return i > 0 && logr(i) < LOGE; }
    // Table of sub-pass i (i >= 1): entries W_M^{m k}, m in [1, R), k in
    // [0, 2^tw_logp(i)), laid out [m-1][k], M = 2^tw_logm(i).
    __host__ __device__ static constexpr int tw_logp(int i) { return factored(i) ? LOGT : logp(i); }
    __host__ __device__ static constexpr int tw_logm(int i) { return factored(i) ? LOGN : logr(i) + logp(i); }
    __host__ __device__ static constexpr int tw_count(int i) { return ((1 << logr(i)) - 1) << tw_logp(i); }
    __host__ __device__ static constexpr int tw_offset(int i) {
        int off = 0;
        for (int s = 1; s < i; ++s) off += tw_count(s);
        return off;
    }
    __host__ __device__ static constexpr int tw_entries() { return tw_offset(NSUB); }
};

// a * W_16^I for a compile-time I (exact special cases where they exist).
template <int I>
GBFFT_HD float2 mul_w16c(float2 a) {
    constexpr int i = I & 15;
    if constexpr (i == 0) return a;
    else if constexpr (i == 1) return mul_w16_1(a);
    else if constexpr (i == 2) return mul_w8_1(a);
    else if constexpr (i == 3) return mul_w16_3(a);
    else if constexpr (i == 4) return mul_mi(a);
    else if constexpr (i == 6) return mul_w8_3(a);
    else if constexpr (i == 8) return make_float2(-a.x, -a.y);
    else if constexpr (i == 9) return mul_w16_9(a);
    else if constexpr (i > 8) {
        const float2 b = mul_w16c<i - 8>(a);
        return make_float2(-b.x, -b.y);
    } else {  // 5, 7
        const float2 b = mul_w16c<i - 4>(a);
        return mul_mi(b);
    }
}

// a * W_32^I for a compile-time I: even I through mul_w16c, odd I with the
// constants cos(pi k / 16), sin(pi k / 16) (k = 1, 3; k = 5, 7 swap them).
constexpr float kCos1_32 = 0.98078528040323044913f;  // cos(pi/16)
constexpr float kSin1_32 = 0.19509032201612826785f;  // sin(pi/16)
constexpr float kCos3_32 = 0.83146961230254523708f;  // cos(3 pi/16)
constexpr float kSin3_32 = 0.55557023301960222474f;  // sin(3 pi/16)
template <int I>
GBFFT_HD float2 mul_w32c(float2 a) {
    constexpr int i = I & 31;
    if constexpr ((i & 1) == 0) return mul_w16c<i / 2>(a);
    else if constexpr (i > 8) return mul_mi(mul_w32c<i - 8>(a));  // W_32^8 = -i
    else {
        // a * (c - i s) with (c, s) = (cos, sin)(pi i / 16)
        constexpr float c = i == 1 ? kCos1_32 : (i == 3 ? kCos3_32 : (i == 5 ? kSin3_32 : kSin1_32));
        constexpr float sn = i == 1 ? kSin1_32 : (i == 3 ? kSin3_32 : (i == 5 ? kCos3_32 : kCos1_32));
        return make_float2(fmaf(a.x, c, a.y * sn), fmaf(a.y, c, -a.x * sn));
    }
}

// 32-point DFT: radix-2 decimation in frequency, then two 16-point DFTs.
template <> struct Dft<32> {
    template <bool PK = true>
    GBFFT_HD static void run(float2 *x) {
        float2 a[16], b[16];
        auto split = [&](auto kc) {
            constexpr int k = decltype(kc)::value;
            a[k] = cadd<PK>(x[k], x[k + 16]);
            b[k] = mul_w32c<k>(csub<PK>(x[k], x[k + 16]));
        };
        [&]<int... Ks>(std::integer_sequence<int, Ks...>) {
            (split(std::integral_constant<int, Ks>{}), ...);
        }(std::make_integer_sequence<int, 16>{});
        Dft<16>::run<PK>(a);
        Dft<16>::run<PK>(b);
        GBFFT_UNROLL
        for (int k = 0; k < 16; ++k) {
            x[2 * k] = a[k];
            x[2 * k + 1] = b[k];
        }
    }
};

template <int LOGE, int LOGR, int B, int M>
struct FactoredTw {
    // W_E^{m b} with E = 2^LOGE expressed in 32nds of a turn
    static constexpr int idx32 = ((M * B) << (5 - LOGE)) & 31;
};

// Engine of the radix-R butterflies: FP32 in registers (DftRegs, packed
// two-lane adds; DftRegsScalar, scalar ones) or, for the split-precision form,
// tensor-core matrix products (fft_tc.cuh).
template <bool PK>
struct DftRegsT {
    template <int R>
    __device__ __forceinline__ void run(float2 (&x)[R]) { Dft<R>::template run<PK>(x); }
};
using DftRegs = DftRegsT<true>;
using DftRegsScalar = DftRegsT<false>;
// The same butterflies, with the sub-pass twiddles applied by the packed
// complex multiply (cmul_x2: same bits, faster in the single-pass kernel).
struct DftRegsX2 : DftRegs {};

// a * twiddle b in the way the engine prefers
template <class Eng>
__device__ __forceinline__ float2 twiddle_mul(float2 a, float2 b) {
    if constexpr (std::is_same_v<Eng, DftRegsX2>) return cmul_x2(a, b);
    else return cmul(a, b);
}

// Butterflies of one sub-pass on the register array v.
template <int LOGE, int LOGR, int LOGP, int LOGT, bool FACT = false, class Eng = DftRegs>
__device__ __forceinline__ void subpass_compute(float2 (&v)[1 << LOGE], int t, const float2 *tw, Eng &eng) {
    constexpr int E = 1 << LOGE, R = 1 << LOGR, NB = E / R, P = 1 << LOGP, T = 1 << LOGT;
    if constexpr (FACT) {
        float2 wt[R];
#pragma unroll
        for (int m = 1; m < R; ++m) wt[m] = ld_tw(tw + (m - 1) * T + t);
        auto body = [&](auto bc) {
            constexpr int b = decltype(bc)::value;
            float2 x[R];
#pragma unroll
            for (int m = 0; m < R; ++m) x[m] = v[b + m * NB];
            auto apply = [&](auto mc) {
                constexpr int M = decltype(mc)::value;
                if constexpr (M > 0)
                    x[M] = twiddle_mul<Eng>(mul_w32c<FactoredTw<LOGE, LOGR, b, M>::idx32>(x[M]), wt[M]);
            };
            [&]<int... Ms>(std::integer_sequence<int, Ms...>) {
                (apply(std::integral_constant<int, Ms>{}), ...);
            }(std::make_integer_sequence<int, R>{});
            eng.template run<R>(x);
#pragma unroll
            for (int q = 0; q < R; ++q) v[b + q * NB] = x[q];
        };
        [&]<int... Bs>(std::integer_sequence<int, Bs...>) {
            (body(std::integral_constant<int, Bs>{}), ...);
        }(std::make_integer_sequence<int, NB>{});
    } else {
#pragma unroll
        for (int b = 0; b < NB; ++b) {
            float2 x[R];
#pragma unroll
            for (int m = 0; m < R; ++m) x[m] = v[b + m * NB];
            if (LOGP > 0) {
                const int j = t + T * b;
                const int k = j & (P - 1);
#pragma unroll
                for (int m = 1; m < R; ++m) x[m] = twiddle_mul<Eng>(x[m], ld_tw(tw + (m - 1) * P + k));
            }
            eng.template run<R>(x);
#pragma unroll
            for (int q = 0; q < R; ++q) v[b + q * NB] = x[q];
        }
    }
}

// Twiddle-table segments of sub-passes 1..NSUB-1 (offsets from `base`).
template <int LOGN, int LE = 4>
inline int subcfg_segments(TwiddleSegment *out, uint64_t base) {
    using C = SubCfg<LOGN, LE>;
    for (int i = 1; i < C::NSUB; ++i)
        out[i - 1] = TwiddleSegment{base + (uint64_t)C::tw_offset(i), (uint64_t)C::tw_count(i), 0, C::tw_logm(i),
                                    C::tw_logp(i), 0};
    return C::NSUB - 1;
}

// Sub-pass I of the schedule of SubCfg<LOGN, LE> (twiddle table already offset).
template <int LOGN, int I, int LE = 4, class Eng = DftRegs>
__device__ __forceinline__ void subpass_run(float2 (&v)[SubCfg<LOGN, LE>::E], int t, const float2 *tw_all, Eng &eng) {
    using C = SubCfg<LOGN, LE>;
    subpass_compute<C::LOGE, C::logr(I), C::logp(I), C::LOGT, C::factored(I), Eng>(v, t, tw_all + C::tw_offset(I),
                                                                                     eng);
}

// Position (within the transform) of output q of butterfly slot b after
// sub-pass (LOGR, LOGP): (j / p) R p + (j mod p) + q p.
template <int LOGR, int LOGP, int LOGT>
GBFFT_HD int subpass_out_pos(int t, int b, int q) {
    const int j = t + (b << LOGT);
    return ((j >> LOGP) << (LOGR + LOGP)) + (j & ((1 << LOGP) - 1)) + (q << LOGP);
}

}  // namespace gbfft
