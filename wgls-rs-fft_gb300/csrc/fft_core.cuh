// Register-level building blocks of the GB300 FFT kernels: complex helpers,
// forward DFTs of radix 2/4/8/16 on register arrays, streaming global access.
//
// All butterflies compute the forward kernel e^{-2 pi i k n / R} in natural
// output order.  The inverse transform conjugates on load and on store
// (x -> conj(FFT(conj x)) / N), the same identity the reference applies on the
// host (larsjoost/wgls-rs-fft src/lib.rs:571-579, 661-669).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

// Butterfly building blocks are host and device functions (the host side
// only serves the CPU tests that check them against an FP64 DFT).
#define GBFFT_HD __host__ __device__ __forceinline__
// loop unrolling hint for code that is also compiled for the host
#if defined(__CUDA_ARCH__)
#define GBFFT_UNROLL _Pragma("unroll")
#else
#define GBFFT_UNROLL
#endif

// Packed FP32: the sm_100 family executes two-lane FP32 operations
// (__fadd2_rn, __fmul2_rn, __ffma2_rn) as one instruction, each lane rounded
// exactly like the scalar operation.  A complex add, subtract or real-factor
// FMA is then one instruction instead of two, with the same bits; the host
// build (the CPU tests of these functions) uses the scalar forms.
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
#define GBFFT_PACKED_F32 1
#endif

namespace gbfft {

// PK selects the packed form (the default) or the scalar one, per kernel:
// packing pairs registers, which costs where a kernel's registers are scarce.
template <bool PK = true>
GBFFT_HD float2 cadd(float2 a, float2 b) {
#ifdef GBFFT_PACKED_F32
    if constexpr (PK) return __fadd2_rn(a, b);
#endif
    return make_float2(a.x + b.x, a.y + b.y);
}
template <bool PK = true>
GBFFT_HD float2 csub(float2 a, float2 b) {
#ifdef GBFFT_PACKED_F32
    if constexpr (PK) return __fadd2_rn(a, make_float2(-b.x, -b.y));
#endif
    return make_float2(a.x - b.x, a.y - b.y);
}
GBFFT_HD float2 cmul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// cmul as one packed multiply and one packed FMA (same bits as cmul).  Its
// operands need the pairs (a.y, a.y), (-b.y, b.x) and (a.x, a.x) built first,
// so it pays only where registers are not scarce: measured +1 % in the
// single-pass kernel at N = 4096, -2 % in the fused pass pairs.
GBFFT_HD float2 cmul_x2(float2 a, float2 b) {
#ifdef GBFFT_PACKED_F32
    const float2 t = __fmul2_rn(make_float2(a.y, a.y), make_float2(-b.y, b.x));
    return __ffma2_rn(make_float2(a.x, a.x), b, t);
#else
    return cmul(a, b);
#endif
}
// x -> s + f y per component (f a real factor absorbed into the add)
template <bool PK = true>
GBFFT_HD float2 cfma(float f, float2 y, float2 s) {
#ifdef GBFFT_PACKED_F32
    if constexpr (PK) return __ffma2_rn(make_float2(f, f), y, s);
#endif
    return make_float2(fmaf(f, y.x, s.x), fmaf(f, y.y, s.y));
}
// a * (-i)
GBFFT_HD float2 mul_mi(float2 a) { return make_float2(a.y, -a.x); }

constexpr float kSqrtHalf = 0.70710678118654752440f;
constexpr float kCos1_16 = 0.92387953251128675613f;  // cos(pi/8)
constexpr float kSin1_16 = 0.38268343236508977173f;  // sin(pi/8)

// a * e^{-i pi/4} = a * (1 - i)/sqrt2
GBFFT_HD float2 mul_w8_1(float2 a) {
    return make_float2((a.x + a.y) * kSqrtHalf, (a.y - a.x) * kSqrtHalf);
}
// a * e^{-3 i pi/4} = a * (-1 - i)/sqrt2
GBFFT_HD float2 mul_w8_3(float2 a) {
    return make_float2((a.y - a.x) * kSqrtHalf, -(a.x + a.y) * kSqrtHalf);
}
// a * e^{-i pi/8}
GBFFT_HD float2 mul_w16_1(float2 a) {
    return make_float2(fmaf(a.x, kCos1_16, a.y * kSin1_16), fmaf(a.y, kCos1_16, -a.x * kSin1_16));
}
// a * e^{-3 i pi/8}
GBFFT_HD float2 mul_w16_3(float2 a) {
    return make_float2(fmaf(a.x, kSin1_16, a.y * kCos1_16), fmaf(a.y, kSin1_16, -a.x * kCos1_16));
}
// a * e^{-9 i pi/8} = -a * e^{-i pi/8}
GBFFT_HD float2 mul_w16_9(float2 a) {
    return make_float2(-fmaf(a.x, kCos1_16, a.y * kSin1_16), -fmaf(a.y, kCos1_16, -a.x * kSin1_16));
}

template <int R> struct Dft;

template <> struct Dft<1> {
    template <bool PK = true>
    GBFFT_HD static void run(float2 *) {}
};

template <> struct Dft<2> {
    template <bool PK = true>
    GBFFT_HD static void run(float2 *x) {
        float2 a = x[0], b = x[1];
        x[0] = cadd<PK>(a, b);
        x[1] = csub<PK>(a, b);
    }
};

template <> struct Dft<4> {
    template <bool PK = true>
    GBFFT_HD static void run(float2 *x) {
        float2 s02 = cadd<PK>(x[0], x[2]), d02 = csub<PK>(x[0], x[2]);
        float2 s13 = cadd<PK>(x[1], x[3]), d13 = mul_mi(csub<PK>(x[1], x[3]));
        x[0] = cadd<PK>(s02, s13);
        x[2] = csub<PK>(s02, s13);
        x[1] = cadd<PK>(d02, d13);
        x[3] = csub<PK>(d02, d13);
    }
};

template <> struct Dft<8> {
    // radix-2 decimation in frequency, then two 4-point DFTs.  The odd half's
    // twiddles W8^1 = k (1 - i) and W8^3 = k (-1 - i) (k = sqrt(1/2)) are
    // applied without k; the second 4-point DFT's last additions take k as FMAs.
    template <bool PK = true>
    GBFFT_HD static void run(float2 *x) {
        float2 a[4], b[4];
        GBFFT_UNROLL
        for (int k = 0; k < 4; ++k) {
            a[k] = cadd<PK>(x[k], x[k + 4]);
            b[k] = csub<PK>(x[k], x[k + 4]);
        }
        Dft<4>::run<PK>(a);
        // b1 (1 - i), b3 (-1 - i): the twiddled inputs of the odd 4-point DFT, up to k
        const float2 q1 = make_float2(b[1].x + b[1].y, b[1].y - b[1].x);
        const float2 q3 = make_float2(b[3].y - b[3].x, -(b[3].x + b[3].y));
        const float2 u2 = mul_mi(b[2]);
        const float2 s02 = cadd<PK>(b[0], u2), d02 = csub<PK>(b[0], u2);
        const float2 S = cadd<PK>(q1, q3), D = mul_mi(csub<PK>(q1, q3));
        x[0] = a[0];
        x[2] = a[1];
        x[4] = a[2];
        x[6] = a[3];
        x[1] = cfma<PK>(kSqrtHalf, S, s02);
        x[3] = cfma<PK>(kSqrtHalf, D, d02);
        x[5] = cfma<PK>(-kSqrtHalf, S, s02);
        x[7] = cfma<PK>(-kSqrtHalf, D, d02);
    }
};

constexpr float kTan1_16 = 0.41421356237309504880f;  // tan(pi/8) = sqrt(2) - 1


template <> struct Dft<16> {
    // 16 = 4 x 4: n = n1 + 4 n2, k = 4 k1 + k2.  Between the two layers of
    // 4-point DFTs, input n1 of column k2 is twiddled by W16^(n1 k2).  Those
    // twiddles are applied up to a real factor that the second layer's last
    // additions take as FMAs:
    //   W16^1 = c (1 - i t), W16^3 = c (t - i), W16^9 = -c (1 - i t)   (c = cos(pi/8), t = tan(pi/8))
    //   W8^1 = k (1 - i),    W8^3 = k (-1 - i)                          (k = sqrt(1/2))
    // Two FMAs per W16 twiddle and two adds per W8 twiddle, instead of four
    // instructions each: 144 instructions for the 16-point DFT instead of 160.
    template <bool PK = true>
    GBFFT_HD static void run(float2 *x) {
        float2 z[4][4];
        GBFFT_UNROLL
        for (int n1 = 0; n1 < 4; ++n1) {
            float2 t[4] = {x[n1], x[n1 + 4], x[n1 + 8], x[n1 + 12]};
            Dft<4>::run<PK>(t);
            GBFFT_UNROLL
            for (int k2 = 0; k2 < 4; ++k2) z[n1][k2] = t[k2];
        }
        {  // k2 = 0: no twiddles
            float2 t[4] = {z[0][0], z[1][0], z[2][0], z[3][0]};
            Dft<4>::run<PK>(t);
            x[0] = t[0];
            x[4] = t[1];
            x[8] = t[2];
            x[12] = t[3];
        }
        {  // k2 = 1: W16^1 (c), W8^1 (k), W16^3 (c)
            const float2 a = z[1][1], b = z[3][1], q = z[2][1];
            const float2 p1 = make_float2(fmaf(a.y, kTan1_16, a.x), fmaf(-a.x, kTan1_16, a.y));  // a (1 - i t)
            const float2 p3 = make_float2(fmaf(b.x, kTan1_16, b.y), fmaf(b.y, kTan1_16, -b.x));  // b (t - i)
            const float2 q2 = make_float2(q.x + q.y, q.y - q.x);                                // q (1 - i)
            const float2 s02 = cfma<PK>(kSqrtHalf, q2, z[0][1]), d02 = cfma<PK>(-kSqrtHalf, q2, z[0][1]);
            const float2 P = cadd<PK>(p1, p3), Q = mul_mi(csub<PK>(p1, p3));
            x[1] = cfma<PK>(kCos1_16, P, s02);
            x[5] = cfma<PK>(kCos1_16, Q, d02);
            x[9] = cfma<PK>(-kCos1_16, P, s02);
            x[13] = cfma<PK>(-kCos1_16, Q, d02);
        }
        {  // k2 = 2: W8^1 (k), -i, W8^3 (k)
            const float2 a = z[1][2], b = z[3][2];
            const float2 q1 = make_float2(a.x + a.y, a.y - a.x);     // a (1 - i)
            const float2 q3 = make_float2(b.y - b.x, -(b.x + b.y));  // b (-1 - i)
            const float2 u2 = mul_mi(z[2][2]);
            const float2 s02 = cadd<PK>(z[0][2], u2), d02 = csub<PK>(z[0][2], u2);
            const float2 S = cadd<PK>(q1, q3), D = mul_mi(csub<PK>(q1, q3));
            x[2] = cfma<PK>(kSqrtHalf, S, s02);
            x[6] = cfma<PK>(kSqrtHalf, D, d02);
            x[10] = cfma<PK>(-kSqrtHalf, S, s02);
            x[14] = cfma<PK>(-kSqrtHalf, D, d02);
        }
        {  // k2 = 3: W16^3 (c), W8^3 (k), W16^9 (-c)
            const float2 a = z[1][3], b = z[3][3], q = z[2][3];
            const float2 p1 = make_float2(fmaf(a.x, kTan1_16, a.y), fmaf(a.y, kTan1_16, -a.x));  // a (t - i)
            const float2 p3 = make_float2(fmaf(b.y, kTan1_16, b.x), fmaf(-b.x, kTan1_16, b.y));  // b (1 - i t)
            const float2 q2 = make_float2(q.y - q.x, -(q.x + q.y));                             // q (-1 - i)
            const float2 s02 = cfma<PK>(kSqrtHalf, q2, z[0][3]), d02 = cfma<PK>(-kSqrtHalf, q2, z[0][3]);
            // u1 = c p1, u3 = -c p3: u1 + u3 = c (p1 - p3), -i (u1 - u3) = c (-i)(p1 + p3)
            const float2 P = csub<PK>(p1, p3), Q = mul_mi(cadd<PK>(p1, p3));
            x[3] = cfma<PK>(kCos1_16, P, s02);
            x[7] = cfma<PK>(kCos1_16, Q, d02);
            x[11] = cfma<PK>(-kCos1_16, P, s02);
            x[15] = cfma<PK>(-kCos1_16, Q, d02);
        }
    }
};

// Options applied to every sample as a transform loads it, in this order:
//   x += noise (if sigma != 0), conjugate (inverse), x *= win[n] (if win).
// The noise is the reference pipeline's NOISE stage
// (larsjoost/wgls-rs-fft examples/parallel_pipeline.rs:36-62): PCG hash of
// n * 1234567 + row * 7654321 + seed, Box-Muller with sigma (0.1 there).
struct LoadOps {
    const float *win;   // real window table of the transform length, or nullptr
    uint32_t noise_seed;
    float noise_sigma;  // 0 disables the noise
    uint32_t row_base;  // batch index of the launch's first row (noise stream)
};

__host__ __device__ __forceinline__ uint32_t pcg_hash(uint32_t v) {
    const uint32_t s = v * 747796405u + 2891336453u;
    const uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
    return (w >> 22u) ^ w;
}

__device__ __forceinline__ float2 pipeline_noise(uint32_t n, uint32_t row, uint32_t seed, float sigma) {
    const uint32_t h1 = pcg_hash(n * 1234567u + row * 7654321u + seed);
    const uint32_t h2 = pcg_hash(h1 + 999983u);
    const float u1 = fmaxf(__uint2float_rn(h1) * 2.328306437e-10f, 1e-7f);
    const float u2 = __uint2float_rn(h2) * 2.328306437e-10f * 6.283185307f;
    const float r = sqrtf(-2.0f * logf(u1)) * sigma;
    float sn, cs;
    sincosf(u2, &sn, &cs);
    return make_float2(r * cs, r * sn);
}

// Streaming global access: every sample is read once and written once.
__device__ __forceinline__ float2 ld_stream(const float2 *p) { return __ldcs(p); }
__device__ __forceinline__ void st_stream(float2 *p, float2 v) { __stcs(p, v); }
__device__ __forceinline__ void st_stream(float4 *p, float4 v) { __stcs(p, v); }
// Twiddles are shared by every transform of a plan: keep them cached.
__device__ __forceinline__ float2 ld_tw(const float2 *p) { return __ldg(p); }
// Bring one 128-byte line toward L2 ahead of its use (a hint: never faults on
// a valid address, changes no data).
__device__ __forceinline__ void prefetch_l2(const void *p) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

}  // namespace gbfft
