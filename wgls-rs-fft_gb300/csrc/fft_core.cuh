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

namespace gbfft {

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// a * (-i)
__device__ __forceinline__ float2 mul_mi(float2 a) { return make_float2(a.y, -a.x); }

constexpr float kSqrtHalf = 0.70710678118654752440f;
constexpr float kCos1_16 = 0.92387953251128675613f;  // cos(pi/8)
constexpr float kSin1_16 = 0.38268343236508977173f;  // sin(pi/8)

// a * e^{-i pi/4} = a * (1 - i)/sqrt2
__device__ __forceinline__ float2 mul_w8_1(float2 a) {
    return make_float2((a.x + a.y) * kSqrtHalf, (a.y - a.x) * kSqrtHalf);
}
// a * e^{-3 i pi/4} = a * (-1 - i)/sqrt2
__device__ __forceinline__ float2 mul_w8_3(float2 a) {
    return make_float2((a.y - a.x) * kSqrtHalf, -(a.x + a.y) * kSqrtHalf);
}
// a * e^{-i pi/8}
__device__ __forceinline__ float2 mul_w16_1(float2 a) {
    return make_float2(fmaf(a.x, kCos1_16, a.y * kSin1_16), fmaf(a.y, kCos1_16, -a.x * kSin1_16));
}
// a * e^{-3 i pi/8}
__device__ __forceinline__ float2 mul_w16_3(float2 a) {
    return make_float2(fmaf(a.x, kSin1_16, a.y * kCos1_16), fmaf(a.y, kSin1_16, -a.x * kCos1_16));
}
// a * e^{-9 i pi/8} = -a * e^{-i pi/8}
__device__ __forceinline__ float2 mul_w16_9(float2 a) {
    return make_float2(-fmaf(a.x, kCos1_16, a.y * kSin1_16), -fmaf(a.y, kCos1_16, -a.x * kSin1_16));
}

template <int R> struct Dft;

template <> struct Dft<1> {
    __device__ __forceinline__ static void run(float2 *) {}
};

template <> struct Dft<2> {
    __device__ __forceinline__ static void run(float2 *x) {
        float2 a = x[0], b = x[1];
        x[0] = cadd(a, b);
        x[1] = csub(a, b);
    }
};

template <> struct Dft<4> {
    __device__ __forceinline__ static void run(float2 *x) {
        float2 s02 = cadd(x[0], x[2]), d02 = csub(x[0], x[2]);
        float2 s13 = cadd(x[1], x[3]), d13 = mul_mi(csub(x[1], x[3]));
        x[0] = cadd(s02, s13);
        x[2] = csub(s02, s13);
        x[1] = cadd(d02, d13);
        x[3] = csub(d02, d13);
    }
};

template <> struct Dft<8> {
    // radix-2 decimation in frequency, then two 4-point DFTs.
    __device__ __forceinline__ static void run(float2 *x) {
        float2 a[4], b[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            a[k] = cadd(x[k], x[k + 4]);
            b[k] = csub(x[k], x[k + 4]);
        }
        b[1] = mul_w8_1(b[1]);
        b[2] = mul_mi(b[2]);
        b[3] = mul_w8_3(b[3]);
        Dft<4>::run(a);
        Dft<4>::run(b);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            x[2 * k] = a[k];
            x[2 * k + 1] = b[k];
        }
    }
};

template <> struct Dft<16> {
    // 16 = 4 x 4: n = n1 + 4 n2, k = 4 k1 + k2.
    __device__ __forceinline__ static void run(float2 *x) {
        float2 z[4][4];
#pragma unroll
        for (int n1 = 0; n1 < 4; ++n1) {
            float2 t[4] = {x[n1], x[n1 + 4], x[n1 + 8], x[n1 + 12]};
            Dft<4>::run(t);
#pragma unroll
            for (int k2 = 0; k2 < 4; ++k2) z[n1][k2] = t[k2];
        }
        z[1][1] = mul_w16_1(z[1][1]);
        z[1][2] = mul_w8_1(z[1][2]);
        z[1][3] = mul_w16_3(z[1][3]);
        z[2][1] = mul_w8_1(z[2][1]);
        z[2][2] = mul_mi(z[2][2]);
        z[2][3] = mul_w8_3(z[2][3]);
        z[3][1] = mul_w16_3(z[3][1]);
        z[3][2] = mul_w8_3(z[3][2]);
        z[3][3] = mul_w16_9(z[3][3]);
#pragma unroll
        for (int k2 = 0; k2 < 4; ++k2) {
            float2 t[4] = {z[0][k2], z[1][k2], z[2][k2], z[3][k2]};
            Dft<4>::run(t);
#pragma unroll
            for (int k1 = 0; k1 < 4; ++k1) x[4 * k1 + k2] = t[k1];
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
// Twiddles are shared by every transform of a plan: keep them cached.
__device__ __forceinline__ float2 ld_tw(const float2 *p) { return __ldg(p); }
// Bring one 128-byte line toward L2 ahead of its use (a hint: never faults on
// a valid address, changes no data).
__device__ __forceinline__ void prefetch_l2(const void *p) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

}  // namespace gbfft
