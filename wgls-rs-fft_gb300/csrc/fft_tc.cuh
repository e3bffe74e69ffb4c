// Tensor-core (tcgen05) 16-point DFTs for the split-precision forms.
//
// Every thread of a tile owns one 16-point vector x (the E = 16 samples of a
// radix-16 sub-pass).  A whole sub-pass is then one real matrix product per
// 128 threads,
//     D[128 x 32] = A[128 x 32] . G[32 x 32],
// with A's row r = [Re x_0..15 | Im x_0..15] of thread r and
//     G[e][q]      =  cos(2 pi q e / 16)   G[16+e][q]    = sin(2 pi q e / 16)
//     G[e][16+q]   = -sin(2 pi q e / 16)   G[16+e][16+q] = cos(2 pi q e / 16)
// so that D's row r = [Re X_0..15 | Im X_0..15], the forward DFT of x.
//
// Precision: A and G are split into hi + lo parts and
// D = Ah.Gh + Ah.Gl + Al.Gh is accumulated in FP32 in tensor memory (the
// Al.Gl term is below the FP32 rounding of the result).  Four operand kinds:
//   FP16 / BF16 (kind::f16): each row is first scaled by an exact power of two
//     so that its largest component lies in [1, 2); FP16's range then always
//     suffices and hi + lo carry 22 significant bits (BF16: 16 bits).
//   TF32 (kind::tf32): hi = x rounded to the nearest TF32 value (an integer
//     add and mask), lo = x - hi (exact in FP32; the tensor core uses its top
//     11 significant bits).  TF32 keeps FP32's exponent range, so no scaling
//     is needed (three instructions per value; the 16-bit forms take a scale,
//     and per pair of values two packed converts and two mixed-precision
//     FMAs, plus the row maximum and the unscale).  About 22 significant bits.
//   BF16 x 6 (kind::f16, BF16 operands): A and G split into three BF16 parts,
//     hi + mid + lo (8 significant bits each, 24 together: FP32's
//     significand), and D = Ah.Gh + Ah.Gm + Am.Gh + Ah.Gl + Al.Gh + Am.Gm, six
//     products; the dropped terms Am.Gl, Al.Gm, Al.Gl are of order 2^-24
//     relative.  BF16 has FP32's exponent range, so no scaling either.
//
// Operands live in shared memory in the canonical K-major, no-swizzle layout
// of the tcgen05 matrix descriptors: core matrices of 8 rows x 16 bytes (8
// 16-bit or 4 32-bit values), row r's K-block j of a 32-value row at
// ((r / 8) * KB + j) * 128 + (r % 8) * 16 bytes with KB = 4 K-blocks (16-bit)
// or 8 (TF32) per row block, so the descriptor's leading-dimension offset
// (between K-adjacent core matrices) is 128 bytes and its stride-dimension
// offset (between row-adjacent ones) KB * 128.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include "fft_core.cuh"

namespace gbfft {

// Operand kinds of the split forms.
enum : int { kTcF16 = 0, kTcBF16 = 1, kTcTF32 = 2, kTcBF16X6 = 3 };

constexpr uint32_t kTcLbo = 128;  // bytes between K-adjacent core matrices

// Geometry of one operand kind for RADIX-point DFTs: 2 RADIX values per
// operand row (Re | Im), a (2 RADIX) x (2 RADIX) G.  RADIX 16 for every kind;
// RADIX 32 (the 32-sample tiles) for the 16-bit kinds.
template <int KIND, int RADIX = 16>
struct TcGeom {
    static_assert(RADIX == 16 || (RADIX == 32 && (KIND == kTcF16 || KIND == kTcBF16)),
                  "radix-32 operands: FP16 and BF16 hi+lo only");
    static constexpr int PARTS = KIND == kTcBF16X6 ? 3 : 2;  // operand parts: hi, (mid,) lo
    static constexpr int VALS = 2 * RADIX;                 // values per row
    static constexpr int ELEM = KIND == kTcTF32 ? 4 : 2;  // bytes per value
    static constexpr int ROW_BYTES = VALS * ELEM;          // one A row
    static constexpr int KB = ROW_BYTES / 16;              // K-blocks (core matrices) per row block
    static constexpr uint32_t SBO = KB * 128u;             // bytes between row-adjacent core matrices
    static constexpr int G_BYTES = VALS * ROW_BYTES;       // one G part (hi or lo)
    static constexpr int NKSTEP = ROW_BYTES / 32;          // MMAs along K (32 bytes of K each)
    // byte offset of the kind's [hi | lo (| mid)] parts in the G table
    static constexpr int GTAB_OFF = RADIX == 32 ? (KIND == kTcF16 ? 16384 : 32768)
                                                : (KIND == kTcF16 ? 0 : (KIND == kTcBF16 ? 4096 :
                                                                         (KIND == kTcTF32 ? 8192 : 49152)));
    // Instruction descriptor: D F32, A/B F16 (0) / BF16 (1) under kind::f16 or
    // TF32 (2) under kind::tf32, both K-major, M = 128, N = 2 RADIX.
    static constexpr uint32_t ATYPE = KIND == kTcF16 ? 0u : (KIND == kTcTF32 ? 2u : 1u);
    static constexpr uint32_t IDESC = (1u << 4) | (ATYPE << 7) | (ATYPE << 10) | (((uint32_t)VALS >> 3) << 17) |
                                      ((128u >> 4) << 24);
    // Byte offset of value (row, k) of a K-major no-swizzle operand.
    __host__ __device__ static constexpr uint32_t elem_offset(uint32_t row, uint32_t k) {
        return ((row >> 3) * KB + ((k * ELEM) >> 4)) * 128u + (row & 7) * 16u + ((k * ELEM) & 15u);
    }
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// tcgen05 shared-memory matrix descriptor (no swizzle, K-major).
__device__ __forceinline__ uint64_t tc_smem_desc(uint32_t saddr, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);        // bits 0-13: start address / 16
    d |= (uint64_t)(kTcLbo >> 4) << 16;             // bits 16-29: leading-dimension byte offset / 16
    d |= (uint64_t)(sbo >> 4) << 32;                // bits 32-45: stride-dimension byte offset / 16
    d |= (uint64_t)1 << 46;                         // bits 46-47: descriptor version 1
    return d;                                       // base offset 0, swizzle mode 0 (none)
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// One warp: allocate `ncols` TMEM columns, address written to *dst.
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

template <int KIND>
__device__ __forceinline__ void tc_mma(uint32_t d_taddr, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate) {
    if constexpr (KIND == kTcTF32) {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.u32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_taddr),
            "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
            : "memory");
    } else {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.u32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_taddr),
            "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
            : "memory");
    }
}
__device__ __forceinline__ void tc_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 32 consecutive TMEM columns of this thread's lane (32x32b shape).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// hi/lo parts of two values packed as 16-bit pairs (a in the low half):
// hi = RN16(v), lo = RN16(v - hi).  The remainder v - hi is exact in FP32 and
// comes from one mixed-precision FMA per value (hi * -1 + v, hi read as FP16
// or BF16 straight from the packed pair), so a pair costs two packed converts
// and two FMAs instead of a convert, a convert back and a subtract per value.
template <bool BF16>
__device__ __forceinline__ void tc_split2(float a, float b, uint32_t &hi, uint32_t &lo) {
    float la, lb;
    if constexpr (BF16) {
        asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(hi) : "f"(b), "f"(a));
        asm("{\n\t.reg .b16 h0, h1, m;\n\tmov.b32 {h0, h1}, %2;\n\tmov.b16 m, 0xBF80;\n\t"
            "fma.rn.f32.bf16 %0, h0, m, %3;\n\tfma.rn.f32.bf16 %1, h1, m, %4;\n\t}"
            : "=f"(la), "=f"(lb)
            : "r"(hi), "f"(a), "f"(b));
        asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(lo) : "f"(lb), "f"(la));
    } else {
        asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(hi) : "f"(b), "f"(a));
        asm("{\n\t.reg .b16 h0, h1, m;\n\tmov.b32 {h0, h1}, %2;\n\tmov.b16 m, 0xBC00;\n\t"
            "fma.rn.f32.f16 %0, h0, m, %3;\n\tfma.rn.f32.f16 %1, h1, m, %4;\n\t}"
            : "=f"(la), "=f"(lb)
            : "r"(hi), "f"(a), "f"(b));
        asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(lo) : "f"(lb), "f"(la));
    }
}

// Three-part BF16 split of two values packed as pairs (a in the low half):
// hi = RN(v), mid = RN(v - hi), lo = RN(v - hi - mid), each remainder exact in
// FP32 (mixed-precision FMAs as in tc_split2), so hi + mid + lo keeps 24
// significant bits of v.
__device__ __forceinline__ void tc_split3_bf16(float a, float b, uint32_t &hi, uint32_t &mid, uint32_t &lo) {
    float ra, rb, sa, sb;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(hi) : "f"(b), "f"(a));
    asm("{\n\t.reg .b16 h0, h1, m;\n\tmov.b32 {h0, h1}, %2;\n\tmov.b16 m, 0xBF80;\n\t"
        "fma.rn.f32.bf16 %0, h0, m, %3;\n\tfma.rn.f32.bf16 %1, h1, m, %4;\n\t}"
        : "=f"(ra), "=f"(rb)
        : "r"(hi), "f"(a), "f"(b));
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(mid) : "f"(rb), "f"(ra));
    asm("{\n\t.reg .b16 h0, h1, m;\n\tmov.b32 {h0, h1}, %2;\n\tmov.b16 m, 0xBF80;\n\t"
        "fma.rn.f32.bf16 %0, h0, m, %3;\n\tfma.rn.f32.bf16 %1, h1, m, %4;\n\t}"
        : "=f"(sa), "=f"(sb)
        : "r"(mid), "f"(ra), "f"(rb));
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(lo) : "f"(sb), "f"(sa));
}

// TF32 split: hi = x rounded to the nearest TF32 value (sign, exponent and 10
// explicit mantissa bits; ties away from zero), lo = x - hi, exact in FP32 and
// of either sign, |lo| <= 2^-11 |x|.  Rounding (rather than clearing the low
// bits) halves lo and, more importantly, makes the error of the tensor core's
// reduction of lo to TF32 unbiased: with truncation every lo shares x's sign
// and the dropped bits pile up coherently through the stages.
__device__ __forceinline__ void tc_split_tf32(float x, uint32_t &hi, uint32_t &lo) {
    hi = (__float_as_uint(x) + 0x1000u) & 0xFFFFE000u;
    lo = __float_as_uint(x - __uint_as_float(hi));
}

// Per-CTA state of the tensor-core DFT.
struct TcState {
    uint8_t *a_hi;       // [threads rows][32 values], canonical layout
    uint8_t *a_lo;
    uint8_t *a_mid;      // BF16 x 6 only
    const uint8_t *g_hi; // [32][32]
    const uint8_t *g_lo;
    const uint8_t *g_mid;
    uint64_t *bar;       // MMA completion barrier
    int *abort;          // shared flag: a completion wait gave up
    uint32_t *err;       // global error flag (set on timeout)
    uint32_t taddr;      // TMEM base (lane 0, first column)
    uint32_t parity;     // phase of *bar expected by the next wait
    uint32_t nmma;       // threads / 128
    uint32_t spin_limit;
};

// Forward RADIX-point DFT of x (natural order in, natural order out) on the
// tensor cores, RADIX = 16 or 32 (32: 16-bit kinds, the 32-sample tiles; the
// state's G parts must then be the radix-32 ones).  Must be called by all
// threads of the CTA at the same point.
template <int KIND, int RADIX>
__device__ __forceinline__ void tc_dft(float2 (&x)[RADIX], TcState &s) {
    using Gm = TcGeom<KIND, RADIX>;
    constexpr int V = Gm::VALS;
    const uint32_t r = threadIdx.x;
    float up = 1.f;
    if constexpr (KIND == kTcBF16X6) {
        // no scaling (BF16 has FP32's exponent range); three parts per value.
        // A shares its bytes with the FP32 exchange tile: every thread must
        // have finished reading its exchange inputs before any thread writes A.
        __syncthreads();
#pragma unroll
        for (int kb = 0; kb < V / 8; ++kb) {
            uint32_t hi[4], mi[4], lo[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int k = 8 * kb + 2 * i;
                const float2 a = x[k % RADIX], b = x[(k + 1) % RADIX];
                if (k < RADIX) tc_split3_bf16(a.x, b.x, hi[i], mi[i], lo[i]);
                else tc_split3_bf16(a.y, b.y, hi[i], mi[i], lo[i]);
            }
            const uint32_t off = Gm::elem_offset(r, 8 * kb);
            *(uint4 *)(s.a_hi + off) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
            *(uint4 *)(s.a_mid + off) = make_uint4(mi[0], mi[1], mi[2], mi[3]);
            *(uint4 *)(s.a_lo + off) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
        }
    } else if constexpr (KIND == kTcTF32) {
        // A shares its bytes with the FP32 exchange tile: every thread must
        // have finished reading its exchange inputs before any thread writes A.
        __syncthreads();
#pragma unroll
        for (int kb = 0; kb < V / 4; ++kb) {  // chunks of 4 K-values (16 bytes)
            uint32_t h[4], l[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int k = 4 * kb + i;
                tc_split_tf32(k < RADIX ? x[k].x : x[k - RADIX].y, h[i], l[i]);
            }
            const uint32_t off = Gm::elem_offset(r, 4 * kb);
            *(uint4 *)(s.a_hi + off) = make_uint4(h[0], h[1], h[2], h[3]);
            *(uint4 *)(s.a_lo + off) = make_uint4(l[0], l[1], l[2], l[3]);
        }
    } else {
        constexpr bool BF16 = KIND == kTcBF16;
        // 1. exact power-of-two scaling: largest |component| to [1, 2)
        float m = 0.f;
#pragma unroll
        for (int e = 0; e < RADIX; ++e) m = fmaxf(m, fmaxf(fabsf(x[e].x), fabsf(x[e].y)));
        int ex = 0;
        if (m > 0.f) {
            ex = (int)((__float_as_uint(m) >> 23) & 0xff) - 127;
            ex = ex < -126 ? -126 : ex;
        }
        ex = ex > 126 ? 126 : ex;
        const float down = __uint_as_float((uint32_t)(127 - ex) << 23);  // 2^-ex (ex in [-126, 126])
        up = __uint_as_float((uint32_t)(127 + ex) << 23);                // 2^ex
        // A shares its bytes with the FP32 exchange tile (see above).
        __syncthreads();
        // 2. split into hi/lo rows of A, 8 K-values (16 bytes) at a time:
        //    K-values 0..RADIX-1 are Re x, RADIX..2 RADIX-1 are Im x
#pragma unroll
        for (int kb = 0; kb < V / 8; ++kb) {
            uint32_t hi[4], lo[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int k = 8 * kb + 2 * i;
                const float2 a = x[k % RADIX], b = x[(k + 1) % RADIX];
                if (k < RADIX) tc_split2<BF16>(a.x * down, b.x * down, hi[i], lo[i]);
                else tc_split2<BF16>(a.y * down, b.y * down, hi[i], lo[i]);
            }
            const uint32_t off = Gm::elem_offset(r, 8 * kb);
            *(uint4 *)(s.a_hi + off) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
            *(uint4 *)(s.a_lo + off) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
        }
    }
    fence_proxy_async_smem();  // generic-proxy writes -> visible to the tensor core
    tc_fence_before();
    __syncthreads();
    // 3. one thread issues D = Ah.Gh + Ah.Gl + Al.Gh for every 128-row block
    //    (skipped once any CTA of the launch has given up waiting)
    if (r == 0) {
        if (*(volatile uint32_t *)s.err != 0u) *s.abort = 1;
        if (!*s.abort) {
            tc_fence_after();
            const uint32_t ah = smem_u32(s.a_hi), al = smem_u32(s.a_lo);
            const uint32_t gh = smem_u32(s.g_hi), gl = smem_u32(s.g_lo);
            for (uint32_t mb = 0; mb < s.nmma; ++mb) {
                const uint32_t d = s.taddr + mb * V;
                const uint32_t arow = mb * 128 * Gm::ROW_BYTES;  // 128 rows = 16 row blocks
                uint32_t acc = 0;
                if constexpr (KIND == kTcBF16X6) {
                    // hh, hm, mh, hl, lh, mm
                    const uint32_t am = smem_u32(s.a_mid), gm = smem_u32(s.g_mid);
                    const uint32_t pa[6] = {ah, ah, am, ah, al, am};
                    const uint32_t pg[6] = {gh, gm, gh, gl, gh, gm};
#pragma unroll
                    for (int part = 0; part < 6; ++part) {
#pragma unroll
                        for (uint32_t ks = 0; ks < (uint32_t)Gm::NKSTEP; ++ks) {
                            tc_mma<KIND>(d, tc_smem_desc(pa[part] + arow + ks * 2 * kTcLbo, Gm::SBO),
                                         tc_smem_desc(pg[part] + ks * 2 * kTcLbo, Gm::SBO), Gm::IDESC, acc);
                            acc = 1;
                        }
                    }
                } else {
#pragma unroll
                    for (int part = 0; part < 3; ++part) {
                        const uint32_t a = (part == 2 ? al : ah) + arow;
                        const uint32_t g = part == 1 ? gl : gh;
#pragma unroll
                        for (uint32_t ks = 0; ks < (uint32_t)Gm::NKSTEP; ++ks) {  // 32 bytes of K per MMA
                            tc_mma<KIND>(d, tc_smem_desc(a + ks * 2 * kTcLbo, Gm::SBO),
                                         tc_smem_desc(g + ks * 2 * kTcLbo, Gm::SBO), Gm::IDESC, acc);
                            acc = 1;
                        }
                    }
                }
            }
            tc_commit(s.bar);
            uint32_t polls = 0;
            while (!mbar_try_wait(s.bar, s.parity)) {
                if (++polls > s.spin_limit) {
                    *s.abort = 1;
                    atomicExch(s.err, 2u);
                    break;
                }
            }
        }
    }
    __syncthreads();
    s.parity ^= 1u;
    // 4. read this thread's row back: lanes of warp (r / 32) % 4, columns of
    //    block r / 128; 32 columns at a time (Re X, then Im X for RADIX 32)
    tc_fence_after();
    const uint32_t taddr = s.taddr + ((((r >> 5) & 3) * 32) << 16) + (r >> 7) * V;
    uint32_t d[32];
    if constexpr (RADIX == 16) {
        tmem_ld32(taddr, d);
#pragma unroll
        for (int q = 0; q < 16; ++q) x[q] = make_float2(__uint_as_float(d[q]) * up, __uint_as_float(d[16 + q]) * up);
    } else {
        tmem_ld32(taddr, d);
#pragma unroll
        for (int q = 0; q < 32; ++q) x[q].x = __uint_as_float(d[q]) * up;
        tmem_ld32(taddr + 32, d);
#pragma unroll
        for (int q = 0; q < 32; ++q) x[q].y = __uint_as_float(d[q]) * up;
    }
    tc_fence_before();
}

template <int KIND>
__device__ __forceinline__ void tc_dft16(float2 (&x)[16], TcState &s) { tc_dft<KIND, 16>(x, s); }

// Butterfly engine for pass_tile / rows_tile: radix-16 butterflies on the
// tensor cores, the radix 2/4/8 remainder on the FP32 pipes.
template <int KIND>
struct DftTc {
    TcState *s;
    template <int R>
    __device__ __forceinline__ void run(float2 (&x)[R]) {
        if constexpr (R == 16) tc_dft16<KIND>(x, *s);
        else Dft<R>::run(x);
    }
};

// Engine for the 32-sample tiles (16-bit kinds): radix-32 butterflies on the
// tensor cores (one per thread, so one operand row per thread), every smaller
// radix on the FP32 pipes.
template <int KIND>
struct DftTc32 {
    TcState *s;
    template <int R>
    __device__ __forceinline__ void run(float2 (&x)[R]) {
        if constexpr (R == 32) tc_dft<KIND, 32>(x, *s);
        else Dft<R>::run(x);
    }
};

// gbfft_precision value -> operand kind
__host__ __device__ constexpr int tc_kind_of_precision(int precision) {
    return precision == 2 ? kTcBF16 : (precision == 3 ? kTcTF32 : (precision == 4 ? kTcBF16X6 : kTcF16));
}

// Operand pointers of a TcState laid out as PARTS A parts of a_bytes each from
// `a`, and PARTS G parts from `g` (order hi, lo, then mid), for the geometry of
// RADIX-point DFTs.
template <int KIND, int RADIX = 16>
__device__ __forceinline__ void tc_state_parts(TcState &st, uint8_t *a, size_t a_bytes, const uint8_t *g) {
    using Gm = TcGeom<KIND, RADIX>;
    st.a_hi = a;
    st.a_lo = a + a_bytes;
    st.a_mid = Gm::PARTS == 3 ? a + 2 * a_bytes : nullptr;
    st.g_hi = g;
    st.g_lo = g + Gm::G_BYTES;
    st.g_mid = Gm::PARTS == 3 ? g + 2 * Gm::G_BYTES : nullptr;
}

constexpr uint32_t kTcSpinLimit = 1u << 20;  // polls of an MMA completion that takes microseconds

}  // namespace gbfft
