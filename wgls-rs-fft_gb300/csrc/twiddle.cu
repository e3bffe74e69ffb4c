// Device-side twiddle-table generation.  Every table entry is computed in
// FP64 with sincospi on an exactly representable argument (2 e / M, M a power
// of two) and rounded once to FP32.  This is the one step of the transform
// kept in FP64.  The reference builds its table on the host from an f32 angle
// (larsjoost/wgls-rs-fft src/lib.rs:761-769), whose rounding reaches ~ulp(2 pi).
#include "gbfft_internal.h"

namespace gbfft {

constexpr int kMaxSegments = 32;

struct SegmentList {
    TwiddleSegment s[kMaxSegments];
    int n;
};

__global__ void twiddle_fill_kernel(float2 *table, SegmentList list, uint64_t total) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    // locate the segment (segments are few; linear scan over prefix counts)
    uint64_t base = 0;
    int s = 0;
    for (; s < list.n; ++s) {
        if (i < base + list.s[s].count) break;
        base += list.s[s].count;
    }
    if (s >= list.n) return;
    const TwiddleSegment seg = list.s[s];
    const uint64_t li = i - base;
    uint64_t e;
    if (seg.kind == 0) {
        const uint64_t p = 1ull << seg.logp;
        e = (li / p + 1) * (li % p);
    } else {
        e = li << seg.logstride;
    }
    const uint64_t m = 1ull << seg.logm;
    e &= (m - 1);
    // angle = -2 pi e / M  ->  sincospi(-2 e / M); 2e/M is exact in FP64.
    const double x = -2.0 * (double)e / (double)m;
    double sn, cs;
    sincospi(x, &sn, &cs);
    table[seg.offset + li] = make_float2((float)cs, (float)sn);
}

cudaError_t twiddle_fill(float2 *table, const TwiddleSegment *segs, int nseg, cudaStream_t stream) {
    if (nseg <= 0) return cudaSuccess;
    if (nseg > kMaxSegments) return cudaErrorInvalidValue;
    SegmentList list;
    uint64_t total = 0;
    for (int i = 0; i < nseg; ++i) {
        list.s[i] = segs[i];
        total += segs[i].count;
    }
    list.n = nseg;
    if (total == 0) return cudaSuccess;
    const unsigned threads = 256;
    const uint64_t blocks = (total + threads - 1) / threads;
    twiddle_fill_kernel<<<(unsigned)blocks, threads, 0, stream>>>(table, list, total);
    return cudaGetLastError();
}

// Hann window w_i = 0.5 (1 - cos(2 pi i / (n - 1))) in FP64, rounded once to
// f32 (the formula of the reference's host-side window, tests/test_utils.rs:
// 39-48); n == 1 gives w_0 = 1.
__global__ void hann_fill_kernel(float *w, uint64_t n) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    w[i] = n == 1 ? 1.0f : (float)(0.5 * (1.0 - cospi(2.0 * (double)i / (double)(n - 1))));
}

cudaError_t hann_fill(float *w, uint64_t n, cudaStream_t stream) {
    const unsigned threads = 256;
    hann_fill_kernel<<<(unsigned)((n + threads - 1) / threads), threads, 0, stream>>>(w, n);
    return cudaGetLastError();
}

}  // namespace gbfft
