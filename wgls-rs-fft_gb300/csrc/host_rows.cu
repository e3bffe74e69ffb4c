// Copies between the caller's host rows and a contiguous device batch, done by
// the GPU itself through the host's page tables.
//
// On a Grace-Blackwell node the GPU reaches ordinary pageable host memory
// (malloc, a Rust Vec, a numpy array) coherently over NVLink-C2C
// (cudaDevAttrPageableMemoryAccess).  The reference's fft() takes its batch as
// separately allocated rows (&[Vec<Complex<f32>>], src/lib.rs:433-438,
// 517-568); instead of staging them through pinned memory with host memcpy,
// these kernels gather the rows straight into HBM before the transform and
// scatter the result straight back into the caller's output rows, so no host
// core touches the data.  The host <-> device link is the only bound.
//
// A chunk is `rows` rows of 2^logn complex<f32> each.  Row r's host address is
// table[r] (a device copy of the caller's row pointers) or, with no table,
// base + r * row bytes (a contiguous pageable batch).  The device side is the
// chunk's rows back to back.  Each thread moves units of VEC bytes (16 when
// every row address is 16-byte aligned and rows hold at least two samples,
// else 8); four units are loaded before any is stored, and a grid of a few
// CTAs per SM keeps enough bytes in flight to cover the link's latency.
#include <algorithm>

#include "gbfft_internal.h"

namespace gbfft {
namespace {

template <int VEC>
struct Unit;
template <>
struct Unit<16> {
    using T = uint4;
};
template <>
struct Unit<8> {
    using T = uint2;
};

template <int VEC, bool TO_DEVICE>
__global__ void __launch_bounds__(256) host_rows_copy_kernel(const uint64_t *__restrict__ table, char *base,
                                                             int unit_log, uint64_t units, char *dev) {
    using T = typename Unit<VEC>::T;
    constexpr int kUnroll = 4;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t mask = (1ull << unit_log) - 1;  // units per row - 1
    for (uint64_t u0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; u0 < units; u0 += kUnroll * stride) {
        T v[kUnroll];
        T *host[kUnroll];
#pragma unroll
        for (int k = 0; k < kUnroll; ++k) {
            const uint64_t u = u0 + k * stride;
            host[k] = nullptr;
            if (u < units) {
                char *row = table ? (char *)table[u >> unit_log] : base + ((u >> unit_log) << unit_log) * VEC;
                host[k] = (T *)row + (u & mask);
                if (TO_DEVICE) v[k] = *host[k];
                else v[k] = ((const T *)dev)[u];
            }
        }
#pragma unroll
        for (int k = 0; k < kUnroll; ++k) {
            const uint64_t u = u0 + k * stride;
            if (u < units) {
                if (TO_DEVICE) ((T *)dev)[u] = v[k];
                else *host[k] = v[k];
            }
        }
    }
}

}  // namespace

cudaError_t host_rows_copy(const uint64_t *table, void *base, uint64_t rows, int logn, void *dev, bool to_device,
                           bool vec16, int sms, cudaStream_t stream) {
    const int unit_log = vec16 ? logn - 1 : logn;  // units of VEC bytes per row
    const uint64_t units = rows << unit_log;
    if (units == 0) return cudaSuccess;
    const uint64_t want = (units + 256 * 4 - 1) / (256 * 4);
    const unsigned grid = (unsigned)std::min<uint64_t>(want, (uint64_t)std::max(1, sms) * 2);
    char *b = (char *)base, *d = (char *)dev;
    if (vec16) {
        if (to_device) host_rows_copy_kernel<16, true><<<grid, 256, 0, stream>>>(table, b, unit_log, units, d);
        else host_rows_copy_kernel<16, false><<<grid, 256, 0, stream>>>(table, b, unit_log, units, d);
    } else {
        if (to_device) host_rows_copy_kernel<8, true><<<grid, 256, 0, stream>>>(table, b, unit_log, units, d);
        else host_rows_copy_kernel<8, false><<<grid, 256, 0, stream>>>(table, b, unit_log, units, d);
    }
    return cudaGetLastError();
}

}  // namespace gbfft
