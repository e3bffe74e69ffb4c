// gbfft_c2c_device_noalloc: the two-pass transform (N = 2^15 .. 2^20) for
// callers that cannot allocate GPU memory.
//
// Who needs it: code that must not call cudaMalloc -- another library's
// allocator hook (an allocation from inside it would re-enter the allocator),
// a process whose device memory is fully reserved by a pool it does not own,
// or a real-time path where an allocation (and the implicit synchronisation
// cudaFree brings) would stall.  The regular entry points allocate on first
// use of a size (twiddle tables, a workspace); this one never calls
// cudaMalloc, cudaFree or any allocating library routine.  (It does launch
// kernels, so it is no more usable than any other CUDA call from places where
// CUDA forbids API calls, such as a stream's host callback.)
//
// Where its memory comes from: two file-scope device arrays of this library,
// a 32 MiB scratch buffer for the intermediate result between the two global
// passes, and a 256 KiB table area for the twiddles of every supported size.
// The CUDA driver reserves them when it loads this library's code on a GPU; every
// GPU that loads the library holds them until the process exits.
//
// Speed: it runs one launch per global pass with 16 samples a thread, the
// plain two-pass schedule.  The regular device entry runs both passes in one
// fused launch at these sizes (32 samples a thread from 2^17), which is
// 10-15 % faster; this entry trades that for needing no workspace.
//
// Set-up: the first call on each device (with that device current) looks up
// the arrays' device addresses with cudaGetSymbolAddress, fills the twiddle
// tables for all supported sizes and synchronises the caller's stream.  Make
// that first call before any stream capture.  Later calls only enqueue the two
// pass kernels on the caller's stream.  The set-up is done once per device for
// the life of the process: after a cudaDeviceReset the arrays are re-created
// empty and this entry must not be called again on that device.
//
// Sharing: every call on a device uses the same scratch array, which keeps
// whatever the previous call left in it.  Nothing in it needs to start at
// zero (the first pass overwrites every sample the second pass reads).  Calls
// that overlap on the GPU (different streams, or concurrent host threads) race
// on the scratch array: serialise them.
#include <atomic>
#include <mutex>
#include <vector>

#include "gbfft_internal.h"
#include "gbfft_plan.h"

namespace gbfft {
namespace {

constexpr int kNaMinLogN = 15;
constexpr int kNaMaxLogN = 20;
constexpr uint64_t kNaScratchSamples = 1ull << 22;  // 32 MiB of complex<f32>
constexpr uint64_t kNaTwiddleEntries = 1ull << 15;  // 256 KiB
constexpr int kNaMaxDevices = 64;

static __device__ __align__(256) float2 g_na_scratch[kNaScratchSamples];
static __device__ __align__(256) float2 g_na_twiddles[kNaTwiddleEntries];

struct NaPlan {
    PassDesc pass[2];
    uint64_t lo_off = 0, hi_off = 0;
    int split = 0;
};

// Per-device state.  `ready` is published with release order after the set-up
// has filled the rest, so a call that reads it true with acquire order sees
// the addresses and plans without taking the lock; `mu` serialises the set-up
// of one device only.
struct NaDevice {
    std::atomic<bool> ready{false};
    std::mutex mu;
    float2 *scratch = nullptr;
    float2 *tw = nullptr;
    NaPlan plan[kNaMaxLogN + 1];
};

NaDevice g_na_dev[kNaMaxDevices];

int na_setup(int dev, cudaStream_t stream, NaDevice &d) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_na_scratch) != cudaSuccess) {
        cudaGetLastError();
        return GBFFT_ERR_CUDA;
    }
    d.scratch = (float2 *)p;
    if (cudaGetSymbolAddress(&p, g_na_twiddles) != cudaSuccess) {
        cudaGetLastError();
        return GBFFT_ERR_CUDA;
    }
    d.tw = (float2 *)p;
    uint64_t off = 0;
    for (int L = kNaMinLogN; L <= kNaMaxLogN; ++L) {
        std::vector<int> parts = split_passes(L);
        if (parts.size() != 2) return GBFFT_ERR_UNSUPPORTED;
        std::vector<PassDesc> passes(2);
        int logp = 0;
        for (int i = 0; i < 2; ++i) {
            if (!pass_kernel_info(parts[i], i == 0, passes[i])) return GBFFT_ERR_UNSUPPORTED;
            if (pass_prepare(passes[i]) != cudaSuccess) return GBFFT_ERR_CUDA;
            passes[i].logp = logp;
            logp += parts[i];
        }
        std::vector<TwiddleSegment> segs;
        NaPlan &np = d.plan[L];
        off = multipass_segments(L, passes, off, segs, np.lo_off, np.hi_off, np.split);
        np.pass[0] = passes[0];
        np.pass[1] = passes[1];
        if (off > kNaTwiddleEntries) return GBFFT_ERR_UNSUPPORTED;
        if (twiddle_fill(d.tw, segs.data(), (int)segs.size(), stream) != cudaSuccess) return GBFFT_ERR_CUDA;
    }
    if (cudaStreamSynchronize(stream) != cudaSuccess) return GBFFT_ERR_CUDA;
    d.ready.store(true, std::memory_order_release);
    (void)dev;
    return GBFFT_OK;
}

}  // namespace
}  // namespace gbfft

using namespace gbfft;

extern "C" int gbfft_c2c_device_noalloc(const void *d_in, void *d_out, uint64_t n, uint64_t batch, int direction,
                                        void *stream) {
    if (direction != GBFFT_FORWARD && direction != GBFFT_INVERSE) return GBFFT_ERR_INVALID_ARGUMENT;
    if (n == 0 || (n & (n - 1)) != 0) return GBFFT_ERR_INVALID_SIZE;
    int L = 0;
    while ((1ull << L) < n) ++L;
    if (L < kNaMinLogN || L > kNaMaxLogN) return GBFFT_ERR_UNSUPPORTED;
    if (batch == 0) return GBFFT_OK;
    if (batch > kNaScratchSamples / n) return GBFFT_ERR_UNSUPPORTED;  // n * batch <= 2^22
    if (!d_in || !d_out) return GBFFT_ERR_INVALID_ARGUMENT;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNaMaxDevices) {
        cudaGetLastError();
        return GBFFT_ERR_NO_DEVICE;
    }
    cudaStream_t s = (cudaStream_t)stream;
    NaDevice &d = g_na_dev[dev];
    if (!d.ready.load(std::memory_order_acquire)) {
        std::lock_guard<std::mutex> lock(d.mu);
        if (!d.ready.load(std::memory_order_relaxed)) {
            int st = na_setup(dev, s, d);
            if (st != GBFFT_OK) return st;
        }
    }
    const NaPlan &np = d.plan[L];
    const bool inv = direction == GBFFT_INVERSE;
    const float scale = inv ? ldexpf(1.0f, -L) : 1.0f;
    // pass 0: input -> scratch (conjugate on load for the inverse)
    cudaError_t e = pass_launch(np.pass[0], (const float2 *)d_in, d.scratch, batch, L, d.tw + np.pass[0].sub_tw_offset,
                                d.tw + np.lo_off, d.tw + np.hi_off, np.split, inv ? -1.0f : 1.0f, 1.0f, 1.0f, s);
    if (e != cudaSuccess) return GBFFT_ERR_CUDA;
    // pass 1: scratch -> output (conjugate and scale by 1/N on store for the inverse)
    e = pass_launch(np.pass[1], d.scratch, (float2 *)d_out, batch, L, d.tw + np.pass[1].sub_tw_offset,
                    d.tw + np.lo_off, d.tw + np.hi_off, np.split, 1.0f, scale, inv ? -scale : 1.0f, s);
    if (e != cudaSuccess) return GBFFT_ERR_CUDA;
    return GBFFT_OK;
}
