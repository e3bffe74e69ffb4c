// Ragged batches: transforms of mixed power-of-two sizes (2^0 .. 2^18) and
// directions, packed back to back, in ONE persistent launch fed by a device
// work queue.  The reference has no such mode -- its GpuFft requires every row
// of a batch to have the same length (larsjoost/wgls-rs-fft src/lib.rs:526-533)
// -- so a ragged workload there is one call per size.
//
// Work items (all move 8192 samples through HBM once):
//   kind 0  G = 8192/N whole transforms of one size N <= 2^13 (single pass)
//   kind 1  first global pass of a transform of N = 2^14 .. 2^18, 16*NG columns
//   kind 2  second global pass of such a transform, 16*NG columns
// The queue mixes first passes and single-pass groups in proportion, and
// places the second pass of each transform a fixed number of items after its
// first pass (twice the CTAs in flight): late enough that it rarely waits,
// early enough that the first pass's output, stored with normal L2 priority,
// is still in L2 when it is read back.  Every CTA claims items in queue order
// with one atomicAdd (the next claim is made while the current item runs).
// A kind-2 item depends only on the kind-1 items of its transform, which sit
// earlier in the queue; the oldest unfinished item is therefore always some
// CTA's current item and can proceed, so every wait ends.  Each wait is still
// bounded (spin_limit polls with __nanosleep): on expiry the kernel sets an
// error flag, every CTA stops taking items, and the host reports
// GBFFT_ERR_TIMEOUT.
//
// Out of place, the first pass writes into the output buffer and the second
// pass rewrites the same samples in place; in place, the first pass writes to
// a workspace.  Producers publish with a CTA barrier, then one thread's
// __threadfence + atomicAdd; the consumer polls with ld.acquire.gpu and reads
// the intermediate with L1-bypassing loads.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "gbfft_internal.h"
#include "gbfft_plan.h"
#include "gbfft_ragged.h"
#include "fft_tc.cuh"
#include "fft_tiles.cuh"

namespace gbfft {

constexpr int kRagThreads = 512;
constexpr int kRagMaxLogN = 18;
constexpr int kRagRowsMaxLogN = 13;

struct RagXform {
    uint64_t offset;     // complex samples from the start of in/out
    uint64_t ws_offset;  // two-pass transforms: start of their workspace slice
    int32_t logn;
    int32_t dir;         // GBFFT_FORWARD / GBFFT_INVERSE
    uint32_t tiles1;     // two-pass transforms: number of first-pass items
    uint32_t pad;
};

struct RagItem {
    uint32_t kind;
    uint32_t a;  // kind 0: first index into order[]; kind 1/2: transform id
    uint32_t b;  // kind 0: transforms in the item;   kind 1/2: tile index
    uint32_t logn;
};

struct RagParams {
    const float2 *in;
    float2 *out;
    float2 *ws;
    int p1_to_out;  // out of place: first-pass output goes to `out` (ws unused)
    const RagItem *items;
    uint32_t nitems;
    uint32_t spin_limit;
    const RagXform *xf;
    const uint32_t *order;
    uint32_t *item_counter;
    uint32_t *done1;
    uint32_t *error;
    const float2 *sub[16];   // sub-pass tables of a length-2^L in-SMEM FFT
    const float2 *lo[kRagMaxLogN + 1];
    const float2 *hi[kRagMaxLogN + 1];
    int split[kRagMaxLogN + 1];
};

__host__ __device__ constexpr int rag_logr1(int L) { return L / 2 + (L & 1); }
__host__ __device__ constexpr int rag_logr2(int L) { return L / 2; }
__host__ __device__ constexpr int rag_groups(int logr) { return kRagThreads / (kCols << (logr - 4)); }

__device__ __forceinline__ uint32_t ld_acquire_gpu(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

template <int L>
__device__ __forceinline__ void rag_rows(const RagParams &P, const RagItem &it, float2 *smem) {
    constexpr int G = kRagThreads / SubCfg<L>::T;
    auto ref = [&](int g) {
        const bool act = (uint32_t)g < it.b;
        const RagXform x = P.xf[P.order[it.a + (act ? g : 0)]];
        const bool inv = x.dir == GBFFT_INVERSE;
        const float sc = inv ? ldexpf(1.0f, -L) : 1.0f;
        return RowRef{P.in + x.offset, P.out + x.offset, act, inv ? -1.0f : 1.0f, sc, inv ? -sc : 1.0f, 0u};
    };
    rows_tile<L, G>(ref, P.sub[L], smem, LoadOps{nullptr, 0u, 0.f, 0u});
}

// Returns false when the wait for the first pass gave up.  Eng: the
// butterfly engine (FP32 registers, or the tensor-core split form).
template <int L, bool FIRST, class Eng>
__device__ __forceinline__ bool rag_pass(const RagParams &P, const RagItem &it, float2 *smem, Eng &eng) {
    // the transform size is a template parameter: strided addresses and
    // twiddle indices become immediates
    constexpr int LOGR = FIRST ? rag_logr1(L) : rag_logr2(L);
    constexpr int NG = rag_groups(LOGR);
    __shared__ int s_abort;
    const RagXform x = P.xf[it.a];
    if (!FIRST) {
        if (threadIdx.x == 0) {
            uint32_t polls = 0;
            int abort = 0;
            while (ld_acquire_gpu(P.done1 + it.a) < x.tiles1) {
                if (++polls > P.spin_limit) {
                    atomicExch(P.error, 1u);
                    abort = 1;
                    break;
                }
                __nanosleep(256);
            }
            s_abort = abort;
        }
        __syncthreads();
        if (s_abort) return false;
    }
    const bool inv = x.dir == GBFFT_INVERSE;
    const float sc = inv ? ldexpf(1.0f, -L) : 1.0f;
    float2 *mid = P.p1_to_out ? P.out + x.offset : P.ws + x.ws_offset;
    PassArgs a;
    a.src = FIRST ? P.in + x.offset : mid;
    a.dst = FIRST ? mid : P.out + x.offset;
    a.logn = L;
    a.logp = FIRST ? 0 : rag_logr1(L);
    a.col0 = it.b * (uint32_t)(kCols * NG);
    a.tw_sub = P.sub[LOGR];
    a.tw_lo = P.lo[L];
    a.tw_hi = P.hi[L];
    a.tw_split = P.split[L];
    a.in_im = (FIRST && inv) ? -1.0f : 1.0f;
    a.out_re = FIRST ? 1.0f : sc;
    a.out_im = FIRST ? 1.0f : (inv ? -sc : 1.0f);
    a.coherent_load = !FIRST;
    a.keep_l2 = FIRST;
    a.row = 0;
    a.ops = LoadOps{nullptr, 0u, 0.f, 0u};
    pass_tile<LOGR, NG, FIRST, Eng, L, FIRST ? 0 : rag_logr1(L)>(a, smem, eng);
    return true;
}

template <bool FIRST, class Eng>
__device__ __forceinline__ bool rag_pass_dispatch(const RagParams &P, const RagItem &it, float2 *smem, Eng &eng) {
    switch (it.logn) {
        case 14: return rag_pass<14, FIRST>(P, it, smem, eng);
        case 15: return rag_pass<15, FIRST>(P, it, smem, eng);
        case 16: return rag_pass<16, FIRST>(P, it, smem, eng);
        case 17: return rag_pass<17, FIRST>(P, it, smem, eng);
        case 18: return rag_pass<18, FIRST>(P, it, smem, eng);
        default: return true;
    }
}

__device__ __forceinline__ uint32_t rag_claim(const RagParams &P) {
    return *(volatile uint32_t *)P.error != 0u ? 0xffffffffu : atomicAdd(P.item_counter, 1u);
}

// The queue loop shared by the FP32 and tensor-core kernels.  Single-pass
// groups always run on the FP32 pipes; two-pass items use `eng`.
template <class Eng>
__device__ __forceinline__ void rag_loop(const RagParams &P, float2 *smem_rag, Eng &eng) {
    // Claimed queue positions, double-buffered: slot `par` holds the current
    // item, slot par ^ 1 receives the next claim while the item runs.
    __shared__ uint32_t s_item[2];
    if (threadIdx.x == 0) s_item[0] = rag_claim(P);
    __syncthreads();
    for (uint32_t par = 0;; par ^= 1u) {
        const uint32_t idx = s_item[par];
        if (idx >= P.nitems) break;
        // The next claim's result stays in a register until the item's end:
        // storing it at once would hold warp 0 for the atomic's round trip.
        uint32_t next = 0;
        if (threadIdx.x == 0) next = rag_claim(P);
        const RagItem it = P.items[idx];
        bool ok = true;
        if (it.kind == 0) {
            switch (it.logn) {
#define GBFFT_RAG_ROWS(L) \
    case L: rag_rows<L>(P, it, smem_rag); break;
                GBFFT_RAG_ROWS(0) GBFFT_RAG_ROWS(1) GBFFT_RAG_ROWS(2) GBFFT_RAG_ROWS(3) GBFFT_RAG_ROWS(4)
                GBFFT_RAG_ROWS(5) GBFFT_RAG_ROWS(6) GBFFT_RAG_ROWS(7) GBFFT_RAG_ROWS(8) GBFFT_RAG_ROWS(9)
                GBFFT_RAG_ROWS(10) GBFFT_RAG_ROWS(11) GBFFT_RAG_ROWS(12) GBFFT_RAG_ROWS(13)
#undef GBFFT_RAG_ROWS
                default: break;
            }
        } else if (it.kind == 1) {
            ok = rag_pass_dispatch<true>(P, it, smem_rag, eng);
        } else {
            ok = rag_pass_dispatch<false>(P, it, smem_rag, eng);
        }
        if (!ok) break;
        // (slot par ^ 1 was last read before the previous item's final barrier)
        if (threadIdx.x == 0) s_item[par ^ 1u] = next;
        __syncthreads();  // the item's stores are issued; shared memory is free
        if (it.kind == 1 && threadIdx.x == 0) {
            // publish: the barrier ordered the CTA's stores before this fence
            __threadfence();
            atomicAdd(P.done1 + it.a, 1u);
        }
    }
}

// (gtab and off_g are the tensor-core kernel's; both kernels take the same arguments)
__global__ void __launch_bounds__(kRagThreads, 2) fft_ragged_kernel(RagParams P, const uint4 *, uint32_t) {
    extern __shared__ float2 smem_rag[];
    DftRegs eng;
    rag_loop(P, smem_rag, eng);
}

// Tensor-core split forms.  Shared memory: the item region (FP32 exchange
// tile + column twiddles, or a rows tile; the hi/lo A operands alias it while
// a tensor-core DFT runs), then the two G operand parts, then the mbarrier.
// TMEM (32 columns per 128 threads) is allocated once for the CTA's whole run.
// `off_g` (the item region rounded up to 1 KB, or twice the A operand bytes
// if larger) is passed by the host.
template <int KIND>
struct RagTcLayout {
    static constexpr int NMMA = kRagThreads / 128;
    static constexpr uint32_t TMEM_COLS = 128;
    static constexpr size_t A_BYTES = (size_t)kRagThreads * TcGeom<KIND>::ROW_BYTES;
    static_assert(NMMA * 32 <= (int)TMEM_COLS, "TMEM columns");
};

template <int KIND>
__global__ void __launch_bounds__(kRagThreads, (KIND == kTcTF32 ? 1 : 2))
fft_ragged_tc_kernel(RagParams P, const uint4 *__restrict__ gtab, uint32_t off_g) {
    using Lay = RagTcLayout<KIND>;
    using Gm = TcGeom<KIND>;
    extern __shared__ __align__(1024) uint8_t smem_rtc[];
    uint64_t *bar = (uint64_t *)(smem_rtc + off_g + Gm::PARTS * Gm::G_BYTES);
    uint32_t *s_taddr = (uint32_t *)(smem_rtc + off_g + Gm::PARTS * Gm::G_BYTES + 8);
    int *s_abort = (int *)(smem_rtc + off_g + Gm::PARTS * Gm::G_BYTES + 12);
    const int tid = threadIdx.x;
    const uint4 *gsrc = gtab + Gm::GTAB_OFF / 16;
    uint4 *gdst = (uint4 *)(smem_rtc + off_g);
    for (int i = tid; i < Gm::PARTS * Gm::G_BYTES / 16; i += kRagThreads) gdst[i] = gsrc[i];
    if (tid < 32) tmem_alloc(s_taddr, Lay::TMEM_COLS);
    if (tid == 0) {
        mbar_init(bar, 1);
        *s_abort = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    TcState st;
    tc_state_parts<KIND>(st, smem_rtc, Lay::A_BYTES, smem_rtc + off_g);
    st.bar = bar;
    st.abort = s_abort;
    st.err = P.error;  // a completion wait that gives up stops the whole launch
    st.taddr = *s_taddr;
    st.parity = 0;
    st.nmma = Lay::NMMA;
    st.spin_limit = kTcSpinLimit;
    DftTc<KIND> eng{&st};
    rag_loop(P, (float2 *)smem_rtc, eng);

    tc_fence_before();
    __syncthreads();
    if (tid == 0 && *s_abort) {
        // a wait gave up: let the MMAs that were issued finish before freeing TMEM
        for (uint32_t polls = 0; polls < kTcSpinLimit && !mbar_try_wait(bar, st.parity ^ 1u); ++polls) {
        }
    }
    __syncthreads();
    tc_fence_after();
    if (tid < 32) tmem_dealloc(st.taddr, Lay::TMEM_COLS);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

static size_t rag_smem_bytes() {
    size_t m = (size_t)kRagThreads * 17 * sizeof(float2);  // rows items (padded buffers: at most 17 a thread)
    for (int lr = 7; lr <= 9; ++lr) {
        const int ng = rag_groups(lr);
        m = std::max(m, ((size_t)ng * kCols * (1u << lr) + (size_t)ng * kCols * 17) * sizeof(float2));
    }
    return m;
}

template <int L>
static int rag_sub_segments(TwiddleSegment *out, uint64_t base) { return subcfg_segments<L>(out, base); }

static int sub_segments(int L, TwiddleSegment *out, uint64_t base, int &entries) {
    switch (L) {
#define GBFFT_RAG_SEG(X) \
    case X: entries = SubCfg<X>::tw_entries(); return rag_sub_segments<X>(out, base);
        GBFFT_RAG_SEG(0) GBFFT_RAG_SEG(1) GBFFT_RAG_SEG(2) GBFFT_RAG_SEG(3) GBFFT_RAG_SEG(4) GBFFT_RAG_SEG(5)
        GBFFT_RAG_SEG(6) GBFFT_RAG_SEG(7) GBFFT_RAG_SEG(8) GBFFT_RAG_SEG(9) GBFFT_RAG_SEG(10)
        GBFFT_RAG_SEG(11) GBFFT_RAG_SEG(12) GBFFT_RAG_SEG(13)
#undef GBFFT_RAG_SEG
        default: entries = 0; return 0;
    }
}

struct RaggedPlanImpl {
    int device = 0;
    uint32_t count = 0;
    uint32_t nitems = 0;
    uint64_t ws_samples = 0;
    uint64_t total_samples = 0;
    uint64_t max_extent = 0;  // one past the last sample any transform touches
    uint32_t spin_limit = 1u << 22;
    bool drop_producers = false;
    uint32_t lag_per_sm = 4;  // GBFFT_RAGGED_OPT_LAG
    bool dirty = true;        // items must be (re)uploaded
    std::vector<RagXform> xf;
    std::vector<RagItem> items;
    std::vector<uint32_t> order;
    std::vector<TwiddleSegment> segs;
    uint64_t tw_entries = 0;
    uint64_t sub_off[16] = {};
    uint64_t lo_off[kRagMaxLogN + 1] = {}, hi_off[kRagMaxLogN + 1] = {};
    int split[kRagMaxLogN + 1] = {};
    bool need_sub[16] = {}, need_2l[kRagMaxLogN + 1] = {};
    DeviceBuffer meta;        // xf | items | order | counters
    DeviceBuffer tw;
    DeviceBuffer ws;
    uint32_t *h_error = nullptr;  // pinned copy of the error flag
    size_t off_items = 0, off_order = 0, off_counters = 0, counters_bytes = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    const void *g_in = nullptr;
    void *g_out = nullptr;
    cudaStream_t capture_stream = nullptr;
    uint64_t launches = 0;
    int sms = 0;
    bool prepared = false;  // kernel attributes set
    int precision = GBFFT_PREC_FP32;
    void *gtab = nullptr;   // split form: the G operand parts (fft_passes_tc.cu)
};

static int rag_tc_kind(const RaggedPlanImpl &p) { return tc_kind_of_precision(p.precision); }
static size_t rag_tc_parts(int kind) { return kind == kTcBF16X6 ? 3 : 2; }
static size_t rag_tc_a_bytes(int kind) {
    return (size_t)kRagThreads * (kind == kTcTF32 ? TcGeom<kTcTF32>::ROW_BYTES : TcGeom<kTcF16>::ROW_BYTES);
}
static size_t rag_tc_off_g(const RaggedPlanImpl &p) {
    const int kind = rag_tc_kind(p);
    return (std::max(rag_smem_bytes(), rag_tc_parts(kind) * rag_tc_a_bytes(kind)) + 1023) & ~(size_t)1023;
}
static size_t rag_tc_smem_bytes(const RaggedPlanImpl &p) {
    const int kind = rag_tc_kind(p);
    const size_t g = kind == kTcTF32 ? TcGeom<kTcTF32>::G_BYTES : TcGeom<kTcF16>::G_BYTES;
    return rag_tc_off_g(p) + rag_tc_parts(kind) * g + 64;
}
static const void *rag_kernel(const RaggedPlanImpl &p) {
    switch (p.precision) {
        case GBFFT_PREC_TC_FP16: return (const void *)fft_ragged_tc_kernel<kTcF16>;
        case GBFFT_PREC_TC_BF16X3: return (const void *)fft_ragged_tc_kernel<kTcBF16>;
        case GBFFT_PREC_TC_TF32: return (const void *)fft_ragged_tc_kernel<kTcTF32>;
        case GBFFT_PREC_TC_BF16X6: return (const void *)fft_ragged_tc_kernel<kTcBF16X6>;
        default: return (const void *)fft_ragged_kernel;
    }
}
static size_t rag_kernel_smem(const RaggedPlanImpl &p) {
    return p.precision == GBFFT_PREC_FP32 ? rag_smem_bytes() : rag_tc_smem_bytes(p);
}

static void build_items(RaggedPlanImpl &p) {
    p.items.clear();
    p.order.clear();
    // kind 0: groups of whole transforms of one size, largest sizes first
    std::vector<std::vector<uint32_t>> by_size(kRagRowsMaxLogN + 1);
    std::vector<uint32_t> two;  // two-pass transforms, in descriptor order
    for (uint32_t i = 0; i < p.count; ++i) {
        const RagXform &x = p.xf[i];
        if (x.logn > kRagRowsMaxLogN) two.push_back(i);
        else by_size[x.logn].push_back(i);
    }
    std::vector<RagItem> rows;
    for (int L = kRagRowsMaxLogN; L >= 0; --L) {
        const uint32_t g = (uint32_t)(kRagThreads / (1 << (L < 4 ? 0 : L - 4)));
        const std::vector<uint32_t> &ids = by_size[L];
        for (size_t s = 0; s < ids.size(); s += g) {
            const uint32_t first = (uint32_t)p.order.size();
            const uint32_t n = (uint32_t)std::min<size_t>(g, ids.size() - s);
            for (uint32_t k = 0; k < n; ++k) p.order.push_back(ids[s + k]);
            rows.push_back(RagItem{0, first, n, (uint32_t)L});
        }
    }
    uint64_t total_p1 = 0;
    for (uint32_t i : two) total_p1 += p.xf[i].tiles1;
    // the second pass of a transform follows its first pass by `lag` items
    const uint64_t lag = (uint64_t)p.lag_per_sm * (uint64_t)std::max(1, p.sms);
    std::vector<std::pair<uint32_t, uint64_t>> pending;  // (transform, release position), FIFO
    size_t head = 0, ri = 0;
    uint64_t p1_seen = 0;
    auto emit_p2 = [&](uint32_t i) {
        const RagXform &x = p.xf[i];
        const int lr2 = rag_logr2(x.logn);
        const uint32_t tiles2 = (1u << (x.logn - lr2)) / (uint32_t)(kCols * rag_groups(lr2));
        for (uint32_t t = 0; t < tiles2; ++t) p.items.push_back(RagItem{2, i, t, (uint32_t)x.logn});
    };
    for (uint32_t i : two) {
        while (head < pending.size() && pending[head].second <= p.items.size()) emit_p2(pending[head++].first);
        const RagXform &x = p.xf[i];
        // test hook: nothing will publish the first pass
        if (!p.drop_producers)
            for (uint32_t t = 0; t < x.tiles1; ++t) p.items.push_back(RagItem{1, i, t, (uint32_t)x.logn});
        p1_seen += x.tiles1;
        pending.emplace_back(i, (uint64_t)p.items.size() + lag);
        // single-pass groups in proportion to the first passes issued so far
        const size_t want = (size_t)((double)rows.size() * (double)p1_seen / (double)total_p1);
        while (ri < want && ri < rows.size()) p.items.push_back(rows[ri++]);
    }
    while (ri < rows.size()) p.items.push_back(rows[ri++]);
    while (head < pending.size()) emit_p2(pending[head++].first);
    if (p.order.empty()) p.order.push_back(0);
    p.nitems = (uint32_t)p.items.size();
    p.dirty = true;
}

int ragged_plan_build(RaggedPlanImpl *&out, int device, const gbfft_ragged_desc *descs, uint32_t count,
                      int precision, std::string &why) {
    out = nullptr;
    RaggedPlanImpl *p = new RaggedPlanImpl();
    p->device = device;
    p->precision = precision;
    cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, device);
    p->count = count;
    p->xf.resize(count);
    uint64_t ws = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const gbfft_ragged_desc &d = descs[i];
        if (d.log2n > kRagMaxLogN) {
            why = "ragged transforms are limited to N <= 2^18 (descriptor " + std::to_string(i) + ")";
            delete p;
            return GBFFT_ERR_UNSUPPORTED;
        }
        if (d.direction != GBFFT_FORWARD && d.direction != GBFFT_INVERSE) {
            why = "descriptor " + std::to_string(i) + ": direction must be -1 or +1";
            delete p;
            return GBFFT_ERR_INVALID_ARGUMENT;
        }
        RagXform &x = p->xf[i];
        x.offset = d.offset;
        x.logn = (int32_t)d.log2n;
        x.dir = d.direction;
        x.ws_offset = 0;
        x.tiles1 = 0;
        x.pad = 0;
        const uint64_t n = 1ull << d.log2n;
        p->total_samples += n;
        p->max_extent = std::max(p->max_extent, d.offset + n);
        if ((int)d.log2n > kRagRowsMaxLogN) {
            const int lr1 = rag_logr1(d.log2n);
            x.ws_offset = ws;
            ws += n;
            x.tiles1 = (uint32_t)((1ull << (d.log2n - lr1)) / (uint64_t)(kCols * rag_groups(lr1)));
            p->need_sub[lr1] = p->need_sub[rag_logr2(d.log2n)] = true;
            p->need_2l[d.log2n] = true;
        } else {
            p->need_sub[d.log2n] = true;
        }
    }
    p->ws_samples = ws;
    // twiddle tables
    uint64_t off = 0;
    for (int L = 0; L < 16; ++L) {
        if (!p->need_sub[L]) continue;
        TwiddleSegment tmp[kMaxSub];
        int entries = 0;
        const int ns = sub_segments(L, tmp, off, entries);
        p->sub_off[L] = off;
        for (int s = 0; s < ns; ++s) p->segs.push_back(tmp[s]);
        off += (uint64_t)entries;
    }
    for (int L = kRagRowsMaxLogN + 1; L <= kRagMaxLogN; ++L) {
        if (!p->need_2l[L]) continue;
        const int s = (L + 1) / 2;
        p->split[L] = s;
        p->lo_off[L] = off;
        p->segs.push_back(TwiddleSegment{off, 1ull << s, 1, L, 0, 0});
        off += 1ull << s;
        p->hi_off[L] = off;
        p->segs.push_back(TwiddleSegment{off, 1ull << (L - s), 1, L, 0, s});
        off += 1ull << (L - s);
    }
    p->tw_entries = off;
    build_items(*p);
    out = p;
    return GBFFT_OK;
}

int ragged_plan_upload(RaggedPlanImpl &p, bool in_place, cudaStream_t stream, std::string &why) {
    if (!p.prepared) {
        cudaError_t e = cudaFuncSetAttribute(rag_kernel(p), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)rag_kernel_smem(p));
        if (e == cudaSuccess && p.precision != GBFFT_PREC_FP32) {
            e = cudaMalloc(&p.gtab, kTcGtabBytes);
            if (e == cudaSuccess) e = tc_gtab_fill(p.gtab, stream);
        }
        if (e != cudaSuccess) {
            why = cudaGetErrorString(e);
            return GBFFT_ERR_CUDA;
        }
        p.prepared = true;
    }
    if (!p.h_error) {
        if (cudaHostAlloc(&p.h_error, sizeof(uint32_t), cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            why = "pinned error flag";
            return GBFFT_ERR_OUT_OF_MEMORY;
        }
        *p.h_error = 0;
    }
    if (p.tw.ptr == nullptr && p.tw_entries > 0) {
        int st = p.tw.ensure(p.tw_entries * sizeof(float2), why);
        if (st != GBFFT_OK) return st;
        for (size_t s = 0; s < p.segs.size(); s += 16) {
            const int n = (int)std::min<size_t>(16, p.segs.size() - s);
            cudaError_t e = twiddle_fill((float2 *)p.tw.ptr, p.segs.data() + s, n, stream);
            if (e != cudaSuccess) {
                why = cudaGetErrorString(e);
                return GBFFT_ERR_CUDA;
            }
        }
    }
    if (in_place && p.ws_samples > 0) {  // out of place, the first pass writes into the output
        int st = p.ws.ensure(p.ws_samples * sizeof(float2), why);
        if (st != GBFFT_OK) return st;
    }
    if (!p.dirty) return GBFFT_OK;
    const size_t xf_bytes = p.xf.size() * sizeof(RagXform);
    const size_t it_bytes = p.items.size() * sizeof(RagItem);
    const size_t or_bytes = p.order.size() * sizeof(uint32_t);
    p.off_items = (xf_bytes + 255) & ~(size_t)255;
    p.off_order = (p.off_items + it_bytes + 255) & ~(size_t)255;
    p.off_counters = (p.off_order + or_bytes + 255) & ~(size_t)255;
    p.counters_bytes = (2 + (size_t)p.count) * sizeof(uint32_t);
    int st = p.meta.ensure(p.off_counters + p.counters_bytes, why);
    if (st != GBFFT_OK) return st;
    std::vector<char> host(p.off_counters, 0);
    if (xf_bytes) memcpy(host.data(), p.xf.data(), xf_bytes);
    if (it_bytes) memcpy(host.data() + p.off_items, p.items.data(), it_bytes);
    memcpy(host.data() + p.off_order, p.order.data(), or_bytes);
    cudaError_t e = cudaMemcpyAsync(p.meta.ptr, host.data(), host.size(), cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) {
        why = cudaGetErrorString(e);
        return GBFFT_ERR_CUDA;
    }
    p.dirty = false;
    return GBFFT_OK;
}

static RagParams rag_params(const RaggedPlanImpl &p, const void *in, void *out) {
    RagParams P;
    memset(&P, 0, sizeof P);
    char *m = (char *)p.meta.ptr;
    P.in = (const float2 *)in;
    P.out = (float2 *)out;
    P.ws = (float2 *)p.ws.ptr;
    P.p1_to_out = in != (const void *)out;
    P.items = (const RagItem *)(m + p.off_items);
    P.nitems = p.nitems;
    P.spin_limit = p.spin_limit;
    P.xf = (const RagXform *)m;
    P.order = (const uint32_t *)(m + p.off_order);
    uint32_t *ctr = (uint32_t *)(m + p.off_counters);
    P.item_counter = ctr;
    P.error = ctr + 1;
    P.done1 = ctr + 2;
    const float2 *tw = (const float2 *)p.tw.ptr;
    for (int L = 0; L < 16; ++L) P.sub[L] = p.need_sub[L] ? tw + p.sub_off[L] : nullptr;
    for (int L = 0; L <= kRagMaxLogN; ++L) {
        P.lo[L] = p.need_2l[L] ? tw + p.lo_off[L] : nullptr;
        P.hi[L] = p.need_2l[L] ? tw + p.hi_off[L] : nullptr;
        P.split[L] = p.split[L];
    }
    return P;
}

// Enqueue counters reset + persistent launch + error-flag readback on `s`.
static cudaError_t rag_enqueue(RaggedPlanImpl &p, const void *in, void *out, cudaStream_t s) {
    char *m = (char *)p.meta.ptr;
    cudaError_t e = cudaMemsetAsync(m + p.off_counters, 0, p.counters_bytes, s);
    if (e != cudaSuccess) return e;
    RagParams P = rag_params(p, in, out);
    if (p.nitems > 0) {
        // two resident CTAs per SM, one for the TF32 split form (its A operands
        // take twice the shared memory)
        const int per_sm = p.precision == GBFFT_PREC_TC_TF32 ? 1 : 2;
        const unsigned grid = (unsigned)std::max(1, std::min<int>(per_sm * p.sms, (int)p.nitems));
        const uint4 *gtab = (const uint4 *)p.gtab;
        uint32_t off_g = (uint32_t)rag_tc_off_g(p);
        void *args[] = {(void *)&P, (void *)&gtab, (void *)&off_g};
        e = cudaLaunchKernel(rag_kernel(p), dim3(grid), dim3(kRagThreads), args, rag_kernel_smem(p), s);
        if (e != cudaSuccess) return e;
    }
    return cudaMemcpyAsync(p.h_error, m + p.off_counters + sizeof(uint32_t), sizeof(uint32_t),
                           cudaMemcpyDeviceToHost, s);
}

int ragged_plan_execute(RaggedPlanImpl &p, const void *in, void *out, cudaStream_t stream, bool use_graph,
                        std::string &why) {
    int st = ragged_plan_upload(p, in == (const void *)out, stream, why);
    if (st != GBFFT_OK) return st;
    cudaError_t e;
    if (!use_graph) {
        e = rag_enqueue(p, in, out, stream);
        if (e != cudaSuccess) {
            why = cudaGetErrorString(e);
            return GBFFT_ERR_CUDA;
        }
        p.launches += p.nitems > 0 ? 1 : 0;
        return GBFFT_OK;
    }
    if (p.graph_exec && (p.g_in != in || p.g_out != out)) {
        cudaGraphExecDestroy(p.graph_exec);
        cudaGraphDestroy(p.graph);
        p.graph_exec = nullptr;
        p.graph = nullptr;
    }
    if (!p.graph_exec) {
        if (!p.capture_stream &&
            cudaStreamCreateWithFlags(&p.capture_stream, cudaStreamNonBlocking) != cudaSuccess) {
            why = "capture stream";
            return GBFFT_ERR_CUDA;
        }
        e = cudaStreamBeginCapture(p.capture_stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            cudaError_t e2 = rag_enqueue(p, in, out, p.capture_stream);
            e = cudaStreamEndCapture(p.capture_stream, &p.graph);
            if (e2 != cudaSuccess) e = e2;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&p.graph_exec, p.graph, 0);
        if (e != cudaSuccess) {
            why = std::string("graph capture: ") + cudaGetErrorString(e);
            return GBFFT_ERR_CUDA;
        }
        p.g_in = in;
        p.g_out = out;
    }
    e = cudaGraphLaunch(p.graph_exec, stream);
    if (e != cudaSuccess) {
        why = cudaGetErrorString(e);
        return GBFFT_ERR_CUDA;
    }
    p.launches += p.nitems > 0 ? 1 : 0;
    return GBFFT_OK;
}

int ragged_plan_wait(RaggedPlanImpl &p, cudaStream_t stream, std::string &why) {
    cudaError_t e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) {
        why = cudaGetErrorString(e);
        return GBFFT_ERR_CUDA;
    }
    if (p.h_error && *p.h_error) {
        why = "a ragged second-pass item gave up waiting for its first pass";
        *p.h_error = 0;
        return GBFFT_ERR_TIMEOUT;
    }
    return GBFFT_OK;
}

int ragged_plan_set(RaggedPlanImpl &p, int option, uint64_t value, std::string &why) {
    switch (option) {
        case GBFFT_RAGGED_OPT_SPIN_LIMIT:
            if (value == 0 || value > 0xffffffffull) {
                why = "spin limit must be in [1, 2^32)";
                return GBFFT_ERR_INVALID_ARGUMENT;
            }
            p.spin_limit = (uint32_t)value;
            break;
        case GBFFT_RAGGED_OPT_TEST_DROP_PRODUCERS:
            p.drop_producers = value != 0;
            build_items(p);
            break;
        case GBFFT_RAGGED_OPT_LAG:
            if (value < 1 || value > 64) {
                why = "lag must be in [1, 64] items per SM";
                return GBFFT_ERR_INVALID_ARGUMENT;
            }
            p.lag_per_sm = (uint32_t)value;
            build_items(p);
            break;
        default:
            why = "unknown ragged plan option";
            return GBFFT_ERR_INVALID_ARGUMENT;
    }
    if (p.graph_exec) {
        cudaGraphExecDestroy(p.graph_exec);
        cudaGraphDestroy(p.graph);
        p.graph_exec = nullptr;
        p.graph = nullptr;
    }
    return GBFFT_OK;
}

void ragged_plan_free(RaggedPlanImpl *p) {
    if (!p) return;
    if (p->graph_exec) cudaGraphExecDestroy(p->graph_exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    if (p->capture_stream) cudaStreamDestroy(p->capture_stream);
    if (p->gtab) cudaFree(p->gtab);
    if (p->h_error) cudaFreeHost(p->h_error);
    delete p;
}

uint64_t ragged_plan_samples(const RaggedPlanImpl &p) { return p.total_samples; }
uint64_t ragged_plan_extent(const RaggedPlanImpl &p) { return p.max_extent; }
uint32_t ragged_plan_items(const RaggedPlanImpl &p) { return p.nitems; }
uint64_t ragged_plan_launches(const RaggedPlanImpl &p) { return p.launches; }

}  // namespace gbfft
