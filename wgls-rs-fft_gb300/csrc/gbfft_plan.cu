// Plan construction and execution (see gbfft_plan.h).
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "gbfft_plan.h"

namespace gbfft {

// GBFFT_DEVICE_ALLOC_CAP=<bytes>: requests above it fail as if the device were
// out of memory (exercises the out-of-memory paths without exhausting a GPU).
static bool over_alloc_cap(size_t want) {
    const char *c = getenv("GBFFT_DEVICE_ALLOC_CAP");
    return c && *c && want > (size_t)strtoull(c, nullptr, 10);
}

int DeviceBuffer::ensure(size_t want, std::string &err) {
    if (bytes >= want) return GBFFT_OK;
    if (over_alloc_cap(want)) {
        err = std::string("device allocation of ") + std::to_string(want) + " bytes exceeds GBFFT_DEVICE_ALLOC_CAP";
        return GBFFT_ERR_OUT_OF_MEMORY;
    }
    release();
    cudaError_t e = cudaMalloc(&ptr, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        ptr = nullptr;
        err = std::string("device allocation of ") + std::to_string(want) + " bytes: " + cudaGetErrorString(e);
        return GBFFT_ERR_OUT_OF_MEMORY;
    }
    bytes = want;
    return GBFFT_OK;
}

void DeviceBuffer::release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}

Plan::~Plan() {
    if (tw) cudaFree(tw);
    if (gtab) cudaFree(gtab);
}

// Split log2 N into global-pass radices 2^5..2^max_logr, largest first, with
// as few passes as that allows.
std::vector<int> split_passes(int logn, int max_logr) {
    int p = (logn + max_logr - 1) / max_logr;
    if (p < 2) p = 2;
    std::vector<int> parts(p, logn / p);
    for (int i = 0; i < logn % p; ++i) parts[i] += 1;
    return parts;
}

uint64_t multipass_segments(int logn, std::vector<PassDesc> &passes, uint64_t off,
                            std::vector<TwiddleSegment> &segs, uint64_t &lo_off, uint64_t &hi_off, int &split) {
    for (PassDesc &d : passes) {
        d.sub_tw_offset = off;
        for (int s = 0; s < d.nseg; ++s) {
            TwiddleSegment seg = d.segs[s];
            seg.offset += off;
            segs.push_back(seg);
        }
        off += (uint64_t)d.tw_entries;
    }
    split = (logn + 1) / 2;
    lo_off = off;
    segs.push_back(TwiddleSegment{off, 1ull << split, 1, logn, 0, 0});
    off += 1ull << split;
    hi_off = off;
    segs.push_back(TwiddleSegment{off, 1ull << (logn - split), 1, logn, 0, split});
    off += 1ull << (logn - split);
    return off;
}

std::vector<PlanVariant> plan_candidates(int logn, int precision) {
    std::vector<PlanVariant> c;
    if (logn <= kRowsMaxLogN && precision != GBFFT_PREC_FP32) {
        c.push_back(PlanVariant{10});  // the split form's single-pass kernel
        return c;
    }
    if (logn <= kRowsMaxLogN) {
        // 2^11 samples per CTA (128 threads, 8 CTAs per SM) measured fastest
        // where a transform fits (N = 2^6 .. 2^11); one CTA per SM leaves no
        // other CTA to overlap with at 2^14, so prefetch helps there
        RowsKernelInfo ri;
        if (rows_kernel_info(logn, ri, 11)) c.push_back(PlanVariant{10, false, false, 11});
        // 32 samples a thread (radix-32 sub-passes, one exchange fewer): measured
        // fastest at 2^13 (330 vs 303 GSa/s); at 2^14 its 16 warps per SM lose to
        // the 32 of the 16-sample layout (253-262 vs 271), so there it is only a candidate
        const bool e32 = rows_kernel_info(logn, ri, 12, 5);
        if (e32 && logn == 13) c.push_back(PlanVariant{10, false, false, 0, 5});
        const bool big = logn >= 14;
        c.push_back(PlanVariant{10, big});
        c.push_back(PlanVariant{10, !big});
        if (rows_kernel_info(logn, ri, 13)) c.push_back(PlanVariant{10, false, false, 13});
        if (e32) {
            if (logn != 13) c.push_back(PlanVariant{10, false, false, 0, 5});
            c.push_back(PlanVariant{10, true, false, 0, 5});
        }
        FusedDesc fd;
        if (precision == GBFFT_PREC_FP32 && fused2_kernel_info(7, logn - 7, fd)) c.push_back(PlanVariant{10, false, true});
        return c;
    }
    const bool tc = precision != GBFFT_PREC_FP32;
    const int top = tc ? 9 : 10;
    FusedDesc fd;
    // three passes (L - 16, 8, 8) with the last two fused: the default where it exists
    if (!tc && fused3_kernel_info(logn, fd)) {
        // its first pass with 32 samples a thread where that exists (radix 2^9 /
        // 2^10: N = 2^25, 2^26), measured faster (2^26: 114.9 vs 112.9 GSa/s)
        // and on 8 columns a CTA (two CTAs per SM instead of one; same bits):
        // 2^26: 118.5 vs 115.9, 2^25: 131.0 vs 128.7 GSa/s
        PassDesc pd;
        const bool e32 = pass_kernel_info(logn - 16, true, pd, 5);
        // its 8-column input tile brought in by the TMA (four tiled copies a
        // tile instead of 32 8-byte loads a thread)
        if (pass_kernel_info(logn - 16, true, pd, 5, 3, true)) {
            c.push_back(PlanVariant{10, false, true, 3, 5, true});
            c.push_back(PlanVariant{10, true, true, 3, 5, true});  // persistent, next tile prefetched to L2
        }
        if (pass_kernel_info(logn - 16, true, pd, 5, 3)) c.push_back(PlanVariant{10, false, true, 3, 5});
        if (e32) c.push_back(PlanVariant{10, false, true, 0, 5});
        c.push_back(PlanVariant{10, false, true});
        // the lone first pass as a persistent tile loop with L2 prefetch of the next tile
        if (e32) c.push_back(PlanVariant{10, true, true, 0, 5});
        c.push_back(PlanVariant{10, true, true});
        if (pass_kernel_info(logn - 16, true, pd, 4, 3)) c.push_back(PlanVariant{10, false, true, 3, 4});
        if (pass_kernel_info(logn - 16, true, pd, 4, 3, true)) c.push_back(PlanVariant{10, false, true, 3, 4, true});
    }
    for (int m = top; m >= 7; --m) {
        const std::vector<int> parts = split_passes(logn, m);
        bool dup = false;
        for (const PlanVariant &v : c) dup |= split_passes(logn, v.max_logr) == parts;
        if (dup || parts[0] < 5) continue;
        // the pair with 32 samples a thread (radix-32 sub-passes) first where a
        // pass has radix 2^9 or more: measured faster at 2^17..2^20 (177 / 178.5 /
        // 150.7 / 155.9 against 174.7 / 166.2 / 145.6 / 144.7 GSa/s); after the
        // 16-sample pair otherwise.  The split form's 32-sample pair (one radix-32
        // tensor-core stage a pass) runs 2 CTAs per SM against 4 and measured
        // slower at 2^16 (FP16 135.6 vs 142.3 GSa/s): a candidate only
        const bool e32 = parts.size() == 2 && (tc ? fused_tc_kernel_info(parts[0], parts[1], precision, fd, 5)
                                                  : fused2_kernel_info(parts[0], parts[1], fd, 5));
        const bool e32_first = e32 && !tc && parts[0] >= 9;
        if (e32_first) c.push_back(PlanVariant{m, false, true, 0, 5});
        if (parts.size() == 2 && (tc ? fused_tc_kernel_info(parts[0], parts[1], precision, fd)
                                     : fused2_kernel_info(parts[0], parts[1], fd)))
            c.push_back(PlanVariant{m, false, true});
        if (e32 && !e32_first) c.push_back(PlanVariant{m, false, true, 0, 5});
        c.push_back(PlanVariant{m, false});
        if (!tc) c.push_back(PlanVariant{m, true});
    }
    return c;
}

int plan_build(Plan &p, int logn, int precision, const PlanVariant &v, cudaStream_t stream, std::string &why) {
    p.logn = logn;
    p.precision = precision;
    p.variant = v;
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&p.sms, cudaDevAttrMultiProcessorCount, dev);
    std::vector<TwiddleSegment> segs;
    cudaError_t e;
    const bool tc = precision != GBFFT_PREC_FP32;
    // N = 2^13, 2^14 may also run as a fused two-pass transform of radix-128
    // tiles (a tuner candidate)
    const bool small_fused = v.fused && !tc && (logn == 13 || logn == 14);
    if (tc && logn <= kRowsMaxLogN) {
        if (!rows_tc_kernel_info(logn, precision, p.rows)) {
            why = logn < 4 ? "the tensor-core split form needs N >= 16 (one radix-16 sub-pass)"
                           : "the TF32 split form runs single-pass sizes up to N = 2^13 (256 B of operands a thread)";
            return GBFFT_ERR_UNSUPPORTED;
        }
        if ((e = rows_tc_prepare(p.rows)) != cudaSuccess) {
            why = cudaGetErrorString(e);
            return GBFFT_ERR_CUDA;
        }
        segs.assign(p.rows.segs, p.rows.segs + p.rows.nseg);
        p.tw_entries = p.rows.tw_entries;
        if ((e = cudaMalloc(&p.gtab, kTcGtabBytes)) != cudaSuccess) {
            cudaGetLastError();
            why = cudaGetErrorString(e);
            return GBFFT_ERR_OUT_OF_MEMORY;
        }
        if ((e = tc_gtab_fill(p.gtab, stream)) != cudaSuccess) {
            why = cudaGetErrorString(e);
            return GBFFT_ERR_CUDA;
        }
    } else if (logn <= kRowsMaxLogN && !small_fused) {
        if (!rows_kernel_info(logn, p.rows, v.tile ? v.tile : 12, v.loge)) {
            why = "no single-pass kernel";
            return GBFFT_ERR_UNSUPPORTED;
        }
        if ((e = rows_prepare(p.rows)) != cudaSuccess) {
            why = cudaGetErrorString(e);
            return GBFFT_ERR_CUDA;
        }
        segs.assign(p.rows.segs, p.rows.segs + p.rows.nseg);
        p.tw_entries = p.rows.tw_entries;
    } else {
        p.multipass = true;
        p.needs_workspace = true;
        // the split form's radix-2^10 tile would not fit in shared memory
        std::vector<int> parts = split_passes(logn, tc ? std::min(9, v.max_logr) : v.max_logr);
        if (small_fused) parts = {7, logn - 7};
        const bool fused3 = v.fused && !tc && fused3_kernel_info(logn, p.fused);
        if (fused3) parts = {logn - 16, 8, 8};
        int logp = 0;
        for (size_t i = 0; i < parts.size(); ++i) {
            PassDesc d;
            const bool ok = tc ? pass_tc_kernel_info(parts[i], i == 0, precision, d)
                               : pass_kernel_info(parts[i], i == 0, d, (fused3 && i == 0) ? v.loge : 4,
                                                  (fused3 && i == 0 && v.tile) ? v.tile : 4, fused3 && i == 0 && v.tma);
            if (!ok) {
                why = std::string("no ") + (tc ? "tensor-core " : "") + "pass kernel for radix 2^" +
                      std::to_string(parts[i]);
                return GBFFT_ERR_UNSUPPORTED;
            }
            if ((e = pass_prepare(d)) != cudaSuccess) {
                why = cudaGetErrorString(e);
                return GBFFT_ERR_CUDA;
            }
            d.logp = logp;
            logp += parts[i];
            p.passes.push_back(d);
        }
        p.tw_entries = multipass_segments(logn, p.passes, 0, segs, p.tw_lo_offset, p.tw_hi_offset, p.tw_split);
        if (fused3 || (v.fused && parts.size() == 2 &&
                       (tc ? fused_tc_kernel_info(parts[0], parts[1], precision, p.fused, v.loge)
                           : fused2_kernel_info(parts[0], parts[1], p.fused, v.loge)))) {
            if (p.fused.loge != 4) {
                // the pair's tiles follow their own sub-pass schedule: append its tables
                int ea = 0, eb = 0;
                TwiddleSegment ts[kMaxSub];
                const int na = pass_sub_segments(parts[0], p.fused.loge, ts, p.tw_entries, ea);
                if (na < 0) {
                    why = "no sub-pass tables for the pair";
                    return GBFFT_ERR_UNSUPPORTED;
                }
                segs.insert(segs.end(), ts, ts + na);
                p.fused.sub_off_a = (int64_t)p.tw_entries;
                p.tw_entries += (uint64_t)ea;
                const int nb = pass_sub_segments(parts[1], p.fused.loge, ts, p.tw_entries, eb);
                if (nb < 0) {
                    why = "no sub-pass tables for the pair";
                    return GBFFT_ERR_UNSUPPORTED;
                }
                segs.insert(segs.end(), ts, ts + nb);
                p.fused.sub_off_b = (int64_t)p.tw_entries;
                p.tw_entries += (uint64_t)eb;
            }
            if ((e = fused_prepare(p.fused)) != cudaSuccess) {
                why = cudaGetErrorString(e);
                return GBFFT_ERR_CUDA;
            }
            p.has_fused = p.fused.ctas_per_sm > 0;
        }
        if (tc) {
            if ((e = cudaMalloc(&p.gtab, kTcGtabBytes)) != cudaSuccess) {
                cudaGetLastError();
                why = cudaGetErrorString(e);
                return GBFFT_ERR_OUT_OF_MEMORY;
            }
            if ((e = tc_gtab_fill(p.gtab, stream)) != cudaSuccess) {
                why = cudaGetErrorString(e);
                return GBFFT_ERR_CUDA;
            }
        }
    }
    if (p.tw_entries > 0) {
        if ((e = cudaMalloc(&p.tw, p.tw_entries * sizeof(float2))) != cudaSuccess) {
            cudaGetLastError();
            why = cudaGetErrorString(e);
            return GBFFT_ERR_OUT_OF_MEMORY;
        }
        if ((e = twiddle_fill(p.tw, segs.data(), (int)segs.size(), stream)) != cudaSuccess) {
            why = cudaGetErrorString(e);
            return GBFFT_ERR_CUDA;
        }
    }
    return GBFFT_OK;
}

int plan_execute_tables(const Plan &p, const uint64_t *tab_in, const uint64_t *tab_out, float2 *work,
                        uint64_t batch, int direction, uint32_t *err, cudaStream_t stream, uint64_t &launches,
                        std::string &why, LoadOps ops, DeviceBuffer *ctr) {
    launches = 0;
    if (batch == 0) return GBFFT_OK;
    if (!p.has_fused || p.passes.size() != 2 || !ctr || batch * p.fused.groups_per_transform > 0x7fffffffull) {
        why = "row tables need a fused two-pass plan";
        return GBFFT_ERR_UNSUPPORTED;
    }
    cudaError_t e;
    const uint64_t ngroups = batch * p.fused.groups_per_transform;
    const size_t want = (2 + (size_t)ngroups) * sizeof(uint32_t);
    if (ctr->bytes < want) {
        int st = ctr->ensure(want, why);
        if (st != GBFFT_OK) return st;
        // the kernel leaves the block zeroed; a new block starts zeroed
        if ((e = cudaMemsetAsync(ctr->ptr, 0, ctr->bytes, stream)) != cudaSuccess) {
            why = cudaGetErrorString(e);
            return GBFFT_ERR_CUDA;
        }
    }
    const bool inv = direction == GBFFT_INVERSE;
    const float scale = inv ? ldexpf(1.0f, -p.logn) : 1.0f;
    const float2 *tw_a = p.fused.sub_off_a >= 0 ? p.tw + p.fused.sub_off_a : p.tw + p.passes[0].sub_tw_offset;
    const float2 *tw_b = p.fused.sub_off_b >= 0 ? p.tw + p.fused.sub_off_b : p.tw + p.passes[1].sub_tw_offset;
    e = fused_launch(p.fused, nullptr, work, batch, tw_a, tw_b, p.tw + p.tw_lo_offset, p.tw + p.tw_hi_offset,
                     inv ? -1.0f : 1.0f, scale, inv ? -scale : 1.0f, ops, (uint32_t *)ctr->ptr, err, p.sms, stream,
                     p.gtab, tab_in, tab_out);
    if (e != cudaSuccess) {
        why = cudaGetErrorString(e);
        return GBFFT_ERR_CUDA;
    }
    launches = 1;
    return GBFFT_OK;
}

int plan_execute(const Plan &p, const float2 *in, float2 *out, uint64_t batch, int direction, DeviceBuffer &ws,
                 uint32_t *err, cudaStream_t stream, uint64_t &launches, std::string &why, LoadOps ops,
                 DeviceBuffer *ctr) {
    launches = 0;
    if (batch == 0) return GBFFT_OK;
    cudaError_t e;
    // Fused pass pair: both passes of a two-pass transform (out of place
    // only: its first pass writes into `out` while other tiles still read
    // `in`), or the last two of three after the first pass into the workspace.
    const bool pair3 = p.has_fused && p.passes.size() == 3;
    const bool pair2 = p.has_fused && p.passes.size() == 2 && (const void *)in != (const void *)out;
    const uint64_t ngroups = batch * p.fused.groups_per_transform;
    if ((pair2 || pair3) && ctr && ngroups <= 0x7fffffffull) {
        const size_t want = (2 + (size_t)ngroups) * sizeof(uint32_t);
        if (ctr->bytes < want) {
            int st = ctr->ensure(want, why);
            if (st != GBFFT_OK) return st;
            // the kernel leaves the block zeroed; a new block starts zeroed
            if ((e = cudaMemsetAsync(ctr->ptr, 0, ctr->bytes, stream)) != cudaSuccess) {
                why = cudaGetErrorString(e);
                return GBFFT_ERR_CUDA;
            }
        }
        const bool inv = direction == GBFFT_INVERSE;
        const float scale = inv ? ldexpf(1.0f, -p.logn) : 1.0f;
        const float2 *pair_in = in;
        const size_t a = pair3 ? 1 : 0;  // index of the pair's first pass
        if (pair3) {
            int st = ws.ensure(((size_t)batch << p.logn) * sizeof(float2), why);
            if (st != GBFFT_OK) return st;
            const PassDesc &d0 = p.passes[0];
            e = pass_launch(d0, in, (float2 *)ws.ptr, batch, p.logn, p.tw + d0.sub_tw_offset, p.tw + p.tw_lo_offset,
                            p.tw + p.tw_hi_offset, p.tw_split, inv ? -1.0f : 1.0f, 1.0f, 1.0f, stream,
                            p.variant.persistent, p.sms, ops, err);
            if (e != cudaSuccess) {
                why = cudaGetErrorString(e);
                return GBFFT_ERR_CUDA;
            }
            ++launches;
            pair_in = (const float2 *)ws.ptr;
        }
        const float2 *tw_a = p.fused.sub_off_a >= 0 ? p.tw + p.fused.sub_off_a : p.tw + p.passes[a].sub_tw_offset;
        const float2 *tw_b =
            p.fused.sub_off_b >= 0 ? p.tw + p.fused.sub_off_b : p.tw + p.passes[a + 1].sub_tw_offset;
        e = fused_launch(p.fused, pair_in, out, batch, tw_a, tw_b, p.tw + p.tw_lo_offset, p.tw + p.tw_hi_offset,
                         (inv && !pair3) ? -1.0f : 1.0f, scale, inv ? -scale : 1.0f,
                         pair3 ? LoadOps{nullptr, 0u, 0.f, 0u} : ops, (uint32_t *)ctr->ptr, err, p.sms, stream,
                         p.gtab);
        if (e != cudaSuccess) {
            why = cudaGetErrorString(e);
            return GBFFT_ERR_CUDA;
        }
        ++launches;
        return GBFFT_OK;
    }
    if (!p.multipass) {
        e = p.precision != GBFFT_PREC_FP32
                ? rows_tc_launch(p.rows, in, out, batch, p.tw, direction, p.logn, p.gtab, err, stream, ops)
                : rows_launch(p.rows, in, out, batch, p.tw, direction, p.logn, p.variant.persistent, p.sms, stream,
                              ops);
        if (e != cudaSuccess) {
            why = cudaGetErrorString(e);
            return GBFFT_ERR_CUDA;
        }
        launches = 1;
        return GBFFT_OK;
    }
    const int np = (int)p.passes.size();
    const size_t bytes = ((size_t)batch << p.logn) * sizeof(float2);
    // Buffer routing.  Pass np-1 may run in place (each CTA reads and writes
    // the same samples); earlier passes must not.  Option A ends pass np-2 in
    // `out`, option B in the workspace.
    std::vector<const float2 *> src(np);
    std::vector<float2 *> dst(np);
    auto route = [&](bool last_in_place, float2 *w) {
        for (int i = 0; i < np - 1; ++i) {
            const bool to_out = ((np - 2 - i) % 2 == 0) == last_in_place;
            dst[i] = to_out ? out : w;
        }
        dst[np - 1] = out;
        src[0] = in;
        for (int i = 1; i < np; ++i) src[i] = dst[i - 1];
    };
    bool need_ws = true;
    route(true, nullptr);
    if (np == 2 && (const void *)in != (const void *)out) need_ws = false;
    if (need_ws) {
        int st = ws.ensure(bytes, why);
        if (st != GBFFT_OK) return st;
        float2 *w = (float2 *)ws.ptr;
        route(true, w);
        if ((const void *)src[0] == (const void *)dst[0]) route(false, w);
    }
    const bool inv = direction == GBFFT_INVERSE;
    const float scale = inv ? ldexpf(1.0f, -p.logn) : 1.0f;
    for (int i = 0; i < np; ++i) {
        const PassDesc &d = p.passes[i];
        const float in_im = (i == 0 && inv) ? -1.0f : 1.0f;
        const float out_re = (i == np - 1) ? scale : 1.0f;
        const float out_im = (i == np - 1 && inv) ? -scale : 1.0f;
        if (d.tc)
            e = pass_tc_launch(d, src[i], dst[i], batch, p.logn, p.tw + d.sub_tw_offset, p.tw + p.tw_lo_offset,
                               p.tw + p.tw_hi_offset, p.tw_split, in_im, out_re, out_im, p.gtab, err, stream,
                               i == 0 ? ops : LoadOps{nullptr, 0u, 0.f, 0u});
        else
            e = pass_launch(d, src[i], dst[i], batch, p.logn, p.tw + d.sub_tw_offset, p.tw + p.tw_lo_offset,
                            p.tw + p.tw_hi_offset, p.tw_split, in_im, out_re, out_im, stream, p.variant.persistent,
                            p.sms, i == 0 ? ops : LoadOps{nullptr, 0u, 0.f, 0u});
        if (e != cudaSuccess) {
            why = cudaGetErrorString(e);
            return GBFFT_ERR_CUDA;
        }
        ++launches;
    }
    return GBFFT_OK;
}

}  // namespace gbfft
