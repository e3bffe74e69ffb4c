// Host-side check of the shared-memory index maps of the single-pass tile
// (fft_tiles.cuh: subpass_out_pos, swz) and of the global-pass tile
// (subpass_out_pos, xch_idx, stage_idx), compiled for the host by nvcc and run
// by tests/test_tile_maps.py.  Single-pass tiles (N = 2^LOGN, 2^LE samples a
// thread): every exchange is a bijection onto the transform's N slots, read back
// where it was written; worst wavefronts of a warp (which spans 32 / T
// transforms when T < 32).  Prints: rows LOGN LE ok wavefronts.
// Global-pass tiles (radix 2^LOGR, 2^LE samples a thread, 2^CL columns):
//   * each exchange after a sub-pass writes every slot of the [row][column]
//     tile once, in bounds, and the next sub-pass reads back (column, row);
//   * a first pass's output staging is a bijection, read back in linear order
//     (as 16-byte pairs when CL < 4);
//   * the worst shared-memory wavefronts of one warp access (8-byte lanes need
//     at least 2, 16-byte lanes 4).
// Prints: pass LOGR LE CL ok exchange_wavefronts staging_wavefronts pair_wavefronts.
#include <algorithm>
#include <cstdio>
#include <map>
#include <set>
#include <vector>

#include "fft_tiles.cuh"
using namespace gbfft;

static int wavefronts(const std::vector<int> &idx) {  // float2 indices of one warp access
    std::map<int, std::set<int>> banks;
    for (int a : idx)
        for (int w = 2 * a; w <= 2 * a + 1; ++w) banks[w % 32].insert(w);
    size_t m = 0;
    for (auto &kv : banks) m = std::max(m, kv.second.size());
    return (int)m;
}

template <int LOGR, int LE, int CL, int I>
void check_exchanges(bool &ok, int &worst) {
    using C = SubCfg<LOGR, LE>;
    if constexpr (I < C::NSUB) {
        constexpr int PR = C::logr(I - 1), PP = C::logp(I - 1);
        constexpr int R = C::N, T = C::T, E = C::E, COLS = 1 << CL, THREADS = COLS * T;
        std::vector<int> owner(COLS * R, -1);
        for (int tid = 0; tid < THREADS; ++tid) {
            const int c = tid & (COLS - 1), t = tid >> CL;
            for (int b = 0; b < (E >> PR); ++b)
                for (int q = 0; q < (1 << PR); ++q) {
                    const int pos = subpass_out_pos<PR, PP, C::LOGT>(t, b, q);
                    const int i = xch_idx<CL, PP, PR>(pos, c);
                    if (pos < 0 || pos >= R || i < 0 || i >= COLS * R || owner[i] != -1) ok = false;
                    else owner[i] = pos * COLS + c;
                }
        }
        for (int tid = 0; tid < THREADS; ++tid) {
            const int c = tid & (COLS - 1), t = tid >> CL;
            for (int e = 0; e < E; ++e) {
                const int i = xch_idx<CL, PP, PR>(t + T * e, c);
                if (i < 0 || i >= COLS * R || owner[i] != (t + T * e) * COLS + c) ok = false;
            }
        }
        for (int w = 0; w < THREADS / 32; ++w) {
            for (int b = 0; b < (E >> PR); ++b)
                for (int q = 0; q < (1 << PR); ++q) {
                    std::vector<int> a;
                    for (int l = 0; l < 32; ++l) {
                        const int tid = 32 * w + l, c = tid & (COLS - 1), t = tid >> CL;
                        a.push_back(xch_idx<CL, PP, PR>(subpass_out_pos<PR, PP, C::LOGT>(t, b, q), c));
                    }
                    worst = std::max(worst, wavefronts(a));
                }
            for (int e = 0; e < E; ++e) {
                std::vector<int> a;
                for (int l = 0; l < 32; ++l) {
                    const int tid = 32 * w + l, c = tid & (COLS - 1), t = tid >> CL;
                    a.push_back(xch_idx<CL, PP, PR>(t + T * e, c));
                }
                worst = std::max(worst, wavefronts(a));
            }
        }
        check_exchanges<LOGR, LE, CL, I + 1>(ok, worst);
    }
}

template <int LOGR, int LE, int CL>
void check_tile() {
    using C = SubCfg<LOGR, LE>;
    constexpr int R = C::N, T = C::T, E = C::E, COLS = 1 << CL, THREADS = COLS * T;
    static_assert(THREADS % 32 == 0, "whole warps");
    bool ok = true;
    int wx = 0, ws = 0, wp = 0;
    check_exchanges<LOGR, LE, CL, 1>(ok, wx);
    // first-pass output staging: the last sub-pass writes, the stores read linearly
    constexpr int LR = C::logr(C::NSUB - 1), LP = C::logp(C::NSUB - 1), NB = E >> LR;
    std::vector<int> owner(COLS * R, -1);
    for (int tid = 0; tid < THREADS; ++tid) {
        const int c = tid & (COLS - 1), t = tid >> CL;
        for (int bb = 0; bb < NB; ++bb)
            for (int q = 0; q < (1 << LR); ++q) {
                const int pos = subpass_out_pos<LR, LP, C::LOGT>(t, bb, q);
                const int i = stage_idx<CL, LOGR>(c, pos);
                if (pos < 0 || pos >= R || i < 0 || i >= COLS * R || owner[i] != -1) ok = false;
                else owner[i] = c * R + pos;
            }
    }
    for (int w = 0; w < THREADS / 32; ++w)
        for (int bb = 0; bb < NB; ++bb)
            for (int q = 0; q < (1 << LR); ++q) {
                std::vector<int> a;
                for (int l = 0; l < 32; ++l) {
                    const int tid = 32 * w + l, c = tid & (COLS - 1), t = tid >> CL;
                    a.push_back(stage_idx<CL, LOGR>(c, subpass_out_pos<LR, LP, C::LOGT>(t, bb, q)));
                }
                ws = std::max(ws, wavefronts(a));
            }
    const int per = CL < kColsLog ? 2 : 1;  // samples a lane reads and stores at once
    for (int w = 0; w < THREADS / 32; ++w)
        for (int e = 0; e < E / per; ++e) {
            std::vector<int> a;
            for (int l = 0; l < 32; ++l) {
                const int lin = per * (32 * w + l + COLS * T * e);
                const int cc = lin >> LOGR, q = lin & (R - 1);
                for (int k = 0; k < per; ++k) {
                    const int i = stage_idx<CL, LOGR>(cc, q + k);
                    if (i < 0 || i >= COLS * R || owner[i] != lin + k) ok = false;
                    if (k == 1 && i != stage_idx<CL, LOGR>(cc, q) + 1) ok = false;
                    a.push_back(i);
                }
                if (per == 2 && (stage_idx<CL, LOGR>(cc, q) & 1)) ok = false;  // 16-byte aligned pair
            }
            wp = std::max(wp, wavefronts(a));
        }
    printf("pass %d %d %d %d %d %d %d\n", LOGR, LE, CL, ok ? 1 : 0, wx, ws, wp);
}

template <int LOGN, int LE, int I>
void check_rows_exchanges(bool &ok, int &worst) {
    using C = SubCfg<LOGN, LE>;
    if constexpr (I < C::NSUB) {
        constexpr int PR = C::logr(I - 1), PP = C::logp(I - 1);
        constexpr int N = C::N, T = C::T, E = C::E;
        constexpr int G = T >= 32 ? 1 : 32 / T;  // transforms one warp spans
        std::vector<int> owner(N, -1);
        for (int t = 0; t < T; ++t)
            for (int b = 0; b < (E >> PR); ++b)
                for (int q = 0; q < (1 << PR); ++q) {
                    const int pos = subpass_out_pos<PR, PP, C::LOGT>(t, b, q);
                    const int i = swz<C::LOGE>(pos, PP);
                    if (pos < 0 || pos >= N || i < 0 || i >= N || owner[i] != -1) ok = false;
                    else owner[i] = pos;
                }
        for (int t = 0; t < T; ++t)
            for (int e = 0; e < E; ++e) {
                const int i = swz<C::LOGE>(t + T * e, PP);
                if (i < 0 || i >= N || owner[i] != t + T * e) ok = false;
            }
        for (int w = 0; w < (G * T) / 32 || w == 0; ++w) {
            for (int b = 0; b < (E >> PR); ++b)
                for (int q = 0; q < (1 << PR); ++q) {
                    std::vector<int> a;
                    for (int l = 0; l < 32; ++l) {
                        const int tid = 32 * w + l, g = tid / T, t = tid % T;
                        a.push_back(g * rows_buf_stride<LOGN, LE>() + swz<C::LOGE>(subpass_out_pos<PR, PP, C::LOGT>(t, b, q), PP));
                    }
                    worst = std::max(worst, wavefronts(a));
                }
            for (int e = 0; e < E; ++e) {
                std::vector<int> a;
                for (int l = 0; l < 32; ++l) {
                    const int tid = 32 * w + l, g = tid / T, t = tid % T;
                    a.push_back(g * rows_buf_stride<LOGN, LE>() + swz<C::LOGE>(t + T * e, PP));
                }
                worst = std::max(worst, wavefronts(a));
            }
            if (T > 32 && w + 1 >= T / 32) break;
        }
        check_rows_exchanges<LOGN, LE, I + 1>(ok, worst);
    }
}

template <int LOGN, int LE>
void check_rows() {
    bool ok = true;
    int w = 0;
    check_rows_exchanges<LOGN, LE, 1>(ok, w);
    printf("rows %d %d %d %d\n", LOGN, LE, ok ? 1 : 0, w);
}

int main() {
    check_rows<4, 4>();
    check_rows<5, 4>();
    check_rows<6, 4>();
    check_rows<7, 4>();
    check_rows<8, 4>();
    check_rows<9, 4>();
    check_rows<10, 4>();
    check_rows<11, 4>();
    check_rows<12, 4>();
    check_rows<13, 4>();
    check_rows<14, 4>();
    check_rows<13, 5>();
    check_rows<14, 5>();
    // 16 columns: every pass radix with 16 samples a thread, 2^7..2^10 with 32
    check_tile<5, 4, 4>();
    check_tile<6, 4, 4>();
    check_tile<7, 4, 4>();
    check_tile<8, 4, 4>();
    check_tile<9, 4, 4>();
    check_tile<10, 4, 4>();
    check_tile<7, 5, 4>();
    check_tile<8, 5, 4>();
    check_tile<9, 5, 4>();
    check_tile<10, 5, 4>();
    // 8 columns: the first pass of N = 2^25 / 2^26
    check_tile<9, 4, 3>();
    check_tile<9, 5, 3>();
    check_tile<10, 4, 3>();
    check_tile<10, 5, 3>();
    return 0;
}
