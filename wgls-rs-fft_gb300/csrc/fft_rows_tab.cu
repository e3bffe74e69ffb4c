// The single-pass kernel over per-row address tables (fft_rows_kernel<...,
// TAB = true>), for the default tiles of every single-pass size: 2^12 samples
// a CTA with 16 samples a thread (N = 2^0 .. 2^14), 2^11 samples a CTA
// (N = 2^6 .. 2^11) and 32 samples a thread (N = 2^13, 2^14).  The host
// entries use it to transform the caller's separate host rows in place of a
// copy through HBM.  Its own translation unit keeps the build parallel.
#include "fft_rows.cuh"

namespace gbfft {

template <int LOGN, int LOGS, int LE>
static void tab_set(RowsKernelInfo &k) {
    k.fn_tab = (const void *)fft_rows_kernel<LOGN, LOGS, -1, LE, true>;
    k.fn_tab_inv = (const void *)fft_rows_kernel<LOGN, LOGS, 1, LE, true>;
}

void rows_tab_describe(int logn, int logs, int loge, RowsKernelInfo &k) {
    k.fn_tab = k.fn_tab_inv = nullptr;
    if (loge == 5 && logs == 12) {
        if (logn == 13) tab_set<13, 12, 5>(k);
        if (logn == 14) tab_set<14, 12, 5>(k);
        return;
    }
    if (loge != 4) return;
    if (logs == 11) {
        switch (logn) {
            case 6: tab_set<6, 11, 4>(k); return;
            case 7: tab_set<7, 11, 4>(k); return;
            case 8: tab_set<8, 11, 4>(k); return;
            case 9: tab_set<9, 11, 4>(k); return;
            case 10: tab_set<10, 11, 4>(k); return;
            case 11: tab_set<11, 11, 4>(k); return;
            default: return;
        }
    }
    if (logs != 12) return;
    switch (logn) {
#define GBFFT_TAB(L) \
    case L: tab_set<L, 12, 4>(k); return;
        GBFFT_TAB(0) GBFFT_TAB(1) GBFFT_TAB(2) GBFFT_TAB(3) GBFFT_TAB(4) GBFFT_TAB(5) GBFFT_TAB(6)
        GBFFT_TAB(7) GBFFT_TAB(8) GBFFT_TAB(9) GBFFT_TAB(10) GBFFT_TAB(11) GBFFT_TAB(12) GBFFT_TAB(13)
        GBFFT_TAB(14)
#undef GBFFT_TAB
        default: return;
    }
}

}  // namespace gbfft
