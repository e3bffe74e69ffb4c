// Fused pass pairs (fft_fused.cuh): the last two passes of a three-pass
// transform with radices (2^(L-16), 256, 256), N = 2^21 .. 2^26.  The first
// pass runs alone (fft_passes.cu) into the workspace; this launch reads it and
// writes the result.
#include "gbfft_internal.h"
#include "gbfft_plan.h"
#include "fft_fused.cuh"

namespace gbfft {

bool fused3_kernel_info(int logn, FusedDesc &d) {
#define GBFFT_F3(L) \
    if (logn == L) { fused_describe<8, 8, 256, L, L - 16>(d); return true; }
    GBFFT_F3(21)
    GBFFT_F3(22)
    GBFFT_F3(23)
    GBFFT_F3(24)
    GBFFT_F3(25)
    GBFFT_F3(26)
#undef GBFFT_F3
    return false;
}

}  // namespace gbfft
