// Host-side check of the register butterflies (Dft<R>, fft_core.cuh /
// fft_smem.cuh) against a direct FP64 DFT: prints the worst relative L2 error
// over 2000 random inputs per radix.  Built and run by tests/test_butterflies.py.
#include <cstdio>
#include <cmath>
#include <random>
#include "fft_smem.cuh"
using namespace gbfft;
template <int R> double check(std::mt19937 &g) {
    std::uniform_real_distribution<float> U(-1.f, 1.f);
    double worst = 0;
    for (int it = 0; it < 2000; ++it) {
        float2 x[R]; double xr[R], xi[R];
        for (int i = 0; i < R; ++i) { x[i] = make_float2(U(g), U(g)); xr[i] = x[i].x; xi[i] = x[i].y; }
        Dft<R>::run(x);
        double num = 0, den = 0;
        for (int k = 0; k < R; ++k) {
            double sr = 0, si = 0;
            for (int n = 0; n < R; ++n) { double a = -2 * M_PI * (double)((k * n) % R) / R; sr += xr[n] * cos(a) - xi[n] * sin(a); si += xr[n] * sin(a) + xi[n] * cos(a); }
            num += (x[k].x - sr) * (x[k].x - sr) + (x[k].y - si) * (x[k].y - si); den += sr * sr + si * si;
        }
        worst = fmax(worst, sqrt(num / den));
    }
    return worst;
}
int main() {
    std::mt19937 g(1);
    printf("2 %.3g\n4 %.3g\n8 %.3g\n16 %.3g\n32 %.3g\n", check<2>(g), check<4>(g), check<8>(g), check<16>(g),
           check<32>(g));
    return 0;
}
