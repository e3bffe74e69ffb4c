// The reference's own GpuFft tests, restated against the C++ mirror
// (include/gbfft.hpp) of the GB300 library.  Expected values come from closed
// forms (impulse, roundtrip, exact helpers) and from a direct double DFT here
// (the reference compares with rustfft 6.4.1, which is not available).
//   tests/gpu_fft_test.rs:8-42        forward vs exact DFT, N = 1024, < 1e-3
//   tests/ifft_test.rs:22-107         roundtrips, ifft vs exact, < 1e-3
//   src/lib.rs:207-227                roundtrip of x_i = 0.1 i, < 1e-4
//   examples/test_parallel.rs:64-130  output shape, impulse, batch independence
// Exit status 0 when every check passes.
#include <cmath>
#include <cstdio>
#include <string>

#include "gbfft.hpp"

using gbfft::Batch;
using gbfft::Complex;

static int g_fail = 0;
#define CHECK(cond, ...)                          \
    do {                                          \
        if (!(cond)) {                            \
            std::printf("FAIL %s: ", #cond);      \
            std::printf(__VA_ARGS__);             \
            std::printf("\n");                    \
            ++g_fail;                             \
        }                                         \
    } while (0)

static std::vector<Complex> dft(const std::vector<Complex> &x, bool inverse) {
    const size_t n = x.size();
    std::vector<Complex> y(n);
    for (size_t k = 0; k < n; ++k) {
        std::complex<double> s = 0;
        for (size_t m = 0; m < n; ++m) {
            const double a = (inverse ? 2.0 : -2.0) * M_PI * (double)((k * m) % n) / (double)n;
            s += std::complex<double>(x[m].real(), x[m].imag()) * std::polar(1.0, a);
        }
        if (inverse) s /= (double)n;
        y[k] = Complex((float)s.real(), (float)s.imag());
    }
    return y;
}

static float max_diff(const std::vector<Complex> &a, const std::vector<Complex> &b) {
    float m = 0.f;
    for (size_t i = 0; i < a.size(); ++i) m = std::fmax(m, std::abs(a[i] - b[i]));
    return m;
}

static std::vector<Complex> make_input(size_t n) {  // tests/gpu_fft_test.rs:8-15
    std::vector<Complex> v(n);
    for (size_t i = 0; i < n; ++i) v[i] = Complex(std::sin((float)i * 0.1f), std::cos((float)i * 0.07f));
    return v;
}

int main() {
    if (!gbfft::GpuFft::is_gpu_available()) {
        std::printf("no GB300 available\n");
        return 2;
    }
    gbfft::GpuFft fft;
    const float eps = 1e-3f;

    // forward vs exact DFT
    auto x = make_input(1024);
    auto X = fft.fft({x});
    CHECK(X.size() == 1 && X[0].size() == 1024, "shape");
    CHECK(max_diff(X[0], dft(x, false)) < eps, "fft vs dft %g", max_diff(X[0], dft(x, false)));

    // ifft of the spectrum vs exact inverse; roundtrips both ways
    auto r = fft.ifft(X);
    CHECK(max_diff(r[0], x) < eps, "roundtrip %g", max_diff(r[0], x));
    CHECK(max_diff(r[0], dft(dft(x, false), true)) < eps, "ifft vs exact");
    auto X2 = fft.fft(r);
    CHECK(max_diff(X2[0], X[0]) < eps, "fft(ifft(fft x))");

    // src/lib.rs:207-227 ramp roundtrip < 1e-4
    std::vector<Complex> ramp(1024);
    for (size_t i = 0; i < ramp.size(); ++i) ramp[i] = Complex((float)i * 0.1f, 0.f);
    auto rr = fft.ifft(fft.fft({ramp}));
    CHECK(max_diff(rr[0], ramp) < 1e-4f, "ramp roundtrip %g", max_diff(rr[0], ramp));

    // impulse -> flat magnitude 1
    std::vector<Complex> imp(256, Complex(0.f, 0.f));
    imp[0] = Complex(1.f, 0.f);
    auto Y = fft.fft({imp});
    float worst = 0.f;
    for (auto &c : Y[0]) worst = std::fmax(worst, std::fabs(std::abs(c) - 1.f));
    CHECK(worst < 1e-3f, "impulse %g", worst);

    // output shapes and batch independence
    for (size_t n : {64, 256, 1024}) {
        auto o = fft.fft({std::vector<Complex>(n, Complex(1.f, 0.f))});
        CHECK(o[0].size() == n, "length %zu", n);
    }
    Batch sig(4, std::vector<Complex>(128));
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 128; ++j) sig[i][j] = Complex((float)(i * 10 + j) * 0.001f, 0.f);
    auto bo = fft.fft(sig);
    CHECK(bo.size() == 4, "batch count");
    for (int i = 0; i < 4; ++i) CHECK(max_diff(fft.fft({sig[i]})[0], bo[i]) < 1e-4f, "batch independence %d", i);
    // into caller-kept rows: the same bits as fft / ifft
    Batch kept(4, std::vector<Complex>(128));
    fft.transform_into(sig, kept);
    for (int i = 0; i < 4; ++i) CHECK(max_diff(kept[i], bo[i]) == 0.f, "transform_into row %d", i);
    fft.transform_into(bo, kept, true);
    auto bi = fft.ifft(bo);
    for (int i = 0; i < 4; ++i) CHECK(max_diff(kept[i], bi[i]) == 0.f, "transform_into inverse row %d", i);

    // empty batch, errors with the reference's messages
    CHECK(fft.fft({}).empty(), "empty batch");
    try {
        fft.fft({std::vector<Complex>(4), std::vector<Complex>(8)});
        CHECK(false, "mismatch not rejected");
    } catch (const gbfft::Error &e) {
        CHECK(e.status() == GBFFT_ERR_LENGTH_MISMATCH, "status %d", e.status());
        CHECK(std::string(e.what()) == "All input vectors in a batch must have the same length", "%s", e.what());
    }
    try {
        fft.ifft({std::vector<Complex>(3)});
        CHECK(false, "non power of two not rejected");
    } catch (const gbfft::Error &e) {
        CHECK(e.status() == GBFFT_ERR_INVALID_SIZE, "status %d", e.status());
        CHECK(std::string(e.what()) == "Transform length must be a non-zero power of two", "%s", e.what());
    }
    CHECK(fft.benchmark_gpu_only(4096, 256, 2, 5) > 0.0, "bench");

    // the window on load equals an explicitly windowed input (tests/test_utils.rs:39-48)
    {
        const size_t n = 2048;
        auto xs = make_input(n);
        std::vector<Complex> xw(n);
        for (size_t i = 0; i < n; ++i) {
            const double w = 0.5 * (1.0 - std::cos(2.0 * M_PI * (double)i / (double)(n - 1)));
            xw[i] = Complex((float)(xs[i].real() * w), (float)(xs[i].imag() * w));
        }
        gbfft::GpuFft wfft;
        wfft.set_window(GBFFT_WINDOW_HANN);
        auto a = wfft.fft({xs});
        auto b = fft.fft({xw});
        CHECK(max_diff(a[0], b[0]) < 1e-3f, "window on load %g", max_diff(a[0], b[0]));
        wfft.set_window(GBFFT_WINDOW_NONE);
        CHECK(max_diff(wfft.fft({xs})[0], fft.fft({xs})[0]) == 0.f, "window off");
    }
    // noise on load: zero input gives a non-zero spectrum, the same for the same seed
    {
        gbfft::GpuFft nfft;
        nfft.set_noise(42, 0.1f);
        auto a = nfft.fft({std::vector<Complex>(1024)});
        auto b = nfft.fft({std::vector<Complex>(1024)});
        float mag = 0.f;
        for (auto &c : a[0]) mag = std::fmax(mag, std::abs(c));
        CHECK(mag > 0.f && max_diff(a[0], b[0]) == 0.f, "noise on load");
    }
    CHECK(fft.autotune(1 << 16, 16) > 0.0, "autotune");
    try {
        std::vector<gbfft_ragged_desc> bad{{0, 19, GBFFT_FORWARD}};
        gbfft::RaggedPlan plan(fft, bad);
        CHECK(false, "ragged 2^19 not rejected");
    } catch (const gbfft::Error &e) {
        CHECK(e.status() == GBFFT_ERR_UNSUPPORTED, "ragged status %d", e.status());
    }
    CHECK(gbfft_launch_count(fft.context()) > 0, "launches");

    std::printf("%s (%d failures)\n", g_fail ? "FAILED" : "OK", g_fail);
    return g_fail ? 1 : 0;
}
