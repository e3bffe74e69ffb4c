// Host-side check of the output-page population that precedes GPU writes to
// pageable host memory (wgls-rs-fft_gb300/csrc/host_pages.h): fresh
// anonymous mappings stand in for freshly allocated outputs.  Prints one line
// per case and exits non-zero on the first failure.
#include <sys/mman.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "host_pages.h"

using gbfft::host_page_size;

static int g_calls = 0;
static void counted(uintptr_t lo, uintptr_t hi) {
    ++g_calls;
    gbfft::populate_pages(lo, hi);
}

static char *fresh(size_t bytes) {
    void *p = mmap(nullptr, bytes, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
    if (p == MAP_FAILED) {
        std::perror("mmap");
        std::exit(2);
    }
    return (char *)p;
}

static size_t present_pages(const char *p, size_t bytes) {
    const uintptr_t page = host_page_size();
    const size_t n = (bytes + page - 1) / page;
    std::vector<unsigned char> v(n);
    if (mincore((void *)p, n * page, v.data()) != 0) return (size_t)-1;
    size_t k = 0;
    for (unsigned char c : v) k += c & 1;
    return k;
}

static int fails = 0;
static void check(bool ok, const char *what) {
    std::printf("%s %s\n", ok ? "ok" : "FAIL", what);
    if (!ok) ++fails;
}

int main() {
    const size_t page = host_page_size();
    const size_t n_big = (16u << 20) / page;  // pages of a 16 MB output

    // 1. a fresh contiguous output: every page becomes present
    char *a = fresh(16u << 20);
    g_calls = 0;
    check(present_pages(a, 16u << 20) == 0, "fresh mapping starts absent");
    gbfft::prefault_output(a, 16u << 20, nullptr, 1, 16u << 20, counted);
    check(present_pages(a, 16u << 20) == n_big && g_calls >= 1, "contiguous fresh output populated");

    // 2. the same output again: recognised as present, nothing populated
    g_calls = 0;
    gbfft::prefault_output(a, 16u << 20, nullptr, 1, 16u << 20, counted);
    check(g_calls == 0, "present contiguous output left alone");

    // 3. partly written (in place): contents kept, the rest populated
    char *b = fresh(8u << 20);
    std::memset(b, 0x5a, 4u << 20);
    g_calls = 0;
    gbfft::prefault_output(b, 8u << 20, nullptr, 1, 8u << 20, counted);
    bool kept = true;
    for (size_t i = 0; i < (4u << 20); i += 4093) kept = kept && b[i] == 0x5a;
    check(kept && b[(8u << 20) - 1] == 0 && present_pages(b, 8u << 20) == (8u << 20) / page && g_calls == 1,
          "written half kept, absent half populated in one run");

    // 4. separate fresh rows of 256 KB, each its own mapping
    std::vector<char *> rows;
    for (int r = 0; r < 20; ++r) rows.push_back(fresh(256u << 10));
    g_calls = 0;
    gbfft::prefault_output(nullptr, 20 * (256u << 10), (float *const *)rows.data(), rows.size(), 256u << 10,
                           counted);
    bool all = true;
    for (char *r : rows) all = all && present_pages(r, 256u << 10) == (256u << 10) / page;
    // (the kernel may place the mappings next to each other: adjacent rows merge)
    check(all && g_calls >= 1 && g_calls <= 20, "fresh 256 KB rows populated");

    // 5. small fresh rows carved from one mapping: merged into one run
    const size_t rb = 32u << 10, nr = 128;
    char *c = fresh(rb * nr);
    std::vector<char *> small;
    for (size_t r = 0; r < nr; ++r) small.push_back(c + r * rb);
    g_calls = 0;
    gbfft::prefault_output(nullptr, rb * nr, (float *const *)small.data(), nr, rb, counted);
    check(present_pages(c, rb * nr) == rb * nr / page && g_calls == 1, "small adjacent rows populated as one run");

    // 6. the same small rows again: three sampled rows say present
    g_calls = 0;
    gbfft::prefault_output(nullptr, rb * nr, (float *const *)small.data(), nr, rb, counted);
    check(g_calls == 0, "present small rows left alone");

    // 7. an output under 128 KB in all is not examined
    char *d = fresh(64u << 10);
    g_calls = 0;
    gbfft::prefault_output(d, 64u << 10, nullptr, 1, 64u << 10, counted);
    check(g_calls == 0 && present_pages(d, 64u << 10) == 0, "small output not examined");

    return fails ? 1 : 0;
}
