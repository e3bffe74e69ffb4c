// Pageable output memory that the GPU is about to write through the host's
// page tables: make its pages present first (host code only).
//
// A GPU write to a page the process has not touched yet (a fresh allocation)
// faults through the SMMU, at about 20 us per 64 KB page on Grace: a freshly
// allocated 128 MB output took 37 ms against 1.2 ms once present (5.2 ms
// populated first).  mincore() finds the absent pages (populating every page
// of present memory cost 3 ms per 512 MB call), and the caller's populate(lo,
// hi) makes each run of them present -- madvise(MADV_POPULATE_WRITE), which
// leaves the contents alone, so in-place calls are safe.  Separate rows are
// merged into runs of adjacent or overlapping pages, so heap-allocated rows
// cost a few calls.  Failures (older kernels, special mappings) are ignored:
// the GPU then faults the pages in itself.
#pragma once
#include <sys/mman.h>
#include <unistd.h>

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <initializer_list>
#include <vector>

#ifndef MADV_POPULATE_WRITE
#define MADV_POPULATE_WRITE 23  // Linux 5.14
#endif

namespace gbfft {

inline uintptr_t host_page_size() {
    static const uintptr_t page = (uintptr_t)sysconf(_SC_PAGESIZE);
    return page;
}

// Outputs below this many bytes in all are not checked, and separate rows of
// at least this size are each examined: the C library allocates such blocks
// with a fresh mmap, so a per-call output vector is absent every call.
constexpr size_t kPrefaultMinBytes = (size_t)128 << 10;

// Populate [lo, hi) (page-aligned) in one call.
inline void populate_pages(uintptr_t lo, uintptr_t hi) {
    if (hi > lo) (void)madvise((void *)lo, hi - lo, MADV_POPULATE_WRITE);
}

inline bool page_present(uintptr_t pg) {
    unsigned char v = 0;
    return mincore((void *)pg, host_page_size(), &v) == 0 && (v & 1);
}

// Present memory, the usual case of a reused output, is recognised from four
// sampled pages (each mincore call costs ~3 us on Grace; a whole-range check
// of a 512 MB output cost 1.4 % of the call); a range whose samples are all
// present is left as it is.  Otherwise every absent run is populated.
template <class Populate>
void prefault_pages(uintptr_t lo, uintptr_t hi, Populate &&populate) {
    if (hi <= lo) return;
    const uintptr_t page = host_page_size();
    const size_t npages = (hi - lo) / page;
    if (npages > 4) {
        bool all = true;
        for (size_t k = 0; k < 4 && all; ++k) all = page_present(lo + (k * (npages - 1) / 3) * page);
        if (all) return;
    }
    thread_local std::vector<unsigned char> present;
    if (present.size() < npages) present.resize(npages);
    if (mincore((void *)lo, hi - lo, present.data()) != 0) {
        populate(lo, hi);
        return;
    }
    for (size_t i = 0; i < npages;) {
        if (present[i] & 1) {
            ++i;
            continue;
        }
        size_t j = i;
        while (j < npages && !(present[j] & 1)) ++j;
        populate(lo + i * page, lo + j * page);
        i = j;
    }
}

// The output of a host call: contiguous at base (rows == nullptr) or the
// separate rows[0 .. nrows), row_bytes each; bytes = the output's total size.
// Rows under kPrefaultMinBytes come from the heap, recycled and present in
// steady state: three sampled rows (first, middle, last) decide whether the
// whole batch is examined (a first call, or a heap that has just grown).
template <class Populate>
void prefault_output(char *base, size_t bytes, float *const *rows, uint64_t nrows, size_t row_bytes,
                     Populate &&populate) {
    const uintptr_t page = host_page_size();
    auto down = [page](uintptr_t a) { return a & ~(page - 1); };
    auto up = [page](uintptr_t a) { return (a + page - 1) & ~(page - 1); };
    if (bytes < kPrefaultMinBytes || nrows == 0) return;
    if (!rows) {
        prefault_pages(down((uintptr_t)base), up((uintptr_t)base + bytes), populate);
        return;
    }
    if (row_bytes < kPrefaultMinBytes) {
        bool present = true;
        for (uint64_t r : {(uint64_t)0, nrows / 2, nrows - 1})
            present = present && page_present(down((uintptr_t)rows[r]));
        if (present) return;
    }
    uintptr_t lo = 0, hi = 0;
    for (uint64_t r = 0; r < nrows; ++r) {
        const uintptr_t a = down((uintptr_t)rows[r]), b = up((uintptr_t)rows[r] + row_bytes);
        if (hi > lo && a <= hi && b >= lo) {
            lo = std::min(lo, a);
            hi = std::max(hi, b);
        } else {
            prefault_pages(lo, hi, populate);
            lo = a;
            hi = b;
        }
    }
    prefault_pages(lo, hi, populate);
}

}  // namespace gbfft
