// canon_pack.h -- the work descriptors of a queued batch, built on the host pool (host
// code; canon_submit_* use it, a host build tests it).
#pragma once
#include <atomic>
#include <cstdint>
#include <functional>
#include <vector>

#include "canon_hostpool.h"

namespace canon {

// The work descriptors of a batch, in order of filled rows (stable), built on the pool.
// Matrices with the same number of filled rows run the same loops, and the threads of a
// warp take consecutive descriptors from the work counter, so sorted descriptors keep a
// warp's lanes together (the 2M mix of partial matrices: 7.6 -> 5.3 ms of kernel time);
// the outputs keep the submission order through Item::out_idx.  copy(lo, hi) runs on the
// same contiguous ranges first (the rows into the pinned staging); make(i, nr) builds the
// descriptor of matrix i.  Returns false, writing no descriptor, if a row count is
// outside [1, maxr] (nrows == nullptr: every matrix has maxr rows).
template <typename ItemT, typename Copy, typename Make>
bool pack_items_by_rows(uint64_t n, const uint8_t *nrows, uint32_t maxr, ItemT *dst, Copy copy, Make make) {
    constexpr unsigned NB = 17;   // row counts 0 .. 16
    HostPool &pool = HostPool::get();
    const unsigned nt = n < (1u << 16) ? 1u : pool.threads();
    std::vector<uint64_t> at((size_t)nt * NB, 0);
    std::atomic<bool> bad{false};
    const std::function<void(unsigned)> count = [&](unsigned t) {
        const uint64_t lo = n * t / nt, hi = n * (t + 1) / nt;
        copy(lo, hi);
        uint64_t *h = &at[(size_t)t * NB];
        bool ok = true;
        for (uint64_t i = lo; i < hi; ++i) {
            const uint32_t nr = nrows ? nrows[i] : maxr;
            ok = ok && nr >= 1 && nr <= maxr;
            ++h[nr < NB ? nr : 0];
        }
        if (!ok)
            bad.store(true, std::memory_order_relaxed);
    };
    if (nt == 1)
        count(0);
    else
        pool.run(nt, count);
    if (bad.load())
        return false;
    uint64_t pos = 0;   // row count major, range minor: the order of a stable sort
    for (unsigned r = 0; r < NB; ++r)
        for (unsigned t = 0; t < nt; ++t) {
            const uint64_t k = at[(size_t)t * NB + r];
            at[(size_t)t * NB + r] = pos;
            pos += k;
        }
    const std::function<void(unsigned)> place = [&](unsigned t) {
        const uint64_t lo = n * t / nt, hi = n * (t + 1) / nt;
        uint64_t *o = &at[(size_t)t * NB];
        for (uint64_t i = lo; i < hi; ++i) {
            const uint32_t nr = nrows ? nrows[i] : maxr;
            dst[o[nr]++] = make(i, nr);
        }
    };
    if (nt == 1)
        place(0);
    else
        pool.run(nt, place);
    return true;
}

}  // namespace canon
