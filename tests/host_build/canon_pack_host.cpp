// canon_pack_host.cpp -- the work-descriptor packing of canon_submit_* (canon_pack.h)
// compiled for the host (test only).
#include <cstdint>
#include <cstring>

#include "../../incidence-system-enumeration_gb300/csrc/canon_pack.h"

struct Desc {
    uint32_t index;
    uint32_t nrows;
};

// packs n descriptors; order[k] = the matrix index placed at position k, copied[i] = 1 for
// every matrix the copy step saw; returns 1, or 0 when a row count is out of range
extern "C" int emu_pack(uint64_t n, const uint8_t *nrows, uint32_t maxr, uint32_t *order, uint32_t *rows_out,
                        uint8_t *copied) {
    std::vector<Desc> d(n);
    const bool ok = canon::pack_items_by_rows(
        n, nrows, maxr, d.data(),
        [&](uint64_t lo, uint64_t hi) {
            for (uint64_t i = lo; i < hi; ++i)
                copied[i] += 1;
        },
        [&](uint64_t i, uint32_t nr) { return Desc{(uint32_t)i, nr}; });
    if (!ok)
        return 0;
    for (uint64_t k = 0; k < n; ++k) {
        order[k] = d[k].index;
        rows_out[k] = d[k].nrows;
    }
    return 1;
}
