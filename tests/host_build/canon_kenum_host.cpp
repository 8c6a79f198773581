// canon_kenum_host.cpp -- the round builder and links test of the enumeration of k-systems
// with groups of 3 or 4 (canon_kenum_rounds.h) compiled for the host (test only).
#include "../../incidence-system-enumeration_gb300/csrc/canon_kenum_rounds.h"

// the children of one parent of d rounds (every second entry), as parent + round rows;
// returns their number, writing at most cap of them to out (out may be null)
extern "C" uint64_t emu_kenum_children(const uint8_t *parent, int d, int np, int g, int links, uint8_t *out,
                                       uint64_t cap) {
    std::vector<uint8_t> buf;
    for (int b = parent[(d - 1) * np + 1] + 1; b < np; ++b) {
        canon::kenum::RoundBuilder rb;
        rb.np = np;
        rb.g = g;
        rb.d = d;
        rb.second = b;
        rb.links = links != 0;
        rb.parent = parent;
        rb.out = &buf;
        rb.run();
    }
    const uint64_t cl = (uint64_t)(d + 1) * np, n = buf.size() / cl;
    if (out)
        std::memcpy(out, buf.data(), (size_t)((n < cap ? n : cap) * cl));
    return n;
}

// the links test of rows R (nr rounds of np players in groups of g)
extern "C" int emu_kenum_links(const uint8_t *R, int nr, int np, int g) {
    uint32_t used[16] = {};
    for (int r = 0; r < nr; ++r)
        for (int q = 0; q < np; q += g)
            for (int e = 0; e < g; ++e)
                for (int f = e + 1; f < g; ++f) {
                    const int x = R[r * np + q + e], y = R[r * np + q + f];
                    used[x] |= 1u << y;
                    used[y] |= 1u << x;
                }
    return canon::kenum::links_complete(used, np, g) ? 1 : 0;
}
