// group_order_ref.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Exposes the reference's own permutation/orbit machinery, CGroupOrder<T> from
// k-Factorization/Utils/Include/GroupOrder.h, compiled in place from the
// reference tree (see oracle/build_ref.sh), behind the same C signatures as the
// oracle's restatement (or_next_permutation / or_add_automorphism /
// or_update_group_order).  The tests swap it into the oracle's checker to pin
// the restatement on the reference's own code.
#include <cstdint>
#include <cstring>
#include <algorithm>
using std::max;
using std::min;
#include "GroupOrder.h"

namespace {
struct RefGroup : public CGroupOrder<unsigned char> {
    using Base = CGroupOrder<unsigned char>;
    void load(unsigned stab, unsigned stab_aut, uint64_t lo, uint64_t hi) {
        setStabilizerLength((ushort)stab);
        setStabilizerLengthAut((ushort)stab_aut);
        setGroupOrder(UInt(hi, lo));
    }
    void store(unsigned *stab, unsigned *stab_aut, uint64_t *lo, uint64_t *hi) const {
        *stab = stabilizerLength();
        *stab_aut = stabilizerLengthAut();
        UInt o = groupOrder();
        *lo = o.lo;
        *hi = o.hi;
    }
    unsigned char next(unsigned char *perm, const unsigned char *orb, unsigned char n,
                       unsigned char idx, unsigned char len_stab) {
        return Base::next_permutation(perm, orb, n, idx, len_stab);
    }
};
}  // namespace

// Layout identical to or_group in canon_oracle.h (unsigned, unsigned, __int128).
struct ref_group_c {
    unsigned stab;
    unsigned stab_aut;
    unsigned __int128 order;
};

extern "C" {

unsigned char ref_next_permutation(ref_group_c *g, unsigned char *perm, const unsigned char *orb,
                                   unsigned char n, unsigned char idx, unsigned char len_stab) {
    RefGroup r;
    r.load(g->stab, g->stab_aut, (uint64_t)g->order, (uint64_t)(g->order >> 64));
    unsigned char ret = r.next(perm, orb, n, idx, len_stab);
    uint64_t lo, hi;
    r.store(&g->stab, &g->stab_aut, &lo, &hi);
    g->order = ((unsigned __int128)hi << 64) | lo;
    return ret;
}

void ref_add_automorphism(ref_group_c *g, unsigned degree, const unsigned char *perm,
                          unsigned char *orb, int row_permut, int calc_group_order) {
    RefGroup r;
    r.load(g->stab, g->stab_aut, (uint64_t)g->order, (uint64_t)(g->order >> 64));
    r.addAutomorphism((ushort)degree, perm, orb, row_permut != 0, false, calc_group_order != 0);
    uint64_t lo, hi;
    r.store(&g->stab, &g->stab_aut, &lo, &hi);
    g->order = ((unsigned __int128)hi << 64) | lo;
}

void ref_update_group_order(ref_group_c *g, unsigned degree, const unsigned char *orb) {
    RefGroup r;
    r.load(g->stab, g->stab_aut, (uint64_t)g->order, (uint64_t)(g->order >> 64));
    r.updateGroupOrder((ushort)degree, orb);
    uint64_t lo, hi;
    r.store(&g->stab, &g->stab_aut, &lo, &hi);
    g->order = ((unsigned __int128)hi << 64) | lo;
}

}  // extern "C"
