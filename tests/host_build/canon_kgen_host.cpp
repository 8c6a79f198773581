// canon_kgen_host.cpp -- the relabeling step of the GPU check of k-systems with groups of
// 3 or 4 (canon_kgen.cuh) compiled for the host and run over every relabeling in the
// order of the reference's cnvCheckNew(), as one warp task of the GPU kernel takes them
// (test only).
#include <algorithm>
#include <cstring>

#include "../../incidence-system-enumeration_gb300/csrc/canon_kgen.cuh"

namespace {

// Heap's permutations of ng groups, one row of 6 bytes each (canonizator() order)
int heap_rows(int ng, uint8_t *out) {
    uint8_t a[7], p[7];
    for (int i = 0; i < ng; ++i)
        a[i] = p[i] = (uint8_t)i;
    p[ng] = (uint8_t)ng;
    int n = 0;
    std::memcpy(out + 6 * n++, a, (size_t)ng);
    int i = 1;
    while (i < ng) {
        p[i]--;
        const int j = (i % 2) ? p[i] : 0;
        std::swap(a[i], a[j]);
        std::memcpy(out + 6 * n++, a, (size_t)ng);
        i = 0;
        while (!p[++i])
            p[i] = (uint8_t)i;
    }
    return n;
}

}  // namespace

// rows R (nr x np bytes); returns 0, or -1 for a shape kg_eval does not take
extern "C" int emu_kgen_check(const uint8_t *R, int nr, int np, int g, int *canonical, int *player_index,
                              uint64_t *n_aut, uint64_t *cands) {
    if (!canon::kg_shape_ok((unsigned)np, (unsigned)g, (unsigned)nr))
        return -1;
    const int ng = np / g;
    static uint8_t heap[720 * 6];
    heap_rows(ng, heap);
    canon::KgTables T;
    std::memset(&T, 0, sizeof(T));
    for (int r = 0; r < nr; ++r) {
        for (int p = 0; p < np; ++p) {
            T.seq[r] = canon::nib_set(T.seq[r], p, R[r * np + p]);
            T.pos[r] = canon::nib_set(T.pos[r], R[r * np + p], p);
        }
        for (int k = 0; k < ng; ++k) {
            uint32_t l[4] = {0, 0, 0, 0};
            for (int e = 0; e < g; ++e)
                l[e] = R[r * np + k * g + e];
            T.okey[r][k] = (uint16_t)canon::kg_key(l, (unsigned)g);
        }
    }
    const uint64_t total = canon::kg_total((unsigned)np, (unsigned)g, (unsigned)nr);
    const int pidx0 = nr * np - g - 1;
    *canonical = 1;
    *player_index = pidx0;
    *n_aut = 0;
    *cands = total - 1;
    for (uint64_t c = 0; c < total; ++c) {
        int pi = pidx0;
        uint64_t ttr = 0;
        const int res = g == 3 ? canon::kg_eval<3>((unsigned)c, (unsigned)np, (unsigned)ng, (unsigned)nr, T, heap,
                                                   pidx0, pi, ttr)
                               : canon::kg_eval<4>((unsigned)c, (unsigned)np, (unsigned)ng, (unsigned)nr, T, heap,
                                                   pidx0, pi, ttr);
        if (res == 0)
            ++*n_aut;
        if (res < 0) {
            *canonical = 0;
            *player_index = pi;
            *cands = c;
            *n_aut = 0;
            break;
        }
    }
    return 0;
}
