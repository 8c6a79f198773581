// canon_kbin_host.cpp -- the search of canon_kbin_core.cuh (the canonical binary matrix
// of a k-system, runCanonizer()) compiled for the host (test only).
#include "../../incidence-system-enumeration_gb300/csrc/canon_kbin_core.cuh"

using namespace canon::kbin;

// rows: v words; out: v words of the canonical matrix; returns 0, or -2 on timeout
extern "C" int emu_kbin(const uint64_t *rows, int v, int b, int g, int nd, int free_days, uint64_t *out,
                        uint64_t *leaves, uint64_t *nodes) {
    static Search S;
    S.sh = Shape{v, b, g, nd, free_days != 0};
    const Result r = canonize(S, rows, 1ull << 32);
    for (int i = 0; i < v; ++i)
        out[i] = S.bound[i];
    *leaves = r.leaves;
    *nodes = r.nodes;
    return r.timeout ? -2 : 0;
}
