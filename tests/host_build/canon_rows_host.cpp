// The device enumerator's row generator (canon_rows.cuh) compiled for the host.
#include "../../incidence-system-enumeration_gb300/csrc/canon_rows.cuh"

extern "C" uint32_t rows_children(int v, int b, int r, int k, int lambda, const uint64_t *parent, int n,
                                  uint64_t *out, uint32_t cap) {
    const canon::rows::Params d{v, b, r, k, lambda};
    if (!out)
        return canon::rows::children<canon::rows::COUNT>(d, parent, n, nullptr, 0);
    return canon::rows::children<canon::rows::CHILD>(d, parent, n, out, cap);
}

// the same with automorphisms of the parent (nibble-packed row permutations) pruning
extern "C" uint32_t rows_children_aut(int v, int b, int r, int k, int lambda, const uint64_t *parent, int n,
                                      uint64_t *out, uint32_t cap, const uint64_t *gens, int ngens) {
    const canon::rows::Params d{v, b, r, k, lambda};
    if (!out)
        return canon::rows::children<canon::rows::COUNT>(d, parent, n, nullptr, 0, gens, ngens);
    return canon::rows::children<canon::rows::CHILD>(d, parent, n, out, cap, gens, ngens);
}
