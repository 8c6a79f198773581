// canon_ksys_rounds_host.cpp -- the device round generator of the k-system enumerator
// (canon_ksys_rounds.cuh) compiled for the host (test only).
#include "../../incidence-system-enumeration_gb300/csrc/canon_ksys_rounds.cuh"

extern "C" uint32_t emu_ksys_children(int np, const uint8_t *parent, int d, uint8_t *dst) {
    return canon::ksys_children(np, parent, d, dst);
}

extern "C" uint32_t emu_ksys_children_part(int np, const uint8_t *parent, int d, uint8_t *dst, int second) {
    return canon::ksys_children(np, parent, d, dst, second);
}
