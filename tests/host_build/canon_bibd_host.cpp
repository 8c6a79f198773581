// canon_bibd_host.cpp -- the device search of canon_bibd_core.cuh compiled for the
// host (test only): CUDA qualifiers are defined away and the intrinsics the search
// uses are given host definitions, so the CPU suite can check the kernel logic
// against the oracle without a GPU.
#include <cstdint>
#include <cstring>
#define __device__
#define __host__
#define __forceinline__ inline
#define __global__
static inline int __ffsll(long long x) { return __builtin_ffsll(x); }
static inline int __ffs(unsigned x) { return __builtin_ffs((int)x); }
static inline int __popcll(unsigned long long x) { return __builtin_popcountll(x); }
static inline unsigned long long __brevll(unsigned long long x) {
    unsigned long long r = 0;
    for (int i = 0; i < 64; ++i)
        r |= ((x >> i) & 1ull) << (63 - i);
    return r;
}
static inline int __popc(unsigned x) { return __builtin_popcount(x); }
static inline int __clzll(long long x) { return x ? __builtin_clzll((unsigned long long)x) : 64; }
static inline int __clz(unsigned x) { return x ? __builtin_clz(x) : 32; }
static inline unsigned long long __umul64hi(unsigned long long a, unsigned long long b) { return (unsigned long long)(((unsigned __int128)a * b) >> 64); }
#include "../../incidence-system-enumeration_gb300/csrc/canon_bibd_core.cuh"
using namespace canon;
using namespace canon::bibd;
extern "C" int emu_check(const uint64_t *rows, unsigned n, unsigned b, unsigned flags, uint64_t max_trials,
                         uint8_t *canonical, uint8_t *status, uint8_t *reject_row, uint64_t *witness, uint64_t *aut, uint64_t *trials) {
    static uint64_t s_rows[VMAX * TPB], s_lvl[(VMAX + 1) * TPB];
    static uint32_t s_vd[VMAX * TPB];
    static uint16_t s_cm[64 * TPB];
    static uint8_t s_pc[64 * TPB];
    Smem sm{s_rows, s_lvl, s_pc, s_cm, s_vd};
    CheckOut o;
    check_one(sm, rows, n, b, flags, max_trials, nullptr, 0, o);
    *canonical = o.canonical; *status = o.status; *reject_row = o.reject_row; *witness = o.witness;
    aut[0] = o.aut_lo; aut[1] = o.aut_hi; *trials = o.trials;
    return 0;
}
// the lex-max search alone: canonical form into rows_out, |Aut|, node count and
// the first rows of the labelings; prune selects the automorphism pruning
extern "C" int emu_maxsearch(const uint64_t *rows, unsigned n, unsigned b, uint64_t *rows_out, uint64_t *leaves,
                             uint64_t *nodes, uint8_t *improved, int prune, unsigned *first_rows) {
    static uint64_t s_rows[VMAX * TPB], s_lvl[(VMAX + 1) * TPB];
    static uint32_t s_vd[VMAX * TPB];
    static uint16_t s_cm[64 * TPB];
    static uint8_t s_pc[64 * TPB];
    Smem sm{s_rows, s_lvl, s_pc, s_cm, s_vd};
    if (!load_rows(sm, rows, n, b, F_RAW))
        return -1;
    MaxOut mo;
    max_search(sm, n, b, 1ull << 30, mo, ID16, prune != 0);
    for (unsigned r = 0; r < n; ++r) rows_out[r] = R_(r);
    *leaves = mo.leaves; *nodes = mo.nodes; *improved = mo.improved;
    if (first_rows)
        *first_rows = mo.first_rows;
    return mo.timeout ? -2 : 0;
}

// one thread's share of a search split by first row: rows in root_mask may come first
extern "C" int emu_maxsearch_root(const uint64_t *rows, unsigned n, unsigned b, unsigned root_mask,
                                  uint64_t *leaves, unsigned *orbit0, uint8_t *improved) {
    static uint64_t s_rows[VMAX * TPB], s_lvl[(VMAX + 1) * TPB];
    static uint32_t s_vd[VMAX * TPB];
    static uint16_t s_cm[64 * TPB];
    static uint8_t s_pc[64 * TPB];
    Smem sm{s_rows, s_lvl, s_pc, s_cm, s_vd};
    if (!load_rows(sm, rows, n, b, F_RAW))
        return -1;
    MaxOut mo;
    max_search(sm, n, b, 1ull << 30, mo, ID16, true, true, root_mask);
    *leaves = mo.leaves; *orbit0 = mo.orbit0; *improved = mo.improved;
    return mo.timeout ? -2 : 0;
}

// a share of a search split by the first two rows
extern "C" int emu_maxsearch_root2(const uint64_t *rows, unsigned n, unsigned b, unsigned root_mask,
                                   unsigned root_mask1, uint64_t *leaves, unsigned *orbit0, unsigned *orbit1,
                                   uint8_t *improved) {
    static uint64_t s_rows[VMAX * TPB], s_lvl[(VMAX + 1) * TPB];
    static uint32_t s_vd[VMAX * TPB];
    static uint16_t s_cm[64 * TPB];
    static uint8_t s_pc[64 * TPB];
    Smem sm{s_rows, s_lvl, s_pc, s_cm, s_vd};
    if (!load_rows(sm, rows, n, b, F_RAW))
        return -1;
    MaxOut mo;
    max_search(sm, n, b, 1ull << 30, mo, ID16, true, true, root_mask, nullptr, root_mask1);
    *leaves = mo.leaves; *orbit0 = mo.orbit0; *orbit1 = mo.orbit1; *improved = mo.improved;
    return mo.timeout ? -2 : 0;
}

// The converged layout of the same search (canon_bibd_conv.cuh), one lane: control
// steps until a node is due, then the node step, as bibd_conv_kernel runs them.
#include "../../incidence-system-enumeration_gb300/csrc/canon_bibd_conv.cuh"
// bt >= b: the columns walked (a mixed launch walks its widest item's columns)
extern "C" int emu_conv_search_bt(const uint64_t *rows, unsigned n, unsigned b, unsigned bt, uint64_t order0,
                                  uint64_t *leaves, uint64_t *nodes, uint8_t *improved, int mode) {
    static uint64_t s_rows[VMAX * TPB], s_lvl[(VMAX + 1) * TPB];
    static uint16_t s_vd[VMAX * TPB];
    static uint16_t s_cm[64 * TPB];
    SmemMax sm{s_rows, s_lvl, nullptr, s_cm, s_vd};
    if (!load_rows(sm, rows, n, b, F_RAW))
        return -1;
    for (unsigned c = b; c < 64; ++c)
        CM_(c) = 0;
    // mode: 0 climb, 1 restart after RESTART_AFTER nodes (the kernels' rule), 2 restart
    // whenever the bound is complete and greater than the searched matrix
    ConvState st;
    conv_start(st, n, order0);
    st.b = b;
    st.w = conv_row_weight(sm, n);     // the count planes, as the kernels choose them
    st.restart_after = mode == 0 ? ~0ull : (mode == 1 ? RESTART_AFTER : 0);
    st.verdict_only = mode == 3;
    int ref_lv = -1;
    unsigned ref_x = 0;
    // the kernels' unrolled node step: the smallest instance of 24, 35, 40 or 64 columns
    // that holds the columns walked, when they fill at least three quarters of it (the
    // rest are empty columns); else the loop over bt columns
    unsigned fb = bt <= 24 ? 24 : bt <= 35 ? 35 : bt <= 40 ? 40 : 64;
    if ((fb - bt) * 4 > fb)
        fb = 0;
    for (;;) {
        if (ref_lv >= 0) {
            if (fb == 24)
                refine_uniform<24>(sm, (unsigned)ref_lv, ref_x, bt);
            else if (fb == 35)
                refine_uniform<35>(sm, (unsigned)ref_lv, ref_x, bt);
            else if (fb == 40)
                refine_uniform<40>(sm, (unsigned)ref_lv, ref_x, bt);
            else if (fb == 64)
                refine_uniform<64>(sm, (unsigned)ref_lv, ref_x, bt);
            else
                refine_uniform(sm, (unsigned)ref_lv, ref_x, bt);
        }
        if (++st.nodes > (1ull << 30))
            return -2;
        unsigned tied = st.allrows & ~st.used;
        uint64_t arr = 0;
        const bool hb = st.i < st.valid;
        const uint64_t bnd = hb ? R_(st.i) : 0ull;
        const int state = fb == 24   ? eval_node_planes<24>(sm, st.w, st.i, b, bt, tied, arr, hb, bnd)
                          : fb == 35 ? eval_node_planes<35>(sm, st.w, st.i, b, bt, tied, arr, hb, bnd)
                          : fb == 40 ? eval_node_planes<40>(sm, st.w, st.i, b, bt, tied, arr, hb, bnd)
                          : fb == 64 ? eval_node_planes<64>(sm, st.w, st.i, b, bt, tied, arr, hb, bnd)
                                     : eval_node_planes(sm, st.w, st.i, b, bt, tied, arr, hb, bnd);
        if (!conv_after_eval(sm, st, state, tied, arr, b))
            break;
        if (!conv_next(sm, st, ref_lv, ref_x))
            break;
    }
    *leaves = conv_leaves(st);
    *nodes = st.nodes;
    *improved = conv_rejected(st);
    return 0;
}

extern "C" int emu_conv_search(const uint64_t *rows, unsigned n, unsigned b, uint64_t order0, uint64_t *leaves,
                               uint64_t *nodes, uint8_t *improved, int aut_only) {
    return emu_conv_search_bt(rows, n, b, b, order0, leaves, nodes, improved, aut_only);
}

// max_search() with a first-row order (the learned order's effect on the search)
extern "C" int emu_maxsearch_order(const uint64_t *rows, unsigned n, unsigned b, uint64_t order0, uint64_t *leaves,
                                   uint64_t *nodes, uint8_t *improved, int aut_only) {
    static uint64_t s_rows[VMAX * TPB], s_lvl[(VMAX + 1) * TPB];
    static uint16_t s_vd[VMAX * TPB];
    static uint16_t s_cm[64 * TPB];
    SmemMax sm{s_rows, s_lvl, nullptr, s_cm, s_vd};
    if (!load_rows(sm, rows, n, b, F_RAW))
        return -1;
    MaxOut mo;
    if (aut_only == 2) {
        max_search(sm, n, b, CLIMB_CAP, mo, order0);
        if (mo.timeout) {
            load_rows(sm, rows, n, b, F_RAW);
            max_search(sm, n, b, 1ull << 30, mo, order0, true, false, 0xFFFFu, nullptr, 0xFFFFu, nullptr, 0, true);
            mo.nodes += CLIMB_CAP;
        }
    } else {
        max_search(sm, n, b, 1ull << 30, mo, order0, true, false, 0xFFFFu, nullptr, 0xFFFFu, nullptr, 0, aut_only != 0);
    }
    *leaves = mo.leaves; *nodes = mo.nodes; *improved = mo.improved;
    return mo.timeout ? -2 : 0;
}
