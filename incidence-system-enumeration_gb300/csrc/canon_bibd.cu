// canon_bibd.cu -- canonicity test of rank-2 incidence matrices (BIBDs, STS) on sm_103a.
//
// One thread owns one matrix and runs the reference's search order exactly:
//   TestCanonicity()            Source/CanonicityChecker.h:255-586 (numParts == 1)
//   checkColOrbit()             Source/CanonicityChecker.cpp:191-223
//   next_permutation()          k-Factorization/Utils/Include/GroupOrder.h:136-248
//   addAutomorphism()/UpdateOrbits()/updateGroupOrder()   GroupOrder.h:30-102
// The permutation and its orbits are nibble-packed in two registers (v <= 16);
// every row is one uint64 bit set (b <= 63); the column orbits of level r are a
// bit mask of orbit-start columns (ColOrbitManager's per-row lists become one
// word per row).  The column arrangement of the permuted matrix (permColumn)
// lives in shared memory as bytes.  Items are taken from a global ticket
// counter so that a thread that finishes a cheap (rejected) matrix immediately
// takes the next one.
#include <mutex>

#include "../../include/canon_gb300.h"
#include "canon_bibd_conv.cuh"

namespace canon {

namespace {

using namespace bibd;

__global__ void __launch_bounds__(TPB) bibd_items_kernel(const Item *__restrict__ items, uint32_t n_items,
                                                         const uint64_t *__restrict__ words, Outputs out,
                                                         uint64_t max_trials, unsigned *ticket) {
    __shared__ uint64_t s_rows[VMAX * TPB];
    __shared__ uint64_t s_lvl[(VMAX + 1) * TPB];
    __shared__ uint32_t s_vd[VMAX * TPB];
    __shared__ uint16_t s_cm[64 * TPB];
    __shared__ uint8_t s_pc[64 * TPB];
    const unsigned tid = threadIdx.x;
    Smem sm{s_rows + tid, s_lvl + tid, s_pc + tid, s_cm + tid, s_vd + tid};
    for (;;) {
        const unsigned it = atomicAdd(ticket, 1u);
        if (it >= n_items)
            break;
        check_item(sm, items[it], words, out, max_trials);
    }
}

__global__ void __launch_bounds__(TPB) bibd_uniform_kernel(uint32_t n_items, uint32_t v, uint32_t b,
                                                           uint32_t flags, const uint64_t *__restrict__ rows,
                                                           uint8_t *canonical, uint8_t *witness16, uint64_t *aut,
                                                           uint8_t *status, uint64_t *trials_out,
                                                           uint64_t max_trials, unsigned *ticket,
                                                           const uint64_t *__restrict__ orders) {
    __shared__ uint64_t s_rows[VMAX * TPB];
    __shared__ uint64_t s_lvl[(VMAX + 1) * TPB];
    __shared__ uint32_t s_vd[VMAX * TPB];
    __shared__ uint16_t s_cm[64 * TPB];
    __shared__ uint8_t s_pc[64 * TPB];
    const unsigned tid = threadIdx.x;
    Smem sm{s_rows + tid, s_lvl + tid, s_pc + tid, s_cm + tid, s_vd + tid};
    for (;;) {
        const unsigned it = atomicAdd(ticket, 1u);
        if (it >= n_items)
            break;
        CheckOut o;
        check_one(sm, rows + (size_t)it * v, v, b, flags & ~F_SAVE_AUTS, max_trials, nullptr, 0, o,
                  orders ? orders[it] : ID16);
        canonical[it] = o.canonical;
        if (witness16)
            store_witness(witness16 + (size_t)it * 16u, o.witness, v);
        if (aut) {
            aut[2 * (size_t)it] = o.aut_lo;
            aut[2 * (size_t)it + 1] = o.aut_hi;
        }
        if (status)
            status[it] = o.status;
        if (trials_out)
            trials_out[it] = o.trials;
    }
}

// The resident check in two passes.  Pass 1 (this kernel): the lex-max search of
// every matrix gives the verdict and |Aut|; it needs neither permColumn nor the
// reference search's state, so it runs with less shared memory (the column masks
// sized by BCAP) and fewer registers.  Pass 2 (bibd_witness_kernel): the
// reference-order search, only for the matrices found non-canonical, gives the
// first rejecting permutation.
// BCAP / VCAP bound the columns / rows of the launch: the smaller the per-thread
// state, the more blocks fit an SM (v <= 15, b <= 35: 348 B, 10 blocks of 64).
template <int BCAP, int VCAP>
__global__ void __launch_bounds__(TPB) bibd_max_kernel(uint32_t n_items, uint32_t v, uint32_t b, uint32_t flags,
                                                       const uint64_t *__restrict__ rows, uint8_t *canonical,
                                                       uint64_t *aut, uint8_t *status, uint64_t max_nodes,
                                                       unsigned *ticket, const uint64_t *__restrict__ orders,
                                                       uint64_t *nodes_out) {
    __shared__ uint64_t s_rows[VCAP * TPB];
    __shared__ uint64_t s_lvl[(VCAP + 1) * TPB];
    __shared__ uint16_t s_vd[VCAP * TPB];
    __shared__ uint16_t s_cm[BCAP * TPB];
    const unsigned tid = threadIdx.x;
    SmemMax sm{s_rows + tid, s_lvl + tid, nullptr, s_cm + tid, s_vd + tid};
    for (;;) {
        const unsigned it = atomicAdd(ticket, 1u);
        if (it >= n_items)
            break;
        MaxOut mo{false, false, 0, 0, 0};
        uint8_t st = 0;
        if (!load_rows(sm, rows + (size_t)it * v, v, b, flags & F_RAW)) {
            st = ST_BADINPUT;
        } else {
            const uint64_t o0 = orders ? orders[it] : ID16;
            max_search(sm, v, b, max_nodes < CLIMB_CAP ? max_nodes : CLIMB_CAP, mo, o0);
            if (mo.timeout && max_nodes > CLIMB_CAP) {
                // the verdict and |Aut(M)| (= |Aut| of the canonical form) with the bound kept at M
                load_rows(sm, rows + (size_t)it * v, v, b, flags & F_RAW);
                max_search(sm, v, b, max_nodes - CLIMB_CAP, mo, o0, true, false, 0xFFFFu, nullptr, 0xFFFFu, nullptr, 0,
                           true);
                mo.nodes += CLIMB_CAP;
            }
            if (mo.timeout)
                st = ST_TIMEOUT;
        }
        const bool can = !st && !mo.improved;
        if (canonical)
            canonical[it] = can ? 1 : 0;
        if (status)
            status[it] = st;
        if (aut) {
            const bool has = !st && (can || (flags & (F_AUT_CANON | F_FULL_AUT)));
            aut[2 * (size_t)it] = has ? mo.leaves : 0;
            aut[2 * (size_t)it + 1] = 0;
        }
        if (nodes_out)
            nodes_out[it] = mo.nodes;
    }
}

// Automorphisms of canonical matrices (the parents of the next enumeration level):
// the pruned lex-max search of each, recording the automorphisms it finds while the
// matrix is still its own bound (at most gcap per matrix, row permutations
// nibble-packed); they prune the parent's children in the row generator.
__global__ void __launch_bounds__(TPB) bibd_autgen_kernel(uint32_t n_items, uint32_t v, uint32_t b,
                                                          const uint64_t *__restrict__ rows, uint64_t *gens,
                                                          uint8_t *ngens, uint32_t gcap, uint64_t max_nodes,
                                                          unsigned *ticket) {
    __shared__ uint64_t s_rows[VMAX * TPB];
    __shared__ uint64_t s_lvl[(VMAX + 1) * TPB];
    __shared__ uint16_t s_vd[VMAX * TPB];
    __shared__ uint16_t s_cm[64 * TPB];
    const unsigned tid = threadIdx.x;
    SmemMax sm{s_rows + tid, s_lvl + tid, nullptr, s_cm + tid, s_vd + tid};
    for (;;) {
        const unsigned it = atomicAdd(ticket, 1u);
        if (it >= n_items)
            break;
        MaxOut mo{};
        uint64_t *g = gens + (size_t)it * gcap;
        if (load_rows(sm, rows + (size_t)it * v, v, b, 0))
            max_search(sm, v, b, max_nodes, mo, ID16, true, false, 0xFFFFu, nullptr, 0xFFFFu, g, gcap);
        // a matrix found not canonical (or out of budget) prunes nothing
        ngens[it] = (uint8_t)((mo.improved || mo.timeout) ? 0 : mo.n_gens);
    }
}

// Throughput of the integer pipes on this GPU: every thread runs eight independent
// chains of 32-bit XOR / ADD / shift-add steps (LOP3 and IADD3 class operations)
// for `iters` rounds; a round is 24 operations per thread.  The result is stored
// only when it matches a value the caller never passes, so the work is not removed.
__global__ void __launch_bounds__(256) int_peak_kernel(uint32_t iters, uint32_t seed, uint32_t never,
                                                       uint32_t *sink) {
    uint32_t a0 = seed ^ threadIdx.x, a1 = a0 * 3u, a2 = a0 * 5u, a3 = a0 * 7u;
    uint32_t a4 = a0 * 11u, a5 = a0 * 13u, a6 = a0 * 17u, a7 = a0 * 19u;
    const uint32_t k = seed | 1u;
#pragma unroll 4
    for (uint32_t i = 0; i < iters; ++i) {
        a0 = ((a0 ^ k) + a1) ^ (a0 >> 1);
        a1 = ((a1 ^ k) + a2) ^ (a1 >> 1);
        a2 = ((a2 ^ k) + a3) ^ (a2 >> 1);
        a3 = ((a3 ^ k) + a4) ^ (a3 >> 1);
        a4 = ((a4 ^ k) + a5) ^ (a4 >> 1);
        a5 = ((a5 ^ k) + a6) ^ (a5 >> 1);
        a6 = ((a6 ^ k) + a7) ^ (a6 >> 1);
        a7 = ((a7 ^ k) + a0) ^ (a7 >> 1);
    }
    const uint32_t r = a0 ^ a1 ^ a2 ^ a3 ^ a4 ^ a5 ^ a6 ^ a7;
    if (r == never)
        sink[0] = r;
}

// Pass 1 in the converged layout (canon_bibd_conv.cuh): the same search, verdict,
// |Aut| and node count as bibd_max_kernel, with every iteration of the loop split
// into control steps (divergent, short) and one node step per thread -- the column
// arrangement for the chosen child and the evaluation of the new node, one pass over
// the b columns with the same trip count in every lane.  A thread that finishes its
// matrix takes the next one inside the control steps, so the lanes keep evaluating
// nodes together until the batch runs out.
template <int BCAP, int VCAP, unsigned RDEPTH = 4>
__global__ void __launch_bounds__(TPB) bibd_conv_kernel(uint32_t n_items, uint32_t v, uint32_t b, uint32_t flags,
                                                        const uint64_t *__restrict__ rows, uint8_t *canonical,
                                                        uint64_t *aut, uint8_t *status, uint64_t max_nodes,
                                                        unsigned *ticket, const uint64_t *__restrict__ orders,
                                                        uint64_t *nodes_out, uint64_t restart_after) {
    __shared__ uint64_t s_rows[VCAP * TPB];
    __shared__ uint64_t s_lvl[(VCAP + 1) * TPB];
    __shared__ uint16_t s_vd[VCAP * TPB];
    __shared__ uint16_t s_cm[BCAP * TPB];
    const unsigned tid = threadIdx.x;
    SmemMax sm{s_rows + tid, s_lvl + tid, nullptr, s_cm + tid, s_vd + tid};
    const bool want_aut = flags & (F_AUT_CANON | F_FULL_AUT);
    ConvState st{};
    uint32_t it = 0;
    bool have = false, done = false;
    // outputs of the matrix this thread has finished (status: 0, ST_BADINPUT, ST_TIMEOUT)
    auto finish = [&](uint8_t stat) {
        const bool can = !stat && !conv_rejected(st);
        if (canonical)
            canonical[it] = can ? 1 : 0;
        if (status)
            status[it] = stat;
        if (aut) {
            aut[2 * (size_t)it] = (!stat && (can || want_aut)) ? conv_leaves(st) : 0;
            aut[2 * (size_t)it + 1] = 0;
        }
        if (nodes_out)
            nodes_out[it] = st.nodes;
        have = false;
    };
    for (;;) {
        // control steps until this thread has a node to evaluate, or no work is left
        int ref_lv = -1;
        unsigned ref_x = 0;
        bool eval = false;
        while (!done && !eval) {
            if (!have) {
                it = atomicAdd(ticket, 1u);
                if (it >= n_items) {
                    done = true;
                    break;
                }
                conv_start(st, v, orders ? orders[it] : ID16);
                st.b = b;
                st.restart_after = restart_after;
                st.verdict_only = flags & F_VERDICT_ONLY;
                have = true;
                if (!load_rows(sm, rows + (size_t)it * v, v, b, flags & F_RAW)) {
                    finish(ST_BADINPUT);
                    continue;
                }
                // columns past the matrix's own are empty: they join its last orbit and change
                // neither a count nor a comparison
                for (unsigned c2 = b; c2 < (unsigned)BCAP; ++c2)
                    CM_(c2) = 0;
                st.w = conv_row_weight(sm, v);
                eval = true;        // the root: no arrangement step
                break;
            }
            if (conv_next(sm, st, ref_lv, ref_x)) {
                eval = true;
                break;
            }
            finish(0);
        }
        if (__all_sync(0xFFFFFFFFu, done))
            break;
        if (!eval)
            continue;
        // the node step: every lane with a node runs the same b-column passes (unrolled
        // when the batch's b is the instance's column capacity)
        // the unrolled node step over the instance's BCAP columns when the matrix fills at
        // least three quarters of them (the rest are empty), else a loop over its b columns
        const bool full = (BCAP - b) * 4 <= (unsigned)BCAP;
        if (ref_lv >= 0) {
            if (full)
                refine_uniform<BCAP, RDEPTH>(sm, (unsigned)ref_lv, ref_x, b);
            else
                refine_uniform(sm, (unsigned)ref_lv, ref_x, b);
        }
        if (++st.nodes > max_nodes) {
            st.timeout = true;
            finish(ST_TIMEOUT);
            continue;
        }
        unsigned tied = st.allrows & ~st.used;
        uint64_t arr = 0;
        const bool hb = st.i < st.valid;
        const uint64_t bnd = hb ? R_(st.i) : 0ull;
        // count planes for the heaviest row among the lanes stepping together
        const unsigned w = __reduce_max_sync(__activemask(), st.w);
        const int state = full ? eval_node_planes<BCAP>(sm, w, st.i, b, b, tied, arr, hb, bnd)
                               : eval_node_planes(sm, w, st.i, b, b, tied, arr, hb, bnd);
        if (!conv_after_eval(sm, st, state, tied, arr, b))
            finish(0);
    }
}

// The lex-max pass over work items (the batched path: canon_sync, and the check
// without allocation) in the converged layout.  Items may differ in rows and
// columns; every lane walks bt columns (the widest item of the launch), the
// columns past an item's own being empty.
template <int BCAP, int VCAP>
__global__ void __launch_bounds__(TPB) bibd_items_conv_kernel(const Item *__restrict__ items, uint32_t n_items,
                                                              const uint64_t *__restrict__ words, Outputs out,
                                                              uint64_t max_nodes, unsigned *ticket, uint32_t bt,
                                                              uint64_t restart_after) {
    __shared__ uint64_t s_rows[VCAP * TPB];
    __shared__ uint64_t s_lvl[(VCAP + 1) * TPB];
    __shared__ uint16_t s_vd[VCAP * TPB];
    __shared__ uint16_t s_cm[BCAP * TPB];
    const unsigned tid = threadIdx.x;
    SmemMax sm{s_rows + tid, s_lvl + tid, nullptr, s_cm + tid, s_vd + tid};
    ConvState st{};
    uint32_t o_i = 0;
    unsigned b = 1;
    bool have = false, done = false;
    auto finish = [&](uint8_t stat) {
        const bool can = !stat && !conv_rejected(st);
        out.canonical[o_i] = can ? 1 : 0;
        out.status[o_i] = stat;
        out.aut[2 * (size_t)o_i] = stat ? 0 : conv_leaves(st);
        out.aut[2 * (size_t)o_i + 1] = 0;
        out.player_index[o_i] = -1;
        out.n_auts[o_i] = 0;
        out.len_aut[o_i] = 0;
        have = false;
    };
    for (;;) {
        int ref_lv = -1;
        unsigned ref_x = 0;
        bool eval = false;
        while (!done && !eval) {
            if (!have) {
                const unsigned it = atomicAdd(ticket, 1u);
                if (it >= n_items) {
                    done = true;
                    break;
                }
                const Item item = items[it];
                const unsigned n = item.nrows;
                b = item.ncols;
                o_i = item.out_idx;
                conv_start(st, n >= 1 && n <= VCAP ? n : 1, ID16);
                st.b = b;
                st.restart_after = restart_after;
                st.verdict_only = item.flags & F_VERDICT_ONLY;
                have = true;
                if (item.kind != KIND_BIBD || n < 1 || n > VCAP || b < 1 || b > BMAX || b > BCAP || b > bt ||
                    !load_rows(sm, words + item.data_off, n, b, item.flags & F_RAW)) {
                    finish(ST_BADINPUT);
                    continue;
                }
                for (unsigned c = b; c < bt; ++c)
                    CM_(c) = 0;
                st.w = conv_row_weight(sm, n);
                eval = true;
                break;
            }
            if (conv_next(sm, st, ref_lv, ref_x)) {
                eval = true;
                break;
            }
            finish(0);
        }
        if (__all_sync(0xFFFFFFFFu, done))
            break;
        if (!eval)
            continue;
        // unrolled when every item of the launch has the instance's column capacity
        // (bt == BCAP then holds for all lanes, and b == bt for every lane with a node)
        const bool full = bt == BCAP && b == BCAP;
        if (ref_lv >= 0) {
            if (full)
                refine_uniform<BCAP>(sm, (unsigned)ref_lv, ref_x, bt);
            else
                refine_uniform(sm, (unsigned)ref_lv, ref_x, bt);
        }
        if (++st.nodes > max_nodes) {
            st.timeout = true;
            finish(ST_TIMEOUT);
            continue;
        }
        unsigned tied = st.allrows & ~st.used;
        uint64_t arr = 0;
        const bool hb = st.i < st.valid;
        const uint64_t bnd = hb ? R_(st.i) : 0ull;
        const unsigned w = __reduce_max_sync(__activemask(), st.w);
        const int state = full ? eval_node_planes<BCAP>(sm, w, st.i, b, bt, tied, arr, hb, bnd)
                               : eval_node_planes(sm, w, st.i, b, bt, tied, arr, hb, bnd);
        if (!conv_after_eval(sm, st, state, tied, arr, b))
            finish(0);
    }
}

// Pass 2: the first rejecting permutation (reference order) of the matrices that
// pass 1 found non-canonical; the others get the 0xFF witness.
__global__ void __launch_bounds__(TPB) bibd_witness_kernel(uint32_t n_items, uint32_t v, uint32_t b, uint32_t flags,
                                                           const uint64_t *__restrict__ rows,
                                                           const uint8_t *__restrict__ canonical,
                                                           uint8_t *witness16, uint8_t *status, uint64_t *trials_out,
                                                           uint64_t max_trials, unsigned *ticket) {
    __shared__ uint64_t s_rows[VMAX * TPB];
    __shared__ uint64_t s_lvl[(VMAX + 1) * TPB];
    __shared__ uint32_t s_vd[VMAX * TPB];
    __shared__ uint16_t s_cm[64 * TPB];
    __shared__ uint8_t s_pc[64 * TPB];
    const unsigned tid = threadIdx.x;
    Smem sm{s_rows + tid, s_lvl + tid, s_pc + tid, s_cm + tid, s_vd + tid};
    for (;;) {
        const unsigned it = atomicAdd(ticket, 1u);
        if (it >= n_items)
            break;
        const uint8_t st0 = status ? status[it] : 0;
        CheckOut o;
        reset_out(o);
        if (!canonical[it] && !st0) {
            load_rows(sm, rows + (size_t)it * v, v, b, flags & F_RAW);
            search(sm, v, b, flags & F_COMPLETE, max_trials, nullptr, 0, o);
            if ((o.status & ST_TIMEOUT) && status)
                status[it] = o.status;
        }
        if (witness16)
            store_witness(witness16 + (size_t)it * 16u, o.witness, v);
        if (trials_out)
            trials_out[it] = o.trials;
    }
}

// The two passes over work items of any shape (the batched path); BCAP bounds the
// columns of every item of the launch, as in bibd_max_kernel.
template <unsigned BCAP, unsigned VCAP>
__global__ void __launch_bounds__(TPB) bibd_items_max_kernel(const Item *__restrict__ items, uint32_t n_items,
                                                             const uint64_t *__restrict__ words, Outputs out,
                                                             uint64_t max_nodes, unsigned *ticket) {
    __shared__ uint64_t s_rows[VCAP * TPB];
    __shared__ uint64_t s_lvl[(VCAP + 1) * TPB];
    __shared__ uint16_t s_vd[VCAP * TPB];
    __shared__ uint16_t s_cm[BCAP * TPB];
    const unsigned tid = threadIdx.x;
    SmemMax sm{s_rows + tid, s_lvl + tid, nullptr, s_cm + tid, s_vd + tid};
    for (;;) {
        const unsigned it = atomicAdd(ticket, 1u);
        if (it >= n_items)
            break;
        const Item item = items[it];
        const unsigned n = item.nrows, b = item.ncols, o_i = item.out_idx;
        MaxOut mo{false, false, 0, 0, 0};
        uint8_t st = 0;
        if (item.kind != KIND_BIBD || n < 1 || n > VCAP || b < 1 || b > BMAX || b > BCAP ||
            !load_rows(sm, words + item.data_off, n, b, item.flags & F_RAW)) {
            st = ST_BADINPUT;
        } else {
            max_search(sm, n, b, max_nodes < CLIMB_CAP ? max_nodes : CLIMB_CAP, mo);
            if (mo.timeout && max_nodes > CLIMB_CAP) {
                load_rows(sm, words + item.data_off, n, b, item.flags & F_RAW);
                max_search(sm, n, b, max_nodes - CLIMB_CAP, mo, ID16, true, false, 0xFFFFu, nullptr, 0xFFFFu, nullptr, 0,
                           true);
                mo.nodes += CLIMB_CAP;
            }
            if (mo.timeout)
                st = ST_TIMEOUT;
        }
        const bool can = !st && !mo.improved;
        out.canonical[o_i] = can ? 1 : 0;
        out.status[o_i] = st;
        out.aut[2 * (size_t)o_i] = st ? 0 : mo.leaves;
        out.aut[2 * (size_t)o_i + 1] = 0;
        out.player_index[o_i] = -1;
        out.n_auts[o_i] = 0;
        out.len_aut[o_i] = 0;
    }
}

__global__ void __launch_bounds__(TPB) bibd_items_witness_kernel(const Item *__restrict__ items, uint32_t n_items,
                                                                 const uint64_t *__restrict__ words, Outputs out,
                                                                 uint64_t max_trials, unsigned *ticket) {
    __shared__ uint64_t s_rows[VMAX * TPB];
    __shared__ uint64_t s_lvl[(VMAX + 1) * TPB];
    __shared__ uint32_t s_vd[VMAX * TPB];
    __shared__ uint16_t s_cm[64 * TPB];
    __shared__ uint8_t s_pc[64 * TPB];
    const unsigned tid = threadIdx.x;
    Smem sm{s_rows + tid, s_lvl + tid, s_pc + tid, s_cm + tid, s_vd + tid};
    for (;;) {
        const unsigned it = atomicAdd(ticket, 1u);
        if (it >= n_items)
            break;
        const Item item = items[it];
        const unsigned n = item.nrows, b = item.ncols, o_i = item.out_idx;
        CheckOut o;
        reset_out(o);
        if (!out.canonical[o_i] && !out.status[o_i]) {
            load_rows(sm, words + item.data_off, n, b, item.flags & F_RAW);
            search(sm, n, b, item.flags & F_COMPLETE, max_trials, nullptr, 0, o);
            if (o.status & ST_TIMEOUT)
                out.status[o_i] = o.status;
        }
        out.reject_row[o_i] = o.reject_row;
        out.row_to_change[o_i] = o.rtc;
        store_witness(out.witness + (size_t)o_i * 16u, o.witness, n);
        out.trials[o_i] = o.trials;
    }
}

// CanonizeMatrix(k = 0), MatrixCanonChecker.cpp:420-564: the matrix is replaced by
// its canonical form, the lex-max matrix that the reference reaches by repeated
// checks; the lex-max search finds it directly, together with |Aut|.
__global__ void __launch_bounds__(TPB) bibd_canonize_kernel(uint32_t n_items, uint32_t v, uint32_t b,
                                                            uint64_t *rows, uint64_t *aut, uint8_t *status,
                                                            uint32_t stride_items, uint32_t first_item,
                                                            uint64_t max_trials, unsigned *ticket) {
    __shared__ uint64_t s_rows[VMAX * TPB];
    __shared__ uint64_t s_lvl[(VMAX + 1) * TPB];
    __shared__ uint32_t s_vd[VMAX * TPB];
    __shared__ uint16_t s_cm[64 * TPB];
    __shared__ uint8_t s_pc[64 * TPB];
    const unsigned tid = threadIdx.x;
    Smem sm{s_rows + tid, s_lvl + tid, s_pc + tid, s_cm + tid, s_vd + tid};
    for (;;) {
        const unsigned t = atomicAdd(ticket, 1u);
        const uint64_t it64 = (uint64_t)first_item + (uint64_t)t * stride_items;
        if (it64 >= n_items)
            break;
        const size_t it = (size_t)it64;
        uint8_t st = 0;
        MaxOut mo{false, false, 0, 0};
        if (!load_rows(sm, rows + it * v, v, b, F_RAW)) {
            st = ST_BADINPUT;
        } else {
            max_search(sm, v, b, max_trials, mo);
            if (mo.timeout)
                st = ST_TIMEOUT;
            else
                for (unsigned r = 0; r < v; ++r)
                    rows[it * v + r] = R_(r);
        }
        if (aut) {
            aut[2 * it] = st ? 0 : mo.leaves;
            aut[2 * it + 1] = 0;
        }
        if (status)
            status[it] = st;
    }
}

// Training labels of the learned order: for every matrix the set of rows that
// start a labeling reaching its canonical form (the first rows of the lex-max
// search's leaves), with |Aut| and the node count of the plain order.
__global__ void __launch_bounds__(TPB) bibd_label_kernel(uint32_t n_items, uint32_t v, uint32_t b, uint32_t flags,
                                                         const uint64_t *__restrict__ rows, uint16_t *first_rows,
                                                         uint64_t *nodes, const uint64_t *__restrict__ orders,
                                                         uint64_t max_nodes, unsigned *ticket) {
    __shared__ uint64_t s_rows[VMAX * TPB];
    __shared__ uint64_t s_lvl[(VMAX + 1) * TPB];
    __shared__ uint32_t s_vd[VMAX * TPB];
    __shared__ uint16_t s_cm[64 * TPB];
    __shared__ uint8_t s_pc[64 * TPB];
    const unsigned tid = threadIdx.x;
    Smem sm{s_rows + tid, s_lvl + tid, s_pc + tid, s_cm + tid, s_vd + tid};
    for (;;) {
        const unsigned it = atomicAdd(ticket, 1u);
        if (it >= n_items)
            break;
        MaxOut mo{false, false, 0, 0, 0};
        if (load_rows(sm, rows + (size_t)it * v, v, b, flags & F_RAW))
            // unpruned when node counts are asked for: they stay comparable between
            // search orders (the first rows are the same either way)
            max_search(sm, v, b, max_nodes, mo, orders ? orders[it] : ID16, nodes == nullptr);
        if (first_rows)
            first_rows[it] = (uint16_t)(mo.timeout ? 0 : mo.first_rows);
        if (nodes)
            nodes[it] = mo.nodes;
    }
}

// The verdict of a small batch with the lex-max search split by its first rows:
// one thread per (matrix, first row) -- or, with levels = 2, per (matrix, first
// row, second row) -- so a level of few matrices still fills the GPU and a
// check's latency is that of its largest subtree, not of the whole search.
// Thread (0[, 1]) takes the identity path and gives the orbit lengths below; the
// others stop each subtree at its first automorphism; the first thread of a
// matrix to improve on M raises its stop flag.  bibd_split_combine_kernel forms
// the verdict and |Aut| = |orbit of row 0| (x |orbit of row 1 under the
// stabilizer of row 0|) x the identity thread's product.
__global__ void __launch_bounds__(TPB) bibd_split_kernel(uint32_t n_items, uint32_t v, uint32_t b, uint32_t flags,
                                                         uint32_t levels, const uint64_t *__restrict__ rows,
                                                         SplitPart *parts, unsigned *stop, uint64_t max_nodes,
                                                         unsigned *ticket) {
    __shared__ uint64_t s_rows[VMAX * TPB];
    __shared__ uint64_t s_lvl[(VMAX + 1) * TPB];
    __shared__ uint16_t s_vd[VMAX * TPB];
    __shared__ uint16_t s_cm[64 * TPB];
    const unsigned tid = threadIdx.x;
    SmemMax sm{s_rows + tid, s_lvl + tid, nullptr, s_cm + tid, s_vd + tid};
    const unsigned per = levels == 2 ? v * v : v;
    const uint64_t total = (uint64_t)n_items * per;
    for (;;) {
        const unsigned it = atomicAdd(ticket, 1u);
        if (it >= total)
            break;
        const unsigned item = it / per, r = it - item * per;
        const unsigned j = levels == 2 ? r / v : r, k = levels == 2 ? r - (r / v) * v : 0u;
        const unsigned mask1 = levels == 2 ? (1u << k) : 0xFFFFu;
        MaxOut mo{false, false, 0, 0, 0, 0, 0};
        uint8_t st = 0;
        if (levels == 2 && j == k) {
            // no path starts with the same row twice
        } else if (!load_rows(sm, rows + (size_t)item * v, v, b, flags & F_RAW)) {
            st = ST_BADINPUT;
        } else if (!((volatile unsigned *)stop)[item]) {
            max_search(sm, v, b, max_nodes, mo, ID16, true, true, 1u << j, stop + item, mask1);
            if (mo.timeout)
                st = ST_TIMEOUT;
            if (mo.improved)
                atomicExch(stop + item, 1u);
        }
        SplitPart p;
        p.leaves = mo.leaves;
        p.orbit0 = (uint8_t)mo.orbit0;
        p.orbit1 = (uint8_t)mo.orbit1;
        p.improved = mo.improved ? 1 : 0;
        p.status = st;
        parts[it] = p;
    }
}

__global__ void bibd_split_combine_kernel(uint32_t n_items, uint32_t v, uint32_t levels, const SplitPart *parts,
                                          const unsigned *stop, uint8_t *canonical, uint64_t *aut,
                                          uint8_t *status) {
    const unsigned per = levels == 2 ? v * v : v;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_items; i += gridDim.x * blockDim.x) {
        const SplitPart *p = parts + (size_t)i * per;
        uint8_t st = 0;
        for (uint32_t q = 0; q < per; ++q)
            st |= p[q].status;
        uint64_t order = 0;
        if (levels == 2) {
            // rows 1.. that some thread (j, k) mapped row 0 to, rows 2.. mapped to row 1
            uint64_t o0 = 1, o1 = 1;
            for (uint32_t j = 1; j < v; ++j) {
                bool any = false;
                for (uint32_t k = 0; k < v; ++k)
                    any = any || p[j * v + k].orbit0;
                o0 += any;
            }
            for (uint32_t k = 2; k < v; ++k)
                o1 += p[k].orbit1;
            order = o0 * o1 * p[1].leaves;
        } else {
            unsigned total0 = 0;
            for (uint32_t j = 0; j < v; ++j)
                total0 += p[j].orbit0;
            order = (uint64_t)total0 * (p[0].leaves / (p[0].orbit0 ? p[0].orbit0 : 1));
        }
        const bool improved = stop[i] != 0;
        if (improved)
            st &= (uint8_t)~ST_TIMEOUT;          // decided: another thread showed M not canonical
        const bool can = !st && !improved;
        canonical[i] = can ? 1 : 0;
        if (aut) {
            aut[2 * (size_t)i] = can ? order : 0;
            aut[2 * (size_t)i + 1] = 0;
        }
        if (status)
            status[i] = st;
    }
}

// Persistent grid: resident blocks per SM x SMs, at most `need` blocks.  A failed
// occupancy query is returned instead of launching a guessed size.
cudaError_t grid_for(const void *kernel, int num_sms, int need, int *grid) {
    int per_sm = 0;
    const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, TPB, 0);
    if (e != cudaSuccess)
        return e;
    if (per_sm < 1)
        per_sm = 1;
    const int g = per_sm * (num_sms > 0 ? num_sms : 1);
    *grid = g < need ? g : need;
    return cudaSuccess;
}

// the restart threshold of the converged lex-max search (nodes).  On 1M STS(15) checks
// (two seeds) 7K - 10K nodes measured best: 0.73 s per batch, against 0.74 s at 14K,
// 0.90 s at 4K and 0.81 - 1.30 s without the restart.
uint64_t restart_nodes() { return RESTART_AFTER; }

#define CANON_TRY(x)                          \
    do {                                      \
        const cudaError_t e_ = (x);           \
        if (e_ != cudaSuccess)                \
            return e_;                        \
    } while (0)

}  // namespace

cudaError_t launch_bibd_check(const Item *d_items, uint32_t n_items, const uint64_t *d_words, Outputs out,
                              uint64_t max_trials, unsigned *tk, int num_sms, cudaStream_t s) {
    if (!n_items)
        return cudaSuccess;
    CANON_TRY(cudaMemsetAsync(tk, 0, sizeof(unsigned), s));
    const int need = (int)((n_items + TPB - 1) / TPB);
    int grid = 0;
    CANON_TRY(grid_for((const void *)bibd_items_kernel, num_sms, need, &grid));
    bibd_items_kernel<<<grid, TPB, 0, s>>>(d_items, n_items, d_words, out, max_trials, tk);
    return cudaGetLastError();
}

cudaError_t launch_bibd_check_two_pass(const Item *d_items, uint32_t n_items, const uint64_t *d_words, Outputs out,
                                       uint64_t max_trials, unsigned *tk, int num_sms, cudaStream_t s,
                                       uint32_t max_b, uint32_t max_v) {
    if (!n_items)
        return cudaSuccess;
    CANON_TRY(cudaMemsetAsync(tk, 0, 2 * sizeof(unsigned), s));
    const int need = (int)((n_items + TPB - 1) / TPB);
    const int shape = (max_v <= 15 && max_b <= 35) ? 0 : (max_b <= 40 ? 1 : 2);
    const uint32_t bt = max_b < 1 ? 1 : (max_b > BMAX ? BMAX : max_b);
    // the lex-max pass in the converged layout (every lane walks the widest item's columns)
    const void *kfn = shape == 0 ? (const void *)bibd_items_conv_kernel<35, 15>
                      : shape == 1 ? (const void *)bibd_items_conv_kernel<40, 16>
                                   : (const void *)bibd_items_conv_kernel<64, 16>;
    int grid = 0;
    CANON_TRY(grid_for(kfn, num_sms, need, &grid));
    if (shape == 0)
        bibd_items_conv_kernel<35, 15><<<grid, TPB, 0, s>>>(d_items, n_items, d_words, out, max_trials, tk, bt,
                                                            restart_nodes());
    else if (shape == 1)
        bibd_items_conv_kernel<40, 16><<<grid, TPB, 0, s>>>(d_items, n_items, d_words, out, max_trials, tk, bt,
                                                            restart_nodes());
    else
        bibd_items_conv_kernel<64, 16><<<grid, TPB, 0, s>>>(d_items, n_items, d_words, out, max_trials, tk, bt,
                                                            restart_nodes());
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    int g2 = 0;
    CANON_TRY(grid_for((const void *)bibd_items_witness_kernel, num_sms, need, &g2));
    bibd_items_witness_kernel<<<g2, TPB, 0, s>>>(d_items, n_items, d_words, out, max_trials, tk + 1);
    return cudaGetLastError();
}

cudaError_t launch_bibd_check_uniform(uint32_t n, uint32_t v, uint32_t b, uint32_t flags,
                                      const uint64_t *d_rows, uint8_t *d_canonical, uint8_t *d_witness16,
                                      uint64_t *d_aut, uint8_t *d_status, uint64_t *d_trials,
                                      uint64_t max_trials, unsigned *tk, int num_sms, cudaStream_t s,
                                      const uint64_t *d_orders, int variant) {
    if (!n)
        return cudaSuccess;
    const int need = (int)((n + TPB - 1) / TPB);
    const bool ref_order = flags & (F_SAVE_AUTS | F_REFERENCE_ORDER);
    const bool depth_variant = variant == VARIANT_CONVERGED_D2 || variant == VARIANT_CONVERGED_D8;
    const bool two = !ref_order && (variant < 0 ? (flags & (F_AUT_CANON | F_FULL_AUT)) != 0
                                                : (variant == VARIANT_TWO_PASS || variant == VARIANT_CONVERGED ||
                                                   depth_variant));
    // the converged layout of the lex-max pass by default; the original one only when
    // the autotuner asks for it by name
    const bool conv = variant != VARIANT_TWO_PASS;
    if (two) {
        // |Aut| wanted for every matrix: two passes, the lex-max search for all,
        // the reference-order witness for the rejected ones.  (Without it the
        // single pass below rejects most non-canonical matrices in a few trials
        // of the reference order and runs the lex-max search only for the rest.)
        CANON_TRY(cudaMemsetAsync(tk, 0, 2 * sizeof(unsigned), s));
        // the smallest instance that holds the shape (the converged pass also has one of 24
        // columns)
        const int shape = (v <= 15 && b <= 35) ? 0 : (b <= 40 ? 1 : 2);
        const bool narrow = conv && b <= 24;
        // the staging depth of the arrangement's loads (2 / 4 / 8 columns ahead): the
        // autotuner's variants, instantiated for the 15 x 35 instance
        const unsigned depth = (shape == 0 && variant == VARIANT_CONVERGED_D2)   ? 2u
                               : (shape == 0 && variant == VARIANT_CONVERGED_D8) ? 8u
                                                                                 : 4u;
        const void *kfn = narrow ? (const void *)bibd_conv_kernel<24, 16>
                          : conv ? (shape == 0   ? (depth == 2   ? (const void *)bibd_conv_kernel<35, 15, 2>
                                                  : depth == 8 ? (const void *)bibd_conv_kernel<35, 15, 8>
                                                               : (const void *)bibd_conv_kernel<35, 15>)
                                  : shape == 1 ? (const void *)bibd_conv_kernel<40, 16>
                                               : (const void *)bibd_conv_kernel<64, 16>)
                               : (shape == 0   ? (const void *)bibd_max_kernel<35, 15>
                                  : shape == 1 ? (const void *)bibd_max_kernel<40, 16>
                                               : (const void *)bibd_max_kernel<64, 16>);
        int grid = 0;
        CANON_TRY(grid_for(kfn, num_sms, need, &grid));
#define CANON_PASS1(K, BC, VC, ...)                                                                             \
    K<BC, VC><<<grid, TPB, 0, s>>>(n, v, b, flags, d_rows, d_canonical, d_aut, d_status, max_trials, tk, d_orders, \
                                   nullptr __VA_ARGS__)
#define CANON_PASS1D(BC, VC, RA, D)                                                                                \
    bibd_conv_kernel<BC, VC, D><<<grid, TPB, 0, s>>>(n, v, b, flags, d_rows, d_canonical, d_aut, d_status, max_trials, \
                                                     tk, d_orders, nullptr, RA)
        if (conv) {
            const uint64_t ra = restart_nodes();
            if (narrow)
                CANON_PASS1(bibd_conv_kernel, 24, 16, , ra);
            else if (shape == 0 && depth == 2)
                CANON_PASS1D(35, 15, ra, 2);
            else if (shape == 0 && depth == 8)
                CANON_PASS1D(35, 15, ra, 8);
            else if (shape == 0)
                CANON_PASS1(bibd_conv_kernel, 35, 15, , ra);
            else if (shape == 1)
                CANON_PASS1(bibd_conv_kernel, 40, 16, , ra);
            else
                CANON_PASS1(bibd_conv_kernel, 64, 16, , ra);
        } else {
            if (shape == 0)
                CANON_PASS1(bibd_max_kernel, 35, 15);
            else if (shape == 1)
                CANON_PASS1(bibd_max_kernel, 40, 16);
            else
                CANON_PASS1(bibd_max_kernel, 64, 16);
        }
#undef CANON_PASS1
#undef CANON_PASS1D
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess)
            return e;
        if (d_witness16 || d_trials) {
            int g2 = 0;
            CANON_TRY(grid_for((const void *)bibd_witness_kernel, num_sms, need, &g2));
            bibd_witness_kernel<<<g2, TPB, 0, s>>>(n, v, b, flags, d_rows, d_canonical, d_witness16, d_status,
                                                   d_trials, max_trials, tk + 1);
        }
        return cudaGetLastError();
    }
    CANON_TRY(cudaMemsetAsync(tk, 0, sizeof(unsigned), s));
    int grid = 0;
    CANON_TRY(grid_for((const void *)bibd_uniform_kernel, num_sms, need, &grid));
    bibd_uniform_kernel<<<grid, TPB, 0, s>>>(n, v, b, flags, d_rows, d_canonical, d_witness16, d_aut, d_status,
                                             d_trials, max_trials, tk, d_orders);
    return cudaGetLastError();
}

cudaError_t launch_bibd_lexmax_nodes(uint32_t n, uint32_t v, uint32_t b, uint32_t flags, const uint64_t *d_rows,
                                     uint64_t *d_nodes, uint64_t max_nodes, unsigned *tk, int num_sms,
                                     cudaStream_t s, const uint64_t *d_orders) {
    if (!n)
        return cudaSuccess;
    CANON_TRY(cudaMemsetAsync(tk, 0, sizeof(unsigned), s));
    const int need = (int)((n + TPB - 1) / TPB);
    const uint64_t ra = restart_nodes();
    int grid = 0;
    // the lex-max pass the resident check runs (converged layout), counting its nodes
#define CANON_NODES(BC, VC)                                                                                    \
    do {                                                                                                       \
        CANON_TRY(grid_for((const void *)bibd_conv_kernel<BC, VC>, num_sms, need, &grid));                     \
        bibd_conv_kernel<BC, VC><<<grid, TPB, 0, s>>>(n, v, b, flags, d_rows, nullptr, nullptr, nullptr, max_nodes, \
                                                      tk, d_orders, d_nodes, ra);                              \
    } while (0)
    if (b <= 24)
        CANON_NODES(24, 16);
    else if (v <= 15 && b <= 35)
        CANON_NODES(35, 15);
    else if (b <= 40)
        CANON_NODES(40, 16);
    else
        CANON_NODES(64, 16);
#undef CANON_NODES
    return cudaGetLastError();
}

cudaError_t launch_bibd_autgen(uint32_t n, uint32_t v, uint32_t b, const uint64_t *d_rows, uint64_t *d_gens,
                               uint8_t *d_ngens, uint32_t gcap, uint64_t max_nodes, unsigned *tk, int num_sms,
                               cudaStream_t s) {
    if (!n)
        return cudaSuccess;
    CANON_TRY(cudaMemsetAsync(tk, 0, sizeof(unsigned), s));
    const int need = (int)((n + TPB - 1) / TPB);
    int grid = 0;
    CANON_TRY(grid_for((const void *)bibd_autgen_kernel, num_sms, need, &grid));
    bibd_autgen_kernel<<<grid, TPB, 0, s>>>(n, v, b, d_rows, d_gens, d_ngens, gcap, max_nodes, tk);
    return cudaGetLastError();
}

cudaError_t launch_int_peak(uint32_t iters, int num_sms, uint32_t *d_sink, cudaStream_t s, uint64_t *ops) {
    const int grid = 8 * (num_sms > 0 ? num_sms : 1);
    int_peak_kernel<<<grid, 256, 0, s>>>(iters, 0x9E3779B9u, 0xFFFFFFFFu, d_sink);
    *ops = (uint64_t)grid * 256u * iters * 32u;
    return cudaGetLastError();
}

cudaError_t launch_bibd_labels(uint32_t n, uint32_t v, uint32_t b, uint32_t flags, const uint64_t *d_rows,
                               uint16_t *d_first_rows, uint64_t *d_nodes, const uint64_t *d_orders,
                               uint64_t max_nodes, unsigned *tk, int num_sms, cudaStream_t s) {
    if (!n)
        return cudaSuccess;
    CANON_TRY(cudaMemsetAsync(tk, 0, sizeof(unsigned), s));
    const int need = (int)((n + TPB - 1) / TPB);
    int grid = 0;
    CANON_TRY(grid_for((const void *)bibd_label_kernel, num_sms, need, &grid));
    bibd_label_kernel<<<grid, TPB, 0, s>>>(n, v, b, flags, d_rows, d_first_rows, d_nodes, d_orders, max_nodes, tk);
    return cudaGetLastError();
}

cudaError_t launch_bibd_check_split(uint32_t n, uint32_t v, uint32_t b, uint32_t flags, const uint64_t *d_rows,
                                    uint8_t *d_canonical, uint64_t *d_aut, uint8_t *d_status, SplitPart *d_parts,
                                    unsigned *d_stop, uint64_t max_trials, unsigned *tk, int num_sms,
                                    cudaStream_t s) {
    if (!n)
        return cudaSuccess;
    // two levels while the threads stay few enough (the parts hold n * v * v)
    const uint32_t levels = split_levels(n, v);
    CANON_TRY(cudaMemsetAsync(tk, 0, sizeof(unsigned), s));
    CANON_TRY(cudaMemsetAsync(d_stop, 0, (size_t)n * sizeof(unsigned), s));
    const uint64_t work = (uint64_t)n * (levels == 2 ? v * v : v);
    const int need = (int)((work + TPB - 1) / TPB);
    int grid = 0;
    CANON_TRY(grid_for((const void *)bibd_split_kernel, num_sms, need, &grid));
    bibd_split_kernel<<<grid, TPB, 0, s>>>(n, v, b, flags, levels, d_rows, d_parts, d_stop, max_trials, tk);
    CANON_TRY(cudaGetLastError());
    const int g2 = (int)((n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024);
    bibd_split_combine_kernel<<<g2, 256, 0, s>>>(n, v, levels, d_parts, d_stop, d_canonical, d_aut, d_status);
    return cudaGetLastError();
}

cudaError_t launch_bibd_canonize(uint32_t n, uint32_t v, uint32_t b, uint64_t *d_rows, uint64_t *d_aut,
                                 uint8_t *d_status, uint32_t stride_items, uint32_t first_item,
                                 uint64_t max_trials, unsigned *tk, int num_sms, cudaStream_t s) {
    if (!n || first_item >= n || !stride_items)
        return cudaSuccess;
    CANON_TRY(cudaMemsetAsync(tk, 0, sizeof(unsigned), s));
    const uint32_t cnt = (n - first_item + stride_items - 1) / stride_items;
    const int need = (int)((cnt + TPB - 1) / TPB);
    int grid = 0;
    CANON_TRY(grid_for((const void *)bibd_canonize_kernel, num_sms, need, &grid));
    bibd_canonize_kernel<<<grid, TPB, 0, s>>>(n, v, b, d_rows, d_aut, d_status, stride_items, first_item,
                                              max_trials, tk);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// canon_check_bibd_noalloc(): the batched check for callers that cannot
// allocate device memory.  Its scratch -- one work descriptor per matrix and the
// work-stealing counter -- lives in this file-scope array instead of in a
// context; every GPU that loads the library holds it until the process exits.
// ---------------------------------------------------------------------------
namespace {

constexpr uint32_t NOALLOC_MAX_ITEMS = CANON_NOALLOC_MAX_ITEMS;     // 65,536 work descriptors
constexpr size_t NOALLOC_COUNTER_OFF = (size_t)NOALLOC_MAX_ITEMS * sizeof(Item);
constexpr size_t NOALLOC_SCRATCH_BYTES = NOALLOC_COUNTER_OFF + 256;   // 1 MiB + 256 B

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mutex;
unsigned char *g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};
int g_noalloc_sms[NOALLOC_MAX_DEVICES] = {};

// one work descriptor per matrix, read from the caller's device arrays
__global__ void noalloc_fill_items(Item *items, uint32_t n, uint32_t v, uint32_t b, uint32_t flags,
                                   const uint8_t *__restrict__ nrows) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t nr = nrows ? nrows[i] : v;
        Item it{};
        it.data_off = i * v;
        it.kind = (nr >= 1 && nr <= v) ? KIND_BIBD : 0xFFu;   // out-of-range rows: flagged bad input
        it.nrows = (uint8_t)nr;
        it.ncols = (uint8_t)b;
        it.flags = (uint8_t)flags;
        it.out_idx = i;
        items[i] = it;
    }
}

// Device address of the scratch on the current device, found once per device.
cudaError_t noalloc_scratch(unsigned char **ptr, int *sms) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES)
        return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            return e;
        int count = 0;
        e = cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess)
            return e;
        g_noalloc_sms[dev] = count;
        g_noalloc_ptr[dev] = static_cast<unsigned char *>(p);
    }
    *ptr = g_noalloc_ptr[dev];
    *sms = g_noalloc_sms[dev];
    return cudaSuccess;
}

}  // namespace

cudaError_t launch_bibd_check_noalloc(uint32_t n, uint32_t v, uint32_t b, uint32_t flags, const uint64_t *d_rows,
                                      const uint8_t *d_nrows, Outputs out, uint64_t max_trials, cudaStream_t s) {
    if (n > NOALLOC_MAX_ITEMS)
        return cudaErrorInvalidValue;
    if (!n)
        return cudaSuccess;
    unsigned char *scratch = nullptr;
    int sms = 0;
    cudaError_t e = noalloc_scratch(&scratch, &sms);
    if (e != cudaSuccess)
        return e;
    Item *items = reinterpret_cast<Item *>(scratch);
    unsigned *counter = reinterpret_cast<unsigned *>(scratch + NOALLOC_COUNTER_OFF);
    int grid = (int)((n + 255) / 256);
    if (grid > 4 * sms)
        grid = 4 * sms;
    noalloc_fill_items<<<grid, 256, 0, s>>>(items, n, v, b, flags, d_nrows);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    // the work counters are cleared by the launchers before the check runs; the
    // route is the one canon_sync takes for the same flags
    const bool two_pass = (flags & (F_AUT_CANON | F_FULL_AUT)) && !(flags & (F_SAVE_AUTS | F_REFERENCE_ORDER));
    if (two_pass)
        return launch_bibd_check_two_pass(items, n, d_rows, out, max_trials, counter, sms, s, b, v);
    return launch_bibd_check(items, n, d_rows, out, max_trials, counter, sms, s);
}

}  // namespace canon
