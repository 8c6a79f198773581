// canon_bibd_conv.cuh -- the lex-max search of canon_bibd_core.cuh (max_search()) laid
// out so that the threads of a warp stay converged.
//
// Each thread owns one matrix, as in bibd_max_kernel, but the search is a state
// machine whose steps are of two kinds:
//   control -- choosing the next child, backtracking, leaves, automorphism orbits,
//              finishing a matrix and taking the next: short, divergent code;
//   node    -- arranging the columns for the chosen child and evaluating the new
//              node: one pass over all b columns of the matrix with the same trip
//              count in every thread, whatever the thread's level and orbits.
// Every iteration of the kernel's loop runs the control steps until each thread has
// one node to evaluate, then all threads evaluate their node together.  In
// max_search() the loops over orbits and over the columns of an orbit have
// data-dependent lengths, so the 32 threads of a warp rarely run the same
// instruction (5.5 of 32 lanes active on STS(15)); here the heavy part runs with
// every active lane.
//
// Until restart_after nodes (see ConvState), the search tree and node count are those
// of max_search() with automorphism pruning (prune = true, stop_on_improve = false, all
// first rows); the verdict and |Aut| always are:
//   - node evaluation: the greatest arranged row over the unused rows, orbit by
//     orbit, bit-sliced over the rows (the comparison of checkColOrbit(),
//     Source/CanonicityChecker.cpp:191-223), compared with the bound as it is built;
//   - column arrangement: inside every orbit of the parent's level the columns with
//     a 1 in the chosen row go first (a one-pass partition; only the set of columns
//     of an orbit matters to later levels, not their order inside it);
//   - the last level's arrangement is skipped: a leaf is never evaluated.
#pragma once
#include "canon_bibd_core.cuh"

namespace canon {
namespace bibd {
namespace {

// the greatest arranged row over `tied` at level lv, compared with `bound`:
// 0 equal, 1 greater, 2 smaller (have_bound false: never compared, 0).
// b: the matrix's columns; bt >= b: the columns every lane of the launch walks (the
// widest matrix of a mixed launch).  Columns b..bt-1 hold no 1 (CM_() is 0 there)
// and each closes an orbit of its own, so they change neither the row nor the
// comparison.
// FB > 0: b == bt == FB, known at compile time (the loop is unrolled, every column's
// shared-memory address and end test are constants).  The orbit ends stay a branch:
// taking the greatest count at every column without one measured 1.45x slower.
// The row is compared with the bound once it is complete: placed 1s-first inside
// every orbit, the first orbit whose counts differ decides, which is the first
// position where the two rows differ (a per-orbit comparison inside the loop
// measured 1.13x slower).
// NP: bit planes of the count (3, 4 or 6).  A row's count inside one orbit is at most
// its weight, so NP = 3 is exact when no row of the matrix has more than 7 ones (STS(15):
// 7) and NP = 4 up to 15 (BIBD(16,24,9,6,3): 9); fewer planes shorten the carry chain
// of every column and the plane tests of every orbit end.
template <unsigned FB = 0, unsigned NP = 6, typename S>
__device__ __forceinline__ int eval_node_uniform(S sm, unsigned lv, unsigned b, unsigned bt, unsigned &tied,
                                                 uint64_t &arr, bool have_bound, uint64_t bound) {
    static_assert(NP == 3 || NP == 4 || NP == 6, "3, 4 or 6 count planes");
    if (FB) {
        b = FB;
        bt = FB;
    }
    const uint64_t lvl = L_(lv);
    // bit p: column p closes an orbit (the next column starts one, or p is the last)
    const uint64_t ends = (lvl >> 1) | (~0ull << (b - 1));
    unsigned t0 = tied;
    uint64_t a = 0;
    unsigned pl[NP];
#pragma unroll
    for (unsigned k = 0; k < NP; ++k)
        pl[k] = 0;
    unsigned s = 0;
#pragma unroll(FB ? FB : 1)
    for (unsigned p = 0; p < bt; ++p) {
        unsigned carry = (unsigned)CM_(p) & t0, t;
#pragma unroll
        for (unsigned k = 0; k + 1 < NP; ++k) {
            t = pl[k] & carry;
            pl[k] ^= carry;
            carry = t;
        }
        pl[NP - 1] ^= carry;
        if ((ends >> p) & 1u) {
            unsigned cstar = 0;
#pragma unroll
            for (int k = (int)NP - 1; k >= 0; --k) {
                t = t0 & pl[k];
                if (t) {
                    t0 = t;
                    cstar |= 1u << k;
                }
            }
            a |= ((1ull << cstar) - 1ull) << s;
#pragma unroll
            for (unsigned k = 0; k < NP; ++k)
                pl[k] = 0;
            s = p + 1;
        }
    }
    int state = 0;
    if (have_bound) {
        const uint64_t ka = __brevll(a), kb = __brevll(bound);
        state = ka > kb ? 1 : (ka < kb ? 2 : 0);
    }
    tied = t0;
    arr = a;
    return state;
}

// the greatest row weight of the n rows in R_() (sets the count planes of a node step)
template <typename S>
__device__ __forceinline__ unsigned conv_row_weight(S sm, unsigned n) {
    unsigned w = 0;
    for (unsigned r = 0; r < n; ++r) {
        const unsigned c = (unsigned)__popcll(R_(r));
        w = c > w ? c : w;
    }
    return w;
}

// the node evaluation with the fewest count planes that hold weight w
template <unsigned FB = 0, typename S>
__device__ __forceinline__ int eval_node_planes(S sm, unsigned w, unsigned lv, unsigned b, unsigned bt,
                                                unsigned &tied, uint64_t &arr, bool have_bound, uint64_t bound) {
    if (w <= 7)
        return eval_node_uniform<FB, 3>(sm, lv, b, bt, tied, arr, have_bound, bound);
    if (w <= 15)
        return eval_node_uniform<FB, 4>(sm, lv, b, bt, tied, arr, have_bound, bound);
    return eval_node_uniform<FB, 6>(sm, lv, b, bt, tied, arr, have_bound, bound);
}

// the columns of level lv+1 after row x was taken at level lv: inside every orbit of
// level lv, the columns with a 1 in row x first (one pass, a write pointer per orbit);
// bt: the columns walked (columns past the matrix's own hold no 1 and never move)
// With FB > 0 the column masks are loaded RD columns ahead of their turn (RD, the
// shared-memory staging depth, is a dimension of the autotuner: 2, 4 or 8): a swap at
// column p writes only positions w <= p, never a column still to come, so the early
// loads read what the in-order pass would, and their latency overlaps the swaps instead
// of following each one (the compiler cannot see that w <= p and would keep every load
// behind the stores before it).
template <unsigned FB = 0, unsigned RD = 4, typename S>
__device__ __forceinline__ void refine_uniform(S sm, unsigned lv, unsigned x, unsigned bt) {
    const uint64_t starts = L_(lv);
    unsigned w = 0;
    if constexpr (FB > 0) {
        static_assert(FB >= RD, "the look-ahead fits the columns");
        uint16_t ahead[RD];
#pragma unroll
        for (unsigned q = 0; q < RD; ++q)
            ahead[q] = CM_(q);
#pragma unroll
        for (unsigned p = 0; p < FB; ++p) {
            if ((starts >> p) & 1u)
                w = p;
            const uint16_t c = ahead[p % RD];
            if (p + RD < FB)
                ahead[p % RD] = CM_(p + RD);
            if ((c >> x) & 1u) {
                CM_(p) = CM_(w);
                CM_(w) = c;
                ++w;
            }
        }
    } else {
        for (unsigned p = 0; p < bt; ++p) {
            if ((starts >> p) & 1u)
                w = p;
            const uint16_t c = CM_(p);
            if ((c >> x) & 1u) {
                CM_(p) = CM_(w);
                CM_(w) = c;
                ++w;
            }
        }
    }
}

// the per-thread state of one lex-max search (max_search()'s locals, and the restart)
//
// Restart.  Climbing, the search raises its bound to the canonical form C and then,
// with the automorphism pruning off (the pruning holds for M's own automorphisms),
// counts every labelling of C: a relabelled matrix whose C has a large group costs
// 41K nodes (|Aut| 192) or 152K (|Aut| 20,160) against 6.2K on average.  So once
// restart_after nodes are spent and the bound is a complete matrix (valid == n), the
// search starts again on the bound: its rows become the matrix searched, the pruning
// is on again, and the first matrix is remembered as rejected.  If the bound was C,
// the new search is the pruned check of C (|Aut| from its orbit product); if not, it
// climbs on and restarts again.  The verdict and |Aut| are those of the climb
// (|Aut(M)| = |Aut(C)|); typical matrices finish before restart_after.
struct ConvState {
    uint64_t perm, orb, order, leaves, nodes, order0, restart_after;
    unsigned n, valid, used, id_top, i, allrows, b;
    uint64_t nmask1;
    bool improved, timeout, rejected;
    bool verdict_only;      // stop at the first greater node (M rejected; no |Aut|)
    unsigned w;             // the greatest row weight (conv_row_weight): the count planes
};

// a fresh search of the n rows in R_(); restart_after, b and verdict_only are the caller's
__device__ __forceinline__ void conv_start(ConvState &st, unsigned n, uint64_t order0) {
    st.rejected = false;
    st.n = n;
    st.allrows = (n >= 16) ? 0xFFFFu : ((1u << n) - 1u);
    st.nmask1 = (n >= 16) ? NIB1 : (NIB1 & ((1ull << (4 * n)) - 1ull));
    st.valid = n;
    st.used = 0;
    st.perm = 0;
    st.orb = ID16;
    st.order = 1;
    st.id_top = 0;
    st.i = 0;
    st.leaves = 0;
    st.nodes = 0;
    st.order0 = order0;
    st.improved = false;
    st.timeout = false;
}

// Control steps from "choose the next child of the node at level st.i" until a node
// is due for evaluation (returns true with ref_lv / ref_x set: ref_lv < 0 for none)
// or the search is over (returns false).
template <typename S>
__device__ __forceinline__ bool conv_next(S sm, ConvState &st, int &ref_lv, unsigned &ref_x) {
    const unsigned n = st.n;
    if (st.improved && st.valid == n && st.nodes > st.restart_after) {
        // the bound is a complete matrix C > the searched one: search C from its root
        build_levels(sm, n, st.b);
        const uint64_t nodes = st.nodes;
        conv_start(st, n, ID16);
        st.nodes = nodes;
        st.rejected = true;
        ref_lv = -1;
        return true;
    }
    for (;;) {
        const bool pr = !st.improved;
        unsigned i = st.i;
        unsigned rem = VD_(i);
        if (pr && st.id_top >= i) {
            // at an identity node only orbit leaders are branched on
            while (rem && pg(st.orb, __ffs(rem) - 1) != (unsigned)(__ffs(rem) - 1))
                rem &= rem - 1;
        }
        if (!rem) {
            if (pr && st.id_top >= i) {
                unsigned len = 0;
                for (unsigned q = i; q < n; ++q)
                    len += pg(st.orb, q) == i;
                st.order *= len;
            }
            if (i == 0)
                return false;
            --i;
            st.used &= ~(1u << pg(st.perm, i));
            if (st.id_top > i)
                st.id_top = i;
            st.i = i;
            continue;
        }
        unsigned x = __ffs(rem) - 1;
        if (i == 0 && st.order0 != ID16 && !(pr && (rem & 1u))) {
            for (unsigned q = 0; q < n; ++q) {
                const unsigned c = pg(st.order0, q);
                if ((rem >> c) & 1u) {
                    x = c;
                    break;
                }
            }
        }
        VD_(i) = (uint16_t)(rem & ~(1u << x));
        st.perm = ps(st.perm, i, x);
        st.used |= 1u << x;
        if (st.id_top == i && x == i)
            st.id_top = i + 1;
        if (i + 1 < n) {
            ref_lv = (int)i;
            ref_x = x;
            st.i = i + 1;
            return true;
        }
        // a leaf
        if (pr && st.id_top < n) {
            // an automorphism moving row id_top: merge its orbits and go back to the
            // identity node it branched from
            st.orb = merge_orbits(st.perm, st.orb, n, st.id_top, st.nmask1);
            st.i = st.id_top;
            st.used = (1u << st.i) - 1u;
            continue;
        }
        ++st.leaves;
        st.used &= ~(1u << pg(st.perm, i));
        if (st.id_top > i)
            st.id_top = i;
        st.i = i;
    }
}

// After the node at level st.i was evaluated: prune, or raise the bound and keep
// the children.  Returns false when the search is over (only at the root).
template <typename S>
__device__ __forceinline__ bool conv_after_eval(S sm, ConvState &st, int state, unsigned tied, uint64_t arr,
                                                unsigned b) {
    const unsigned i = st.i;
    if (state == 2) {
        // smaller than the bound: every extension is smaller too
        if (i == 0)
            return false;
        st.i = i - 1;
        st.used &= ~(1u << pg(st.perm, i - 1));
        if (st.id_top > i - 1)
            st.id_top = i - 1;
        return true;
    }
    if (state == 1 || i >= st.valid) {
        if (state == 1) {
            st.improved = true;
            st.leaves = 0;
            if (st.verdict_only)
                return false;
        }
        const uint64_t cols = (1ull << b) - 1ull;
        R_(i) = arr;
        L_(i + 1) = L_(i) | ((arr ^ (arr << 1)) & cols & ~1ull);
        st.valid = i + 1;
    }
    VD_(i) = (uint16_t)tied;
    return true;
}

// |Aut| (the number of labelings reaching the canonical form) once the search is over
__device__ __forceinline__ uint64_t conv_leaves(const ConvState &st) { return st.improved ? st.leaves : st.order; }

// M is not canonical (a greater matrix was found in this search or one before it)
__device__ __forceinline__ bool conv_rejected(const ConvState &st) { return st.improved || st.rejected; }

}  // namespace
}  // namespace bibd
}  // namespace canon
