// canon_bibd_core.cuh -- device search of the rank-2 incidence-matrix checker.
//
// Included by canon_bibd.cu; written in plain CUDA C++ so that the same
// functions can also be compiled for the host.
#pragma once
#include "canon_internal.h"
#include "canon_nibble.cuh"

namespace canon {
namespace bibd {
// internal linkage: the header is compiled into more than one translation unit
namespace {

constexpr int TPB = 64;                  // threads per block (one matrix each)
constexpr uint64_t ID16 = 0xFEDCBA9876543210ull;
constexpr uint64_t NIB1 = 0x1111111111111111ull;

__device__ __forceinline__ unsigned pg(uint64_t p, unsigned i) {
    return (unsigned)(p >> ((i & 15u) << 2)) & 15u;
}
__device__ __forceinline__ uint64_t ps(uint64_t p, unsigned i, unsigned x) {
    const unsigned sh = (i & 15u) << 2;
    return (p & ~(15ull << sh)) | ((uint64_t)(x & 15u) << sh);
}

// revert(), GroupOrder.h:25-28: reverse positions i+1 .. j-1
__device__ __forceinline__ uint64_t revert(uint64_t p, unsigned j, unsigned i) {
    while (++i < --j) {
        const unsigned a = pg(p, i), c = pg(p, j);
        p = ps(p, i, c);
        p = ps(p, j, a);
    }
    return p;
}

struct Group {
    uint64_t perm, orb;     // nibble-packed permRow() and row orbits
    unsigned stab;          // stabilizerLength()
    unsigned stab_aut;      // stabilizerLengthAut()
    uint64_t ord_lo, ord_hi;
};

__device__ __forceinline__ void mul_order(uint64_t &lo, uint64_t &hi, uint64_t m) {
    const uint64_t nlo = lo * m;
    hi = hi * m + __umul64hi(lo, m);
    lo = nlo;
}

// orbit length of stabilizerLengthAut(), updateGroupOrder() GroupOrder.h:63-73
__device__ __forceinline__ unsigned orbit_len(const Group &g, unsigned n) {
    unsigned len = 1;
    unsigned idx = g.stab_aut & 0xFFFFu;
    while (++idx < n)
        if (pg(g.orb, idx) == g.stab_aut)
            len++;
    return len;
}

// next_permutation(), GroupOrder.h:136-248 (the recursive call becomes a second pass)
__device__ unsigned next_perm(Group &g, unsigned n, unsigned idx, unsigned lenStab) {
    for (int pass = 0; pass < 2; ++pass) {
        uint64_t perm = g.perm;
        const uint64_t orb = g.orb;
        unsigned temp, i, j;
        if (idx == IMAX && pg(perm, g.stab) == n - 1)
            idx = EMAX;
        if (idx == IMAX) {
            i = g.stab;
            idx = i;
            temp = pg(perm, i);
            for (j = n; --j > temp;)
                perm = ps(perm, j, j);
            unsigned k = j++;
            while (k-- > i)
                perm = ps(perm, k + 1, k);
        } else if (idx >= IMAX) {
            j = i = n;
            while (--i > 0 && pg(perm, i - 1) >= pg(perm, i))
                ;
            if (i == lenStab) {
                g.perm = perm;
                return EMAX;
            }
            temp = pg(perm, --i);
            while (pg(perm, --j) <= temp)
                ;
        } else {
            i = j = idx;
            temp = pg(perm, i);
            while (++j < n && pg(perm, j) <= temp)
                ;
            if (j >= n) {
                g.perm = revert(perm, n, i);
                idx = EMAX;
                lenStab = 0;
                continue;
            }
        }

        if (g.stab == i) {
            bool flag = false;
            unsigned k = j, tmp = pg(perm, j);
            if (idx >= IMAX) {
                while (k > i && pg(orb, pg(perm, k)) != pg(perm, k))
                    k--;
                if (k != j) {
                    if (!k) {
                        g.perm = perm;
                        return EMAX;
                    }
                    flag = (k == i);
                    tmp = pg(perm, k--);
                    while (++k < j)
                        perm = ps(perm, k, pg(perm, k + 1));
                }
            } else {
                while (k < n && pg(orb, pg(perm, k)) != pg(perm, k))
                    k++;
                if (k != j) {
                    flag = (k == n);
                    if (flag) {
                        if (!i) {
                            g.perm = perm;
                            return EMAX;
                        }
                        k = (idx - 1) & 0xFFu;           // uint8 arithmetic of the reference
                        while ((k = (k + 1) & 0xFFu) < j)
                            perm = ps(perm, k, k);
                    } else {
                        tmp = pg(perm, k++);
                        while (--k > j)
                            perm = ps(perm, k, pg(perm, k - 1));
                    }
                }
            }
            perm = ps(perm, j, tmp);
            if (flag) {
                j = idx >= IMAX ? n - 1 : i;
                temp = pg(perm, --i);
                g.stab = i;
            }
        }

        perm = ps(perm, i, pg(perm, j));
        perm = ps(perm, j, temp);
        if (idx >= IMAX) {
            if (g.stab > i)
                g.stab = i;
            perm = revert(perm, n, i);
        }
        g.perm = perm;
        return i;
    }
    return EMAX;  // not reached
}

// Update_Orbits(), GroupOrder.h:30-49, on nibble-packed orbits (SWAR replace)
__device__ __forceinline__ uint64_t merge_orbits(uint64_t perm, uint64_t orb, unsigned n, unsigned idx,
                                                 uint64_t nmask1) {
    do {
        unsigned a = pg(orb, idx);
        unsigned c = pg(orb, pg(perm, idx));
        if (a == c)
            continue;
        if (c < a) {
            const unsigned t = a;
            a = c;
            c = t;
        }
        const uint64_t t = orb ^ (NIB1 * c);
        uint64_t y = t | (t >> 1);
        y |= y >> 2;
        const uint64_t z = ~y & nmask1;          // nibble LSB set where the nibble equals c
        const uint64_t m = z * 15u;
        orb = (orb & ~m) | ((NIB1 * a) & m);
    } while (++idx < n);
    return orb;
}

template <typename VD>
struct SmemT {
    uint64_t *rows;  // rows[r * TPB]: row r as a bit set of columns
    uint64_t *lvl;   // lvl[r * TPB]: orbit-start masks of level r (also scratch)
    uint8_t *pc;     // pc[j * TPB]: permColumn
    uint16_t *cm;    // cm[c * TPB]: column c as a bit set of rows
    VD *vd;          // vd[r * TPB]: search(): verdicts at level r, bits 0-15 "greater"
                     // (reject), 16-31 "equal"; max_search(): the rows still to visit
};
// the reference-order search needs 32-bit verdict words; the lex-max search alone
// (its own kernels) keeps 16-bit row sets, 32 B less shared memory per thread
using Smem = SmemT<uint32_t>;
using SmemMax = SmemT<uint16_t>;

#define R_(r) sm.rows[(r) * TPB]
#define L_(r) sm.lvl[(r) * TPB]
#define PC_(j) sm.pc[(j) * TPB]
#define CM_(c) sm.cm[(c) * TPB]
#define VD_(r) sm.vd[(r) * TPB]

struct CheckOut {
    uint8_t canonical, status, reject_row, rtc;
    uint64_t witness;
    uint64_t aut_lo, aut_hi;
    uint64_t trials;
    uint16_t n_auts;
    uint8_t len_aut;
};

// Brings the columns into orbit normal form: sorted in decreasing order of their
// pattern read from row 0 down.  Equal in content to GenerateBinaryColumnOrbits()
// applied to rows 0..n-1 (MatrixCanonChecker.cpp:186-263), which swaps the first 0
// and the last 1 inside every orbit until each row is 1s-first.
template <typename S>
__device__ void normalize_columns(S sm, unsigned n, unsigned b) {
    // codes (16 bit) are kept four to a word in the lvl scratch area
    for (unsigned c = 0; c < b; ++c) {
        unsigned code = 0;
        for (unsigned r = 0; r < n; ++r)
            code = (code << 1) | (unsigned)((R_(r) >> c) & 1u);
        const unsigned w = c >> 2, sh = (c & 3u) * 16u;
        uint64_t cur = (c & 3u) ? L_(w) : 0ull;
        cur = (cur & ~(0xFFFFull << sh)) | ((uint64_t)code << sh);
        L_(w) = cur;
    }
    uint64_t acc[VMAX];
#pragma unroll
    for (unsigned r = 0; r < VMAX; ++r)
        acc[r] = 0;
    for (unsigned c = 0; c < b; ++c) {
        const unsigned kc = (unsigned)(L_(c >> 2) >> ((c & 3u) * 16u)) & 0xFFFFu;
        unsigned rank = 0;
        for (unsigned c2 = 0; c2 < b; ++c2) {
            const unsigned k2 = (unsigned)(L_(c2 >> 2) >> ((c2 & 3u) * 16u)) & 0xFFFFu;
            rank += (k2 > kc) || (k2 == kc && c2 < c);
        }
#pragma unroll
        for (unsigned r = 0; r < VMAX; ++r)
            if (r < n)
                acc[r] |= (uint64_t)((kc >> (n - 1 - r)) & 1u) << rank;
    }
#pragma unroll
    for (unsigned r = 0; r < VMAX; ++r)
        if (r < n)
            R_(r) = acc[r];
}

// Orbit-start masks of every level and the column-major copy of the matrix;
// returns false if a row is not 1s-first inside the orbits of the rows above it.
template <typename S>
__device__ bool build_levels(S sm, unsigned n, unsigned b) {
    const uint64_t cols = (1ull << b) - 1ull;
    uint64_t m = 1ull;
    bool ok = true;
    for (unsigned r = 0; r < n; ++r) {
        L_(r) = m;
        const uint64_t x = R_(r);
        if (x & ~cols)
            ok = false;
        if (x & ~(x << 1) & ~m & cols & ~1ull)
            ok = false;
        m |= (x ^ (x << 1)) & cols & ~1ull;
    }
    L_(n) = m;
    for (unsigned c = 0; c < b; ++c) {
        unsigned col = 0;
        for (unsigned r = 0; r < n; ++r)
            col |= (unsigned)((R_(r) >> c) & 1u) << r;
        CM_(c) = (uint16_t)col;
    }
    return ok;
}

// Verdicts of every row as the candidate for position `lv` (the comparison of
// row lv of the matrix with the candidate row under the current column
// arrangement, checkColOrbit() CanonicityChecker.cpp:191-223 and :349-365),
// evaluated for all rows at once: each orbit of level lv is one bit-parallel
// step over the row masks of its image columns.
__device__ void level_verdicts(Smem sm, unsigned lv, unsigned b, unsigned allrows) {
    const uint64_t x = R_(lv);
    const uint64_t m = L_(lv) | (1ull << b);
    unsigned undec = allrows, rej = 0;
    unsigned s = 0;
    while (s < b && undec) {
        const unsigned e = __ffsll((long long)(m & (~0ull << (s + 1)))) - 1;
        if (e == s + 1) {
            const unsigned ones = CM_(PC_(s));
            if ((x >> s) & 1u) {
                undec &= ones;                 // a 0 against the matrix's 1: smaller, pruned
            } else {
                rej |= undec & ones;           // a 1 against 0: the permuted matrix is greater
                undec &= ~ones;
            }
        } else {
            const unsigned len = e - s;
            const unsigned c = __popcll(x & (((1ull << len) - 1ull) << s));
            // bit-sliced per-row counts of 1s among the image columns of the orbit
            unsigned p0 = 0, p1 = 0, p2 = 0, p3 = 0, p4 = 0, p5 = 0;
            for (unsigned j = s; j < e; ++j) {
                unsigned carry = CM_(PC_(j)), t;
                t = p0 & carry; p0 ^= carry; carry = t;
                t = p1 & carry; p1 ^= carry; carry = t;
                t = p2 & carry; p2 ^= carry; carry = t;
                t = p3 & carry; p3 ^= carry; carry = t;
                t = p4 & carry; p4 ^= carry; carry = t;
                p5 ^= carry;
            }
            const unsigned pl[6] = {p0, p1, p2, p3, p4, p5};
            unsigned gt = 0, eq = 0xFFFFFFFFu;
#pragma unroll
            for (int k = 5; k >= 0; --k) {
                if ((c >> k) & 1u) {
                    eq &= pl[k];
                } else {
                    gt |= eq & pl[k];
                    eq &= ~pl[k];
                }
            }
            rej |= undec & gt;
            undec &= eq;
        }
        s = e;
    }
    VD_(lv) = (rej & 0xFFFFu) | ((undec & 0xFFFFu) << 16);
}

// The column arrangement for level lv+1 after row `cand` compared equal at level
// lv: inside every orbit of level lv that row lv splits, the image columns holding
// a 1 in row `cand` move to the front (the reordering of checkColOrbit()).
__device__ void refine(Smem sm, unsigned lv, unsigned cand, unsigned b) {
    const uint64_t x = R_(lv);
    const uint64_t m = L_(lv) | (1ull << b);
    uint64_t split = L_(lv + 1) & ~L_(lv);   // starts of the second parts
    while (split) {
        const unsigned t = __ffsll((long long)split) - 1;
        split &= split - 1;
        // the orbit [s, e) of level lv containing t
        const uint64_t below = L_(lv) & ((1ull << t) - 1ull);
        const unsigned s = 63 - __clzll((long long)below);
        const unsigned e = __ffsll((long long)(m & (~0ull << (s + 1)))) - 1;
        (void)x;
        unsigned lo = s, hi = e - 1;
        while (lo < hi) {
            while (lo < hi && ((CM_(PC_(lo)) >> cand) & 1u))
                ++lo;
            while (lo < hi && !((CM_(PC_(hi)) >> cand) & 1u))
                --hi;
            if (lo < hi) {
                const uint8_t tmp = PC_(lo);
                PC_(lo) = PC_(hi);
                PC_(hi) = tmp;
            }
        }
    }
}

// the set of entries at positions 0..i of a nibble-packed permutation
__device__ __forceinline__ unsigned prefix_set(uint64_t perm, unsigned i) {
    unsigned m = 0;
    for (unsigned p = 0; p <= i; ++p)
        m |= 1u << nib_get(perm, p);
    return m;
}

// positions i+1.. of perm := the elements of `set` in increasing order
__device__ __forceinline__ uint64_t write_suffix(uint64_t perm, unsigned i, unsigned set) {
    unsigned p = i + 1;
    while (set) {
        const unsigned t = __ffs(set) - 1;
        set &= set - 1;
        perm = ps(perm, p++, t);
    }
    return perm;
}

// TestCanonicity() for one matrix whose rows are in shared memory: the
// reference's search order (next_permutation() over row permutations with the
// orbit pruning of the automorphisms found so far), with every comparison of
// a candidate row taken from the verdict masks of its level.  A run of
// candidates that compare "smaller" at one position (each of which the
// reference tries and prunes in turn) is passed over in one step; the trial
// count still counts each of them.
__device__ void search(Smem sm, unsigned n, unsigned b, unsigned flags, uint64_t max_trials, uint8_t *aut_dst,
                       unsigned aut_cap, CheckOut &o) {
    const bool row_permut = flags & F_COMPLETE;
    const bool full = flags & F_FULL_AUT;
    const bool save = (flags & F_SAVE_AUTS) && aut_dst;
    const uint64_t nmask1 = (n >= 16) ? NIB1 : (NIB1 & ((1ull << (4 * n)) - 1ull));
    const unsigned allrows = (n >= 16) ? 0xFFFFu : ((1u << n) - 1u);
    const uint64_t lastLvl = L_(n);
    const uint64_t colsMask = (1ull << b) - 1ull;

    for (unsigned j = 0; j < b; ++j)
        PC_(j) = (uint8_t)j;
    // verdicts along the trivial permutation (every prefix of it compares equal)
    for (unsigned lv = 0; lv < n; ++lv) {
        level_verdicts(sm, lv, b, allrows);
        if (lv + 1 < n)
            refine(sm, lv, lv, b);
    }

    // init(), CanonicityChecker.cpp:35-84
    Group g;
    g.perm = ID16;
    g.orb = ID16;
    g.stab = n - 1;
    g.stab_aut = EMAX;
    g.ord_lo = 1;
    g.ord_hi = 0;
    uint64_t part_lo = 1, part_hi = 0;   // |Aut| of a partial matrix (addition)
    unsigned n_auts = 0;
    o.n_auts = 0;
    o.len_aut = 0;
    if (row_permut) {
        n_auts = 1;                      // the trivial row permutation is saved by init()
        o.len_aut = (uint8_t)n;
        if (save && aut_cap)
            for (unsigned i = 0; i < n; ++i)
                aut_dst[i] = (uint8_t)i;
    }
    bool rejected = false, overflow = false;
    uint64_t trials = 0;

    unsigned i = next_perm(g, n, EMAX, 0);
    while (i != EMAX) {
        if (++trials > max_trials) {
            o.status |= ST_TIMEOUT;
            break;
        }
        bool descended_to_end = false;
        for (;;) {
            const unsigned x = pg(g.perm, i);
            const unsigned vd = VD_(i);
            const bool is_rej = (vd >> x) & 1u;
            const bool is_eq = (vd >> (16 + x)) & 1u;
            if (is_rej && !rejected) {
                rejected = true;
                o.canonical = 0;
                o.reject_row = (uint8_t)i;
                o.witness = g.perm;
                unsigned rtc = i;                        // rowToChange(), CanonicityChecker.cpp:320-330
                for (unsigned q = 0; q <= i; ++q)
                    if (rtc < pg(g.perm, q))
                        rtc = pg(g.perm, q);
                o.rtc = (uint8_t)rtc;
                if (!full)
                    break;
            }
            if (is_eq) {
                refine(sm, i, x, b);
                if (i + 1 == n) {
                    descended_to_end = true;
                    break;
                }
                ++i;
                level_verdicts(sm, i, b, allrows);
                continue;
            }
            // pruned at position i ("smaller", or "greater" once counting |Aut| only)
            if (g.stab != i) {
                const unsigned used = prefix_set(g.perm, i);
                const unsigned rest = allrows & ~used;
                const unsigned larger = rest & ~((2u << x) - 1u);
                const unsigned good = larger & ((vd >> 16) | (full ? 0u : vd));
                if (good) {
                    const unsigned y = __ffs(good) - 1;
                    const unsigned skipped = __popc(larger & ((1u << y) - 1u));
                    trials += skipped + 1;
                    if (trials > max_trials) {
                        o.status |= ST_TIMEOUT;
                        i = EMAX;
                        break;
                    }
                    g.perm = ps(g.perm, i, y);
                    g.perm = write_suffix(g.perm, i, (rest & ~(1u << y)) | (1u << x));
                    continue;
                }
                trials += __popc(larger);
                if (larger) {
                    const unsigned mx = 31 - __clz(larger);
                    g.perm = ps(g.perm, i, mx);
                    g.perm = write_suffix(g.perm, i, (rest & ~(1u << mx)) | (1u << x));
                }
            }
            i = next_perm(g, n, i, 0);
            break;
        }
        if (rejected && !full)
            break;
        if (!descended_to_end)
            continue;

        // automorphism found, CanonicityChecker.h:421-476
        const uint64_t moved = g.perm ^ ID16;
        const unsigned first = moved ? (unsigned)(__ffsll((long long)moved) - 1) >> 2 : n;
        if (!row_permut) {
            if (save) {
                // permutation of the column orbits of the last level (:430-450)
                const unsigned len = __popcll(lastLvl & colsMask);
                o.len_aut = (uint8_t)len;
                if (n_auts == 0) {
                    if (aut_cap)
                        for (unsigned q = 0; q < len; ++q)
                            aut_dst[q] = (uint8_t)q;
                    n_auts = 1;
                }
                if (n_auts < aut_cap) {
                    uint8_t *dst = aut_dst + n_auts * 64u;
                    uint64_t starts = lastLvl & colsMask;
                    unsigned q = 0;
                    while (starts) {
                        const unsigned s0 = __ffsll((long long)starts) - 1;
                        starts &= starts - 1;
                        const unsigned col = PC_(s0);
                        dst[q++] = (uint8_t)(__popcll(lastLvl & ((2ull << col) - 1ull)) - 1);
                    }
                } else {
                    overflow = true;
                }
                ++n_auts;
            }
            if (g.stab_aut > first)
                mul_order(part_lo, part_hi, orbit_len(g, n));
        }
        // addAutomorphism() -> udpdateStabLength() + Update_Orbits()
        if (row_permut && g.stab_aut > first)
            mul_order(g.ord_lo, g.ord_hi, orbit_len(g, n));
        g.stab_aut = first;
        g.stab = first;
        g.orb = merge_orbits(g.perm, g.orb, n, first, nmask1);
        if (row_permut && save) {
            if (n_auts < aut_cap) {
                uint8_t *dst = aut_dst + n_auts * 64u;
                for (unsigned q = 0; q < n; ++q)
                    dst[q] = (uint8_t)pg(g.perm, q);
            } else {
                overflow = true;
            }
            ++n_auts;
        }
        i = next_perm(g, n, IMAX, 0);
    }

    if (row_permut) {
        mul_order(g.ord_lo, g.ord_hi, orbit_len(g, n));
        o.aut_lo = g.ord_lo;
        o.aut_hi = g.ord_hi;
    } else {
        mul_order(part_lo, part_hi, orbit_len(g, n));
        o.aut_lo = part_lo;
        o.aut_hi = part_hi;
    }
    if (rejected && !full) {
        o.aut_lo = 0;                    // the reference leaves |Aut| undefined here
        o.aut_hi = 0;
    }
    if (overflow)
        o.status |= ST_PERM_OVF;
    o.trials = trials;
    o.n_auts = (uint16_t)(n_auts > 0xFFFFu ? 0xFFFFu : n_auts);
}

// Lex-max search: the greatest matrix reachable from M by row and column
// permutations (the canonical form that CanonizeMatrix() converges to,
// MatrixCanonChecker.cpp:420-496) and the number of row permutations that reach
// it (|Aut|, the order updateGroupOrder() accumulates, GroupOrder.h:63-73).
// Depth-first over row prefixes; at each level the candidate rows whose best
// column arrangement gives the greatest row are found bit-parallel, orbit by
// orbit (the same comparison as checkColOrbit()), and only they are branched on.
// The rows of M serve as the first bound; a greater row replaces the bound from
// that level down (the subtrees already searched are all smaller than it), so M
// is canonical iff the bound never rises.  On return R_() holds the canonical
// form.
//
// Automorphism pruning (prune = true), while the bound is still M: the identity
// path is searched first; below it, a subtree is left at its first leaf, which is
// an automorphism fixing the rows above the branch point d and moving row d.  The
// row orbits of all automorphisms found so far are then those of the pointwise
// stabilizer of rows 0..d-1 (every one was found below level d), so at level d
// only orbit leaders are branched on, and |Aut| is the product over d of the
// length of the orbit of d -- the orbit-stabilizer count of Update_Orbits() /
// updateGroupOrder() (GroupOrder.h:30-73), with the leaders tried in increasing
// order as next_permutation() does.  Skipped subtrees are images of searched ones
// under an automorphism of M, so they hold no greater matrix: once the bound
// rises the search goes on unpruned and counts the leaves that reach the new
// bound, exactly as without pruning.
struct MaxOut {
    bool improved;      // M is not canonical
    bool timeout;
    uint64_t leaves;    // |Aut|
    uint64_t nodes;
    unsigned first_rows;  // rows that start a labeling reaching the canonical form
    unsigned orbit0;      // pruned search of a canonical M: the first rows found in the orbit of row 0
    unsigned orbit1;      // ... and the second rows (under row 0) found in the orbit of row 1
    unsigned n_gens;      // automorphisms written to gens_out (pruned search, M canonical so far)
};

// The arranged column masks for level lv+1 after row `cand` was taken at level
// lv: inside every orbit of level lv that the bound's row lv splits, the columns
// holding a 1 in row `cand` move to the front.  CM_() holds the row masks of the
// columns in arranged order (the column masks permuted by permColumn).
template <typename S>
__device__ __forceinline__ void refine_arranged(S sm, unsigned lv, unsigned cand, unsigned b) {
    const uint64_t m = L_(lv) | (1ull << b);
    uint64_t split = L_(lv + 1) & ~L_(lv);
    while (split) {
        const unsigned t = __ffsll((long long)split) - 1;
        split &= split - 1;
        const uint64_t below = L_(lv) & ((1ull << t) - 1ull);
        const unsigned s = 63 - __clzll((long long)below);
        const unsigned e = __ffsll((long long)(m & (~0ull << (s + 1)))) - 1;
        unsigned lo = s, hi = e - 1;
        while (lo < hi) {
            while (lo < hi && ((CM_(lo) >> cand) & 1u))
                ++lo;
            while (lo < hi && !((CM_(hi) >> cand) & 1u))
                --hi;
            if (lo < hi) {
                const uint16_t tmp = CM_(lo);
                CM_(lo) = CM_(hi);
                CM_(hi) = tmp;
            }
        }
    }
}

// order0: the order in which the rows are tried as the first row (nibble-packed;
// ID16 = increasing, the plain order).  Only the search order changes with it;
// with pruning, row 0 (the identity path) still comes first while M may be
// canonical, and the other first rows follow order0.  stop_on_improve: return as soon as M is known not to be
// canonical (leaves, first_rows and R_() are then incomplete).  root_mask: the
// rows that may come first (a search split over several threads by first row).
// With pruning and M canonical, orbit0 counts the rows of root_mask found in the
// orbit of row 0, and the thread whose root_mask holds row 0 alone has
// leaves = the product of the orbit lengths below level 0; split searches then
// combine as |Aut| = (sum of orbit0) x (that product).  root_mask1 restricts the
// second rows the same way; orbit1 counts those found in the orbit of row 1
// under the automorphisms that fix row 0.
// stop: a flag that another thread of a split search raises once it has shown M
// not to be canonical; it is read every 64 nodes and ends this share early.
// gens_out: the automorphisms the pruned search finds while M may still be canonical,
// as row permutations (nibble i = the row at position i), at most gens_cap of them;
// they generate the group whose orbits the pruning uses.
// aut_only: the verdict and |Aut| without the canonical form.  A node greater than M
// marks M not canonical and is pruned like a smaller one, so the bound stays M, the
// automorphism pruning stays on, and the leaves that reach M give |Aut(M)|, which is
// |Aut| of the canonical form (an isomorphism invariant).  A non-canonical matrix with
// a large group then costs what a canonical one does, instead of an unpruned count of
// every labeling of its canonical form.  leaves, first_rows and R_() are then about M.
template <typename S>
__device__ void max_search(S sm, unsigned n, unsigned b, uint64_t max_nodes, MaxOut &o,
                           uint64_t order0 = ID16, bool prune = true, bool stop_on_improve = false,
                           unsigned root_mask = 0xFFFFu, const volatile unsigned *stop = nullptr,
                           unsigned root_mask1 = 0xFFFFu, uint64_t *gens_out = nullptr, unsigned gens_cap = 0,
                           bool aut_only = false) {
    const unsigned allrows = (n >= 16) ? 0xFFFFu : ((1u << n) - 1u);
    const uint64_t cols = (1ull << b) - 1ull;
    const uint64_t sentinel = 1ull << b;
    const uint64_t nmask1 = (n >= 16) ? NIB1 : (NIB1 & ((1ull << (4 * n)) - 1ull));
    o.improved = false;
    o.timeout = false;
    o.leaves = 0;
    o.nodes = 0;
    o.first_rows = 0;
    o.orbit0 = 0;
    o.orbit1 = 0;
    o.n_gens = 0;
    unsigned valid = n;        // rows 0..valid-1 of the bound (and levels 0..valid) are set
    unsigned used = 0;
    uint64_t perm = 0;
    uint64_t orb = ID16;       // row orbits of the automorphisms found (pruned mode)
    uint64_t order = 1;        // product of the orbit lengths of the finished levels
    unsigned id_top = 0;       // perm[0..id_top-1] is the identity
    unsigned i = 0;
    bool enter = true;         // entering the node at level i (else: next child of level i)
    for (;;) {
        const bool pr = prune && (aut_only || !o.improved);
        if (enter) {
            if (i == n) {
                if (pr && id_top < n) {
                    // an automorphism moving row id_top: merge its orbits and go back
                    // to the identity node it branched from
                    if (gens_out && o.n_gens < gens_cap)
                        gens_out[o.n_gens++] = perm;
                    orb = merge_orbits(perm, orb, n, id_top, nmask1);
                    i = id_top;
                    used = (1u << i) - 1u;
                    enter = false;
                    continue;
                }
                ++o.leaves;
                o.first_rows |= 1u << pg(perm, 0);
                enter = false;
                --i;
                used &= ~(1u << pg(perm, i));
                if (id_top > i)
                    id_top = i;
                continue;
            }
            if (++o.nodes > max_nodes) {
                o.timeout = true;
                return;
            }
            if (stop && !(o.nodes & 63u) && *stop)
                return;
            // the greatest arranged row over the unused rows, orbit by orbit, compared
            // with the bound as it is built: 0 equal so far, 1 greater, 2 smaller
            const bool have_bound = i < valid;
            const uint64_t bound = have_bound ? R_(i) : 0ull;
            unsigned tied = allrows & ~used;
            uint64_t arr = 0;
            int state = 0;
            uint64_t st = (L_(i) | sentinel) & ~1ull;
            if (aut_only) {
                // the rows whose best arrangement equals M's row i go on; a row whose best
                // arrangement is greater shows M not canonical (and is not followed)
                unsigned s2 = 0;
                unsigned greater = 0;
                uint64_t st2 = st;
                while (tied) {
                    const unsigned e = __ffsll((long long)st2) - 1;
                    if (e == s2 + 1) {
                        const unsigned col = CM_(s2);
                        if ((bound >> s2) & 1u) {
                            tied &= col;
                        } else {
                            greater |= tied & col;
                            tied &= ~col;
                        }
                    } else {
                        unsigned p0 = 0, p1 = 0, p2 = 0, p3 = 0, p4 = 0, p5 = 0;
                        for (unsigned j = s2; j < e; ++j) {
                            unsigned carry = CM_(j) & tied, t;
                            t = p0 & carry; p0 ^= carry; carry = t;
                            t = p1 & carry; p1 ^= carry; carry = t;
                            t = p2 & carry; p2 ^= carry; carry = t;
                            t = p3 & carry; p3 ^= carry; carry = t;
                            t = p4 & carry; p4 ^= carry; carry = t;
                            p5 ^= carry;
                        }
                        const unsigned pl[6] = {p0, p1, p2, p3, p4, p5};
                        const unsigned cb = __popcll(bound & (((1ull << (e - s2)) - 1ull) << s2));
                        unsigned gt = 0, eq = tied;
#pragma unroll
                        for (int k = 5; k >= 0; --k) {
                            if ((cb >> k) & 1u) {
                                eq &= pl[k];
                            } else {
                                gt |= eq & pl[k];
                                eq &= ~pl[k];
                            }
                        }
                        greater |= gt;
                        tied = eq;
                    }
                    if (e >= b)
                        break;
                    s2 = e;
                    st2 &= st2 - 1;
                }
                if (greater) {
                    o.improved = true;
                    if (stop_on_improve)
                        return;
                }
                if (!tied) {
                    enter = false;
                    if (i == 0)
                        break;
                    --i;
                    used &= ~(1u << pg(perm, i));
                    if (id_top > i)
                        id_top = i;
                    continue;
                }
                VD_(i) = (i == 0) ? (tied & root_mask) : (i == 1 ? (tied & root_mask1) : tied);
                goto next_child;
            }
            unsigned s = 0;
            for (;;) {
                const unsigned e = __ffsll((long long)st) - 1;
                if (e == s + 1) {
                    const unsigned ones = CM_(s) & tied;
                    const unsigned mx = ones ? 1u : 0u;
                    if (ones) {
                        tied = ones;
                        arr |= 1ull << s;
                    }
                    if (state == 0 && have_bound) {
                        const unsigned bb = (unsigned)(bound >> s) & 1u;
                        state = mx > bb ? 1 : (mx < bb ? 2 : 0);
                    }
                } else {
                    unsigned p0 = 0, p1 = 0, p2 = 0, p3 = 0, p4 = 0, p5 = 0;
                    for (unsigned j = s; j < e; ++j) {
                        unsigned carry = CM_(j) & tied, t;
                        t = p0 & carry; p0 ^= carry; carry = t;
                        t = p1 & carry; p1 ^= carry; carry = t;
                        t = p2 & carry; p2 ^= carry; carry = t;
                        t = p3 & carry; p3 ^= carry; carry = t;
                        t = p4 & carry; p4 ^= carry; carry = t;
                        p5 ^= carry;
                    }
                    const unsigned pl[6] = {p0, p1, p2, p3, p4, p5};
                    unsigned cstar = 0;
#pragma unroll
                    for (int k = 5; k >= 0; --k) {
                        const unsigned t = tied & pl[k];
                        if (t) {
                            tied = t;
                            cstar |= 1u << k;
                        }
                    }
                    const uint64_t rng = ((1ull << (e - s)) - 1ull) << s;
                    arr |= ((1ull << cstar) - 1ull) << s;
                    if (state == 0 && have_bound) {
                        const unsigned cb = __popcll(bound & rng);
                        state = cstar > cb ? 1 : (cstar < cb ? 2 : 0);
                    }
                }
                if (state == 2 || e >= b)
                    break;
                s = e;
                st &= st - 1;
            }
            if (state == 2) {
                // smaller than the bound: every extension is smaller too
                enter = false;
                if (i == 0)
                    break;
                --i;
                used &= ~(1u << pg(perm, i));
                if (id_top > i)
                    id_top = i;
                continue;
            }
            if (state == 1 || !have_bound) {
                if (state == 1) {
                    o.improved = true;
                    o.leaves = 0;
                    o.first_rows = 0;
                    if (stop_on_improve)
                        return;
                }
                R_(i) = arr;
                L_(i + 1) = L_(i) | ((arr ^ (arr << 1)) & cols & ~1ull);
                valid = i + 1;
            }
            // children still to visit (16 bits)
            VD_(i) = (i == 0) ? (tied & root_mask) : (i == 1 ? (tied & root_mask1) : tied);
        }
    next_child:
        // next child of the node at level i
        unsigned rem = VD_(i);
        if (pr && id_top >= i) {
            // at an identity node only orbit leaders are branched on
            while (rem && pg(orb, __ffs(rem) - 1) != (unsigned)(__ffs(rem) - 1))
                rem &= rem - 1;
        }
        if (!rem) {
            if (pr && id_top >= i) {
                unsigned len = 0;
                for (unsigned q = i; q < n; ++q)
                    len += pg(orb, q) == i;
                order *= len;
                if (i == 0)
                    for (unsigned q = 0; q < n; ++q)
                        o.orbit0 += ((root_mask >> q) & 1u) && pg(orb, q) == 0;
                if (i == 1)
                    for (unsigned q = 1; q < n; ++q)
                        o.orbit1 += ((root_mask1 >> q) & 1u) && pg(orb, q) == 1;
            }
            if (i == 0)
                break;
            enter = false;
            --i;
            used &= ~(1u << pg(perm, i));
            if (id_top > i)
                id_top = i;
            continue;
        }
        unsigned x = __ffs(rem) - 1;
        if (i == 0 && order0 != ID16 && !(pr && (rem & 1u))) {
            for (unsigned q = 0; q < n; ++q) {
                const unsigned c = pg(order0, q);
                if ((rem >> c) & 1u) {
                    x = c;
                    break;
                }
            }
        }
        VD_(i) = rem & ~(1u << x);
        refine_arranged(sm, i, x, b);
        perm = ps(perm, i, x);
        used |= 1u << x;
        if (id_top == i && x == i)
            id_top = i + 1;
        ++i;
        enter = true;
    }
    if (prune && (aut_only || !o.improved)) {
        o.leaves = order;
        unsigned fr = 0;
        for (unsigned q = 0; q < n; ++q)
            fr |= (pg(orb, q) == 0 ? 1u : 0u) << q;
        o.first_rows = fr;
    }
}

// The lex-max pass of the two-pass check climbs to the canonical form (the bound rises
// with every greater row); a matrix whose canonical form has a large group then counts
// every labeling of it without automorphism pruning (151,636 nodes for a relabelled
// PG(3,2) against 5.8K on average).  After this many nodes the pass starts again with the
// bound kept at M (aut_only), where the pruning stays on; both give the same verdict and
// |Aut|, and keeping M costs more on typical matrices (its tied tree is wider than the
// canonical form's), so it is the fallback rather than the rule.  The cap sits above
// the climbs of the next-largest STS(15) groups (|Aut| 192: about 41K nodes, where
// keeping M takes 5K - 77K depending on the labelling).
constexpr uint64_t CLIMB_CAP = 49152;

// The converged search's restart threshold (canon_bibd_conv.cuh): typical STS(15) climbs
// end within 10K nodes (6.2K on average), the climbs of large groups go on far longer.
constexpr uint64_t RESTART_AFTER = 10000;

// Trials the reference-order search may spend before the lex-max search decides:
// a complete canonical matrix needs far more in the reference order (~52K for an
// STS(15)), a partial one often far fewer than the lex-max search's nodes.
constexpr uint64_t QUICK_TRIALS_COMPLETE = 256;
constexpr uint64_t QUICK_TRIALS_PARTIAL = 2048;

__device__ __forceinline__ void reset_out(CheckOut &o) {
    o.canonical = 1;
    o.status = 0;
    o.reject_row = 0xFF;
    o.rtc = 0xFF;
    o.witness = ~0ull;
    o.aut_lo = 1;
    o.aut_hi = 0;
    o.trials = 0;
    o.n_auts = 0;
    o.len_aut = 0;
}

template <typename S>
__device__ __forceinline__ bool load_rows(S sm, const uint64_t *src, unsigned n, unsigned b, unsigned flags) {
    for (unsigned r = 0; r < n; ++r)
        R_(r) = src[r];
    if (flags & F_RAW)
        normalize_columns(sm, n, b);
    return build_levels(sm, n, b);
}

// The reference path: TestCanonicity() in its own search order (exact trial
// counts and automorphism lists); with F_AUT_CANON a rejected complete matrix is
// then canonised as CanonizeMatrix() does (MatrixCanonChecker.cpp:420-496: move
// the rows as the witness says, renormalise, check again) and |Aut| is that of
// its canonical form.  Outputs other than |Aut| are those of the first check.
__device__ void check_reference(Smem sm, unsigned n, unsigned b, unsigned flags, uint64_t max_trials,
                                uint8_t *aut_dst, unsigned aut_cap, CheckOut &o) {
    search(sm, n, b, flags, max_trials, aut_dst, aut_cap, o);
    if ((flags & F_AUT_CANON) && (flags & F_COMPLETE) && !o.canonical && !o.status) {
        CheckOut c = o;
        for (int round = 0; round < 4096 && !c.canonical && !c.status; ++round) {
            uint64_t tmp[VMAX];
#pragma unroll
            for (unsigned r = 0; r < VMAX; ++r)
                tmp[r] = (r < n) ? R_(r) : 0ull;
            for (unsigned r = 0; r < n; ++r) {
                const unsigned src = pg(c.witness, r);
                uint64_t val = 0;
#pragma unroll
                for (unsigned q = 0; q < VMAX; ++q)
                    if (q == src)
                        val = tmp[q];
                R_(r) = val;
            }
            normalize_columns(sm, n, b);
            build_levels(sm, n, b);
            c.canonical = 1;
            c.witness = ~0ull;
            search(sm, n, b, F_COMPLETE, max_trials, nullptr, 0, c);
        }
        o.aut_lo = c.canonical ? c.aut_lo : 0;
        o.aut_hi = c.canonical ? c.aut_hi : 0;
        o.status |= c.canonical ? c.status : (uint8_t)(c.status | ST_TIMEOUT);
    }
}

// TestCanonicity() of one matrix (rows at `src`, n words).  Unless the reference
// order is required (F_SAVE_AUTS: automorphism lists in the reference's order;
// F_REFERENCE_ORDER: its trial counts), the verdict and |Aut| come from the
// lex-max search, and the witness from a reference-order search: a short one
// first (a random non-canonical matrix is rejected within a few trials), a full
// one only if the lex-max search shows a matrix to be non-canonical that the
// short search did not reject.  Verdict, witness, rowToChange and |Aut| are
// identical either way; `trials` counts the reference-order trials spent.
__device__ void check_one(Smem sm, const uint64_t *src, unsigned n, unsigned b, unsigned flags,
                          uint64_t max_trials, uint8_t *aut_dst, unsigned aut_cap, CheckOut &o,
                          uint64_t order0 = ID16) {
    reset_out(o);
    if (!load_rows(sm, src, n, b, flags)) {
        o.status = ST_BADINPUT;
        o.canonical = 0;
        return;
    }
    if (flags & (F_SAVE_AUTS | F_REFERENCE_ORDER)) {
        check_reference(sm, n, b, flags, max_trials, aut_dst, aut_cap, o);
    } else {
        const unsigned sflags = flags & ~(F_FULL_AUT | F_AUT_CANON);
        const bool aut_always = flags & (F_AUT_CANON | F_FULL_AUT);
        const uint64_t quick_cap = (flags & F_COMPLETE) ? QUICK_TRIALS_COMPLETE : QUICK_TRIALS_PARTIAL;
        search(sm, n, b, sflags, quick_cap < max_trials ? quick_cap : max_trials, nullptr, 0, o);
        if (!(o.status & ST_TIMEOUT)) {
            // the reference-order search finished within the short budget (typical for
            // rejected matrices and for partial matrices with large groups)
            if (!o.canonical) {
                o.aut_lo = 0;            // rejected: the reference leaves |Aut| undefined
                o.aut_hi = 0;
                if (aut_always) {
                    MaxOut mo;
                    max_search(sm, n, b, max_trials, mo, order0);
                    if (mo.timeout)
                        o.status = ST_TIMEOUT;
                    else
                        o.aut_lo = mo.leaves;
                }
            }
        } else {
            const uint64_t quick = o.trials;
            o.status = 0;
            MaxOut mo;
            max_search(sm, n, b, max_trials, mo, order0, true, !aut_always);
            if (mo.timeout) {
                o.status = ST_TIMEOUT;
            } else if (mo.improved && (flags & F_VERDICT_ONLY)) {
                o.canonical = 0;
                o.aut_lo = aut_always ? mo.leaves : 0;
                o.aut_hi = 0;
            } else if (mo.improved) {
                // non-canonical, rejected late in the reference order: find its witness
                load_rows(sm, src, n, b, flags);
                reset_out(o);
                search(sm, n, b, sflags, max_trials, nullptr, 0, o);
                o.trials += quick;
                o.aut_lo = aut_always ? mo.leaves : 0;
                o.aut_hi = 0;
            } else {
                o.canonical = 1;
                o.aut_lo = mo.leaves;
                o.aut_hi = 0;
            }
        }
    }
    if (o.status & ST_TIMEOUT)
        o.canonical = 0;
}

__device__ __forceinline__ void store_witness(uint8_t *dst16, uint64_t w, unsigned n) {
    uint32_t wd[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        uint32_t v = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const unsigned i = q * 4 + k;
            const unsigned byte = (w == ~0ull || i >= n) ? 0xFFu : pg(w, i);
            v |= byte << (8 * k);
        }
        wd[q] = v;
    }
    reinterpret_cast<uint4 *>(dst16)[0] = make_uint4(wd[0], wd[1], wd[2], wd[3]);
}

// One work item of a batch: the check and the writes of every output array.
__device__ void check_item(Smem sm, const Item &item, const uint64_t *__restrict__ words, Outputs out,
                           uint64_t max_trials) {
    const unsigned n = item.nrows, b = item.ncols, o_i = item.out_idx;
    CheckOut o;
    if (item.kind != KIND_BIBD || n < 1 || n > VMAX || b < 1 || b > BMAX) {
        o = CheckOut{0, ST_BADINPUT, 0xFF, 0xFF, ~0ull, 0, 0, 0, 0, 0};
    } else {
        uint8_t *adst =
            (item.flags & F_SAVE_AUTS) && out.auts ? out.auts + (size_t)o_i * out.aut_cap * 64u : nullptr;
        check_one(sm, words + item.data_off, n, b, item.flags, max_trials, adst, out.aut_cap, o);
    }
    out.canonical[o_i] = o.canonical;
    out.status[o_i] = o.status;
    out.reject_row[o_i] = o.reject_row;
    out.row_to_change[o_i] = o.rtc;
    out.player_index[o_i] = -1;
    store_witness(out.witness + (size_t)o_i * 16u, o.witness, n);
    out.aut[2 * (size_t)o_i] = o.aut_lo;
    out.aut[2 * (size_t)o_i + 1] = o.aut_hi;
    out.trials[o_i] = o.trials;
    out.n_auts[o_i] = o.n_auts;
    out.len_aut[o_i] = o.len_aut;
}

}  // namespace
}  // namespace bibd
}  // namespace canon
