// canon_kbin_core.cuh -- the canonical binary matrix of a k-system (runCanonizer()),
// host and device code.
//
// The reference's plugin (createCanonizer / runCanonizer, Source/CDTools.cpp:5-52)
// writes a k-system of v players as a binary matrix: one column per group of each
// day, row p = player p (convertToBinaryMatrix, Source/matrix.h:198-209), under a first
// row that colours the columns by day (prepareFirstMatrixRow, matrix.h:192-197), and
// canonises it with CanonizeMatrix(k, NULL, numClasses)
// (Source/MatrixCanonChecker.cpp:420-564): repeated TestCanonicity() calls until no
// row permutation with the best column arrangement gives a greater matrix, and, for a
// complete k-system, the same over every permutation of the days (the "classes"),
// keeping the greatest.  The result is therefore the lexicographically greatest
// binary matrix (rows top to bottom, columns left to right) over
//   - permutations of the players (rows),
//   - permutations of the groups inside each day (columns inside a day block),
//   - permutations of the days (whole blocks), when all days are given; with fewer
//     days the day order is fixed by the colours.
// Here it is found by one depth-first lex-max search over the rows, like the
// incidence-matrix search: at each level the best arranged row over the unused
// players is computed, the bound's row is raised when it is beaten, and only the
// players that tie are branched on.  The arrangement of a candidate row is greedy:
// inside every column orbit (columns equal in the rows above) its 1s first, and
// inside every block orbit (days whose blocks are equal in the rows above, so
// interchangeable) the blocks in decreasing order of their arranged part.  Every
// leaf that reaches the final bound is a labeling of the canonical form; their number
// is the order of the group of the binary matrix.
#pragma once
#include <cstdint>

#ifndef __CUDACC__
#define __host__
#define __device__
#endif

namespace canon {
namespace kbin {

constexpr int KB_VMAX = 16;      // players
constexpr int KB_BMAX = 63;      // columns (days x groups)
constexpr int KB_DMAX = 16;      // days

struct Shape {
    int v;        // players (rows)
    int b;        // columns
    int g;        // columns of one day
    int nd;       // days
    bool free_days;   // the days may be permuted (a complete k-system)
};

__host__ __device__ inline int kb_popc64(uint64_t x) {
#ifdef __CUDA_ARCH__
    return __popcll(x);
#else
    return __builtin_popcountll(x);
#endif
}
__host__ __device__ inline int kb_ffs(unsigned x) {
#ifdef __CUDA_ARCH__
    return __ffs(x);
#else
    return __builtin_ffs((int)x);
#endif
}
__host__ __device__ inline uint64_t kb_brev(uint64_t x) {
#ifdef __CUDA_ARCH__
    return __brevll(x);
#else
    uint64_t r = 0;
    for (int i = 0; i < 64; ++i)
        r |= ((x >> i) & 1ull) << (63 - i);
    return r;
#endif
}

struct Search {
    Shape sh;
    uint16_t cm[KB_BMAX + 1];        // arranged columns: the players with a 1 in each
    uint64_t bound[KB_VMAX];          // the best rows so far, arranged (bit p = position p)
    uint64_t lvl[KB_VMAX + 1];        // column-orbit starts of each level (block starts included)
    uint32_t blvl[KB_VMAX + 1];       // block-orbit starts of each level (bit t = block t)
    uint32_t rem[KB_VMAX];            // players still to try at each level
    uint8_t perm[KB_VMAX];
};

// The sub-row of player x in block t at level lv: inside every column orbit of the
// block its 1s first, as a g-bit key whose first column is the most significant.
__host__ __device__ inline uint32_t block_key(const Search &S, int lv, int t, int x) {
    const int g = S.sh.g, c0 = t * g;
    const uint64_t st = S.lvl[lv];
    uint32_t key = 0;
    int s = c0;
    while (s < c0 + g) {
        int e = s + 1;
        while (e < c0 + g && !((st >> e) & 1ull))
            ++e;
        int cnt = 0;
        for (int p = s; p < e; ++p)
            cnt += (S.cm[p] >> x) & 1u;
        for (int q = 0; q < cnt; ++q)
            key |= 1u << (g - 1 - (s - c0 + q));
        s = e;
    }
    return key;
}

// The arranged row of player x at level lv: blocks of every block orbit in decreasing
// order of key (bit p = position p)
__host__ __device__ inline uint64_t arranged_row(const Search &S, int lv, int x) {
    const int nd = S.sh.nd, g = S.sh.g;
    const uint32_t bst = S.blvl[lv];
    uint64_t a = 0;
    int t0 = 0;
    while (t0 < nd) {
        int t1 = t0 + 1;
        while (t1 < nd && !((bst >> t1) & 1u))
            ++t1;
        uint32_t keys[KB_DMAX];
        int nk = 0;
        for (int t = t0; t < t1; ++t) {
            const uint32_t k = block_key(S, lv, t, x);
            int j = nk++;
            while (j > 0 && keys[j - 1] < k) {
                keys[j] = keys[j - 1];
                --j;
            }
            keys[j] = k;
        }
        for (int j = 0; j < nk; ++j)
            for (int q = 0; q < g; ++q)
                if ((keys[j] >> (g - 1 - q)) & 1u)
                    a |= 1ull << ((t0 + j) * g + q);
        t0 = t1;
    }
    return a;
}

// Level lv+1 after player x was taken at level lv: inside every block orbit the blocks
// in decreasing order of x's key (stable), split where the keys differ; inside every
// column orbit x's 1s first, split where x's 1s end.
__host__ __device__ inline void refine(Search &S, int lv, int x) {
    const int nd = S.sh.nd, g = S.sh.g;
    const uint32_t bst = S.blvl[lv];
    uint32_t nb = bst;
    int t0 = 0;
    while (t0 < nd) {
        int t1 = t0 + 1;
        while (t1 < nd && !((bst >> t1) & 1u))
            ++t1;
        if (t1 - t0 > 1) {
            uint32_t keys[KB_DMAX];
            uint8_t idx[KB_DMAX];
            int nk = 0;
            for (int t = t0; t < t1; ++t) {
                const uint32_t k = block_key(S, lv, t, x);
                int j = nk++;
                while (j > 0 && keys[j - 1] < k) {
                    keys[j] = keys[j - 1];
                    idx[j] = idx[j - 1];
                    --j;
                }
                keys[j] = k;
                idx[j] = (uint8_t)t;
            }
            uint16_t buf[KB_BMAX + 1];
            for (int j = 0; j < nk; ++j)
                for (int q = 0; q < g; ++q)
                    buf[j * g + q] = S.cm[idx[j] * g + q];
            for (int j = 0; j < nk * g; ++j)
                S.cm[t0 * g + j] = buf[j];
            for (int j = 1; j < nk; ++j)
                if (keys[j] != keys[j - 1])
                    nb |= 1u << (t0 + j);
        }
        t0 = t1;
    }
    S.blvl[lv + 1] = nb;
    const uint64_t st = S.lvl[lv];
    uint64_t ns = st;
    const int b = S.sh.b;
    int s = 0;
    while (s < b) {
        int e = s + 1;
        while (e < b && !((st >> e) & 1ull))
            ++e;
        int w = s;
        for (int p = s; p < e; ++p) {
            const uint16_t c = S.cm[p];
            if ((c >> x) & 1u) {
                S.cm[p] = S.cm[w];
                S.cm[w] = c;
                ++w;
            }
        }
        if (w > s && w < e)
            ns |= 1ull << w;
        s = e;
    }
    S.lvl[lv + 1] = ns;
}

struct Result {
    uint64_t leaves;      // labelings reaching the canonical form
    uint64_t nodes;
    bool timeout;
};

// rows: v player rows, bit c = column c (day d's groups at columns d*g .. d*g+g-1).
// On return S.bound[0..v-1] hold the canonical matrix (bit p = column p).
__host__ __device__ inline Result canonize(Search &S, const uint64_t *rows, uint64_t max_nodes) {
    const int v = S.sh.v, b = S.sh.b, g = S.sh.g;
    for (int c = 0; c < b; ++c) {
        uint16_t m = 0;
        for (int r = 0; r < v; ++r)
            m |= (uint16_t)(((rows[r] >> c) & 1ull) << r);
        S.cm[c] = m;
    }
    uint64_t starts = 0;
    for (int t = 0; t < S.sh.nd; ++t)
        starts |= 1ull << (t * g);
    S.lvl[0] = starts;
    S.blvl[0] = S.sh.free_days ? 1u : ((1u << S.sh.nd) - 1u);
    Result res{0, 0, false};
    int valid = 0;                   // rows 0..valid-1 of the bound are set
    unsigned used = 0;
    int i = 0;
    bool enter = true;
    for (;;) {
        if (enter) {
            if (i == v) {
                ++res.leaves;
                enter = false;
                --i;
                used &= ~(1u << S.perm[i]);
                continue;
            }
            if (++res.nodes > max_nodes) {
                res.timeout = true;
                return res;
            }
            // the greatest arranged row over the unused players
            uint64_t best = 0, best_key = 0;
            unsigned tied = 0;
            for (int x = 0; x < v; ++x) {
                if ((used >> x) & 1u)
                    continue;
                const uint64_t a = arranged_row(S, i, x);
                const uint64_t k = kb_brev(a);
                if (!tied || k > best_key) {
                    best = a;
                    best_key = k;
                    tied = 1u << x;
                } else if (k == best_key) {
                    tied |= 1u << x;
                }
            }
            int state = 0;      // 1: greater than the bound, 2: smaller
            if (i < valid) {
                const uint64_t bk = kb_brev(S.bound[i]);
                state = best_key > bk ? 1 : (best_key < bk ? 2 : 0);
            }
            if (state == 2) {
                enter = false;
                if (i == 0)
                    break;
                --i;
                used &= ~(1u << S.perm[i]);
                continue;
            }
            if (state == 1 || i >= valid) {
                if (state == 1)
                    res.leaves = 0;
                S.bound[i] = best;
                valid = i + 1;
            }
            S.rem[i] = tied;
        }
        // the next tied player at level i
        const unsigned rm = S.rem[i];
        if (!rm) {
            if (i == 0)
                break;
            enter = false;
            --i;
            used &= ~(1u << S.perm[i]);
            continue;
        }
        const int x = kb_ffs(rm) - 1;
        S.rem[i] = rm & (rm - 1);
        if (i + 1 < v)
            refine(S, i, x);
        S.perm[i] = (uint8_t)x;
        used |= 1u << x;
        ++i;
        enter = true;
    }
    return res;
}

}  // namespace kbin
}  // namespace canon
