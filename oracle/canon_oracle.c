/*
 * canon_oracle.c -- CPU oracle (TEST INFRASTRUCTURE ONLY).
 *
 * Plain-C restatement of the reference canonicity checkers.  Used by tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker of
 * the CUDA path.  The product library never links or calls this file.
 *
 * Parity pins (see tests/): the GroupOrder restatement is cross-checked
 * against the reference's own CGroupOrder<T> compiled in place from
 * k-Factorization/Utils/Include/GroupOrder.h; the full checkers are pinned on
 * the reference's published known answers (BIBD |Aut| histograms in the
 * Results/BIBDs per-v folders, the 396 canonical K10 matrices in
 * k-Factorization/Results/Complete_graphs/10/10x9x2/K_OrderedMatrices.txt).
 */
#include "canon_oracle.h"
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;

/* =====================================================================
 * GroupOrder.h restatement (k-Factorization/Utils/Include/GroupOrder.h)
 * ===================================================================== */

/* revert(), GroupOrder.h:25-28: reverse perm[i+1 .. j-1] */
static void or_revert(uint8_t *perm, uint8_t j, uint8_t i)
{
    while (++i < --j) {
        uint8_t t = perm[i];
        perm[i] = perm[j];
        perm[j] = t;
    }
}

/* Update_Orbits(), GroupOrder.h:30-49: merge orbits under permut, starting at idx */
static void or_merge_orbits(const uint8_t *permut, unsigned len, uint8_t *orb, unsigned idx)
{
    do {
        uint8_t a = orb[idx];
        uint8_t c = orb[permut[idx]];
        if (a == c)
            continue;
        if (c < a) {
            uint8_t t = a;
            a = c;
            c = t;
        }
        for (unsigned k = len; k--;)
            if (orb[k] == c)
                orb[k] = a;
    } while (++idx < len);
}

/* updateGroupOrder(), GroupOrder.h:63-73 */
void or_update_group_order(or_group *g, unsigned degree, const uint8_t *orb)
{
    unsigned long len = 1;
    uint16_t idx = (uint16_t)g->stab_aut;
    while (++idx < degree) {
        if (orb[idx] == g->stab_aut)
            len++;
    }
    g->order *= len;
}

/* addAutomorphism() -> UpdateOrbits() -> udpdateStabLength() + Update_Orbits(),
 * GroupOrder.h:56-62, 76-79, 88-102 (needUpdate() is always true for the checker). */
void or_add_automorphism(or_group *g, unsigned degree, const uint8_t *perm, uint8_t *orb,
                         int row_permut, int calc_group_order)
{
    uint8_t idx = 0;
    while (idx == perm[idx])
        idx++;
    if (calc_group_order) {
        if (row_permut && g->stab_aut > idx)
            or_update_group_order(g, degree, orb);
        g->stab_aut = idx;
    }
    g->stab = idx;
    or_merge_orbits(perm, degree, orb, idx);
}

/* next_permutation(), GroupOrder.h:136-248.  Lexicographic successor of perm
 * that changes a position >= len_stab, skipping candidates that are not orbit
 * leaders at position stabilizerLength().  idx: ELEMENT_MAX = plain successor;
 * IDX_MAX = first call after an automorphism; otherwise the row whose
 * comparison was "greater" (every permutation sharing perm[0..idx] is skipped). */
uint8_t or_next_permutation(or_group *g, uint8_t *perm, const uint8_t *orb, uint8_t n,
                            uint8_t idx, uint8_t len_stab)
{
    uint8_t temp, i, j;

    if (idx == OR_IMAX && perm[g->stab] == (uint8_t)(n - 1))
        idx = OR_EMAX;

    if (idx == OR_IMAX) {
        /* first call after an automorphism: smallest permutation with the
         * prefix (0 .. s-1, perm[s]) where s = stabilizerLength() */
        i = (uint8_t)g->stab;
        idx = i;
        temp = perm[i];
        for (j = n; --j > temp;)
            perm[j] = j;
        uint8_t k = j++;
        while (k-- > i)
            perm[k + 1] = k;
    } else if (idx >= OR_IMAX) {
        j = i = n;
        while (--i > 0 && perm[i - 1] >= perm[i])
            ;
        if (i == len_stab)
            return OR_EMAX;
        temp = perm[--i];
        while (perm[--j] <= temp)
            ;
    } else {
        temp = perm[j = i = idx];
        while (++j < n && perm[j] <= temp)
            ;
        if (j >= n) {
            or_revert(perm, n, i);
            return or_next_permutation(g, perm, orb, n, OR_EMAX, 0);
        }
    }

    if (g->stab == i) {
        int flag = 0;
        uint8_t k = j, tmp = perm[j];
        if (idx >= OR_IMAX) {
            while (k > i && orb[perm[k]] != perm[k])
                k--;
            if (k != j) {
                if (!k)
                    return OR_EMAX;
                flag = (k == i);
                tmp = perm[k--];
                while (++k < j)
                    perm[k] = perm[k + 1];
            }
        } else {
            while (k < n && orb[perm[k]] != perm[k])
                k++;
            if (k != j) {
                flag = (k == n);
                if (flag) {
                    if (!i)
                        return OR_EMAX;
                    k = (uint8_t)(idx - 1);
                    while (++k < j)
                        perm[k] = k;
                } else {
                    tmp = perm[k++];
                    while (--k > j)
                        perm[k] = perm[k - 1];
                }
            }
        }
        perm[j] = tmp;
        if (flag) {
            j = idx >= OR_IMAX ? (uint8_t)(n - 1) : i;
            temp = perm[--i];
            g->stab = i;
        }
    }

    perm[i] = perm[j];
    perm[j] = temp;
    if (idx >= OR_IMAX) {
        if (g->stab > i)
            g->stab = i;
        or_revert(perm, n, i);
    }
    return i;
}

/* The checker below calls the permutation machinery through these pointers so
 * that the tests can substitute the reference's own CGroupOrder<T> (compiled in
 * place from GroupOrder.h) and compare every output. */
typedef uint8_t (*or_np_fn)(or_group *, uint8_t *, const uint8_t *, uint8_t, uint8_t, uint8_t);
typedef void (*or_aa_fn)(or_group *, unsigned, const uint8_t *, uint8_t *, int, int);
typedef void (*or_ugo_fn)(or_group *, unsigned, const uint8_t *);
static or_np_fn g_np = or_next_permutation;
static or_aa_fn g_aa = or_add_automorphism;
static or_ugo_fn g_ugo = or_update_group_order;

void or_set_group_impl(void *np_fn, void *aa_fn, void *ugo_fn)
{
    g_np = np_fn ? (or_np_fn)np_fn : or_next_permutation;
    g_aa = aa_fn ? (or_aa_fn)aa_fn : or_add_automorphism;
    g_ugo = ugo_fn ? (or_ugo_fn)ugo_fn : or_update_group_order;
}

/* =====================================================================
 * Column orbits of a rank-2 incidence matrix.
 * The reference keeps per-row linked lists of {length,next} nodes
 * (Source/ColOrbits.h:4-53, ColOrbitManager.h:19-74) built by MakeRow
 * (MatrixCanonChecker.cpp:14-93): the orbits of row n are the classes of
 * columns that are identical in rows 0..n-1, each a contiguous range because
 * every row is 1s-first inside every orbit of the rows above it.  Here the
 * orbits of level n are given by their start columns.
 * ===================================================================== */
#define OR_BMAX 64
#define OR_RMAX 16      /* entries below this (rank of the coloured first row of a k-system) */
#define OR_KS_NPMAX 16  /* players of a k-system whose binary matrix is canonised */
typedef struct {
    int n;                    /* number of orbits */
    uint8_t start[OR_BMAX];
    uint8_t len[OR_BMAX];
} or_orbits;

static void or_level_orbits(const uint8_t *M, int level, int b, or_orbits *o)
{
    o->n = 0;
    int s = 0;
    for (int c = 1; c <= b; c++) {
        int same = c < b;
        for (int r = 0; same && r < level; r++)
            if (M[r * b + c] != M[r * b + c - 1])
                same = 0;
        if (!same) {
            o->start[o->n] = (uint8_t)s;
            o->len[o->n] = (uint8_t)(c - s);
            o->n++;
            s = c;
        }
    }
}

int or_bibd_is_normal(const uint8_t *M, int nrows, int b)
{
    or_orbits o;
    for (int r = 0; r < nrows; r++) {
        or_level_orbits(M, r, b, &o);
        for (int q = 0; q < o.n; q++) {
            int seen0 = 0;
            for (int c = o.start[q]; c < o.start[q] + o.len[q]; c++) {
                if (M[r * b + c] > 1)
                    return 0;
                if (!M[r * b + c])
                    seen0 = 1;
                else if (seen0)
                    return 0;
            }
        }
    }
    return 1;
}

/* GenerateBinaryColumnOrbits(), MatrixCanonChecker.cpp:186-263, applied to rows
 * 0..nrows-1 in turn with column swaps carried into the rows below (pColPermut
 * == NULL branch): inside every orbit the first 0 from the left is swapped with
 * the last 1 from the right until the row is 1s-first. */
/* GenerateBinaryColumnOrbits() of binary rows from..nrows-1 (rows above `from` are
 * kept as they are; they may hold other values, as the coloured first row of a
 * k-system's binary matrix does) */
static void or_normalize_rows(uint8_t *M, int nrows, int b, int from)
{
    or_orbits o;
    for (int r = from; r < nrows; r++) {
        or_level_orbits(M, r, b, &o);
        uint8_t *row = M + r * b;
        for (int q = 0; q < o.n; q++) {
            int s = o.start[q], e = s + o.len[q];
            if (o.len[q] < 2)
                continue;
            int ones = 0;
            for (int c = s; c < e; c++)
                ones += row[c];
            if (!ones || ones == o.len[q])
                continue;
            int j1 = s, j2 = e;
            const int jlast = s + ones;
            while (j1 < jlast) {
                while (row[j1])
                    j1++;
                if (j1 == jlast)
                    break;
                while (!row[--j2])
                    ;
                for (int r2 = r + 1; r2 < nrows; r2++) {
                    uint8_t *nx = M + r2 * b;
                    uint8_t t = nx[j1];
                    nx[j1] = nx[j2];
                    nx[j2] = t;
                }
                row[j1++] = 1;
                row[j2] = 0;
            }
        }
    }
}

void or_bibd_normalize(uint8_t *M, int nrows, int b)
{
    or_normalize_rows(M, nrows, b, 0);
}

/* checkColOrbit(), CanonicityChecker.cpp:191-223: compare, from the greatest value
 * down to 1, the number of entries of each value of row `row` inside orbit
 * [s, s+len) with the same count of the permuted row under the current column
 * arrangement; on equality reorder permCol inside the orbit by decreasing value
 * (each value class keeping its order).  Rank 2 is the incidence-matrix case
 * (counts of 1s); the binary matrix of a k-system has a first row of rank > 2. */
static int or_check_col_orbit(int len, int s, const uint8_t *row, const uint8_t *rowPerm,
                              uint8_t *permCol, int rank)
{
    int cnt_row[OR_RMAX] = {0}, cnt_perm[OR_RMAX] = {0};
    for (int i = 0; i < len; i++) {
        cnt_row[row[s + i]]++;
        cnt_perm[rowPerm[permCol[s + i]]]++;
    }
    for (int v = rank - 1; v >= 1; v--) {
        const int diff = cnt_row[v] - cnt_perm[v];
        if (diff < 0)
            return -1;
        if (diff > 0)
            return 1;
    }
    uint8_t out[OR_BMAX];
    int k = 0;
    for (int v = rank - 1; v >= 0; v--)
        for (int i = 0; i < len; i++)
            if (rowPerm[permCol[s + i]] == v)
                out[k++] = permCol[s + i];
    memcpy(permCol + s, out, len);
    return 0;
}

/* every row non-increasing inside every column orbit of the rows above it (for rank
 * 2: 1s-first); values below `rank` */
static int or_rank_is_normal(const uint8_t *M, int nrows, int b, int rank)
{
    or_orbits o;
    for (int r = 0; r < nrows; r++) {
        or_level_orbits(M, r, b, &o);
        for (int q = 0; q < o.n; q++)
            for (int c = o.start[q]; c < o.start[q] + o.len[q]; c++) {
                if (M[r * b + c] >= rank)
                    return 0;
                if (c > o.start[q] && M[r * b + c] > M[r * b + c - 1])
                    return 0;
            }
    }
    return 1;
}

/* TestCanonicity(), Source/CanonicityChecker.h:255-586, for numParts == 1, no
 * group on parts, no row-solution pruning (pRowSolution == NULL).  Complete
 * matrices: out_info = OR_SAVE_ROW_PERM | OR_SAVE_ROW_TO_CHANGE (Enumerator.cpp:696);
 * partial matrices: OR_SAVE_NOTHING (Enumerator.cpp:446-447), automorphisms are
 * stored as permutations of the column orbits of the last level (:427-451). */
static int or_test_rank(const uint8_t *M, int nrows, int b, int rank, unsigned out_info, int len_stab,
                        or_bibd_result *res);

int or_bibd_test(const uint8_t *M, int nrows, int b, unsigned out_info, int len_stab,
                 or_bibd_result *res)
{
    return or_test_rank(M, nrows, b, 2, out_info, len_stab, res);
}

/* TestCanonicity() for entries below `rank` (the reference's rank(): maxElement + 1) */
static int or_test_rank(const uint8_t *M, int nrows, int b, int rank, unsigned out_info, int len_stab,
                        or_bibd_result *res)
{
    if (nrows < 1 || nrows > 64 || b < 1 || b > OR_BMAX || rank < 2 || rank > OR_RMAX)
        return -1;
    if (!or_rank_is_normal(M, nrows, b, rank))
        return -2;

    const int row_permut = (out_info & OR_SAVE_ROW_PERM) != 0;
    const int full_aut = (out_info & OR_FULL_AUT) != 0;
    const uint8_t n = (uint8_t)nrows;

    or_orbits lv[65];
    for (int r = 0; r <= nrows; r++)
        or_level_orbits(M, r, b, &lv[r]);

    memset(&res->st, 0, sizeof(res->st));
    res->canonical = 1;
    res->reject_row = -1;
    res->row_to_change = -1;
    res->aut_lo = 0;   /* |Aut| stays 0 when the check stops at a rejection */
    res->aut_hi = 0;
    res->n_perm = 0;
    res->len_perm = 0;
    res->perm_overflow = 0;

    /* init(), CanonicityChecker.cpp:35-84 */
    or_group g;
    g.stab = n - 1;
    g.stab_aut = OR_EMAX;
    g.order = 1;
    uint8_t perm[64], orb[64], permCol[OR_BMAX];
    for (int i = 0; i < nrows; i++)
        perm[i] = orb[i] = (uint8_t)i;
    for (int c = 0; c < b; c++)
        permCol[c] = (uint8_t)c;
    /* Extension: partial checks (no row permutations saved) do not call
     * updateGroupOrder() in the reference; the same orbit-length product is
     * accumulated here so that |Aut| of a partial matrix is reported too. */
    u128 part_order = 1;

    /* colIndex(): orbit index of each start column of the last level
     * (constructColIndex, CanonicityChecker.cpp:332-342) */
    uint8_t colIndex[OR_BMAX];
    uint8_t orbitOf[OR_BMAX];
    const or_orbits *last = &lv[nrows];
    for (int q = 0; q < last->n; q++)
        for (int c = last->start[q]; c < last->start[q] + last->len[q]; c++) {
            orbitOf[c] = (uint8_t)q;
            colIndex[c] = (uint8_t)q;
        }
    if (row_permut && res->perm_arena && res->perm_cap > 0) {
        /* init() saves the trivial row permutation when rows are permuted */
        memcpy(res->perm_arena, perm, n);
        res->n_perm = 1;
        res->len_perm = n;
    } else if (row_permut) {
        res->n_perm = 1;
        res->len_perm = n;
    }

    int rejected = 0;
    uint8_t nRow = OR_EMAX;
    for (;;) {
    next_permut:
        nRow = g_np(&g, perm, orb, n, nRow, (uint8_t)len_stab);
        if (nRow == OR_EMAX)   /* lenStabilizer() == 0 for BIBDs (:330) */
            break;
        res->st.trials++;
        for (; nRow < n; nRow++) {
            const uint8_t *row = M + nRow * b;
            const uint8_t *rowPerm = M + perm[nRow] * b;
            const or_orbits *o = &lv[nRow];
            res->st.rows++;
            for (int q = 0; q < o->n; q++) {
                int s = o->start[q], len = o->len[q], diff;
                res->st.orbits++;
                if (len > 1)
                    diff = or_check_col_orbit(len, s, row, rowPerm, permCol, rank);
                else
                    diff = (int)row[s] - (int)rowPerm[permCol[s]];
                if (diff > 0)
                    goto next_permut;
                if (!diff)
                    continue;
                /* diff < 0: the permuted matrix is greater */
                if (!rejected) {
                    rejected = 1;
                    res->canonical = 0;
                    res->reject_row = nRow;
                    memcpy(res->witness, perm, n);
                    /* rowToChange(), CanonicityChecker.cpp:320-330 */
                    uint8_t rtc = nRow;
                    for (int i = nRow; i >= 0; i--)
                        if (rtc < perm[i])
                            rtc = perm[i];
                    res->row_to_change = rtc;
                }
                if (!full_aut)
                    return 0;
                goto next_permut;
            }
        }

        /* automorphism found (:421-476) */
        res->st.auts++;
        if (!row_permut) {
            /* permutation of the column orbits of the last level (:430-450) */
            if (res->n_perm == 0) {
                res->len_perm = last->n;
                if (res->perm_arena && res->perm_cap > 0)
                    for (int q = 0; q < last->n; q++)
                        res->perm_arena[q] = (uint8_t)q;  /* identity placeholder */
                res->n_perm = 1;
            }
            if (res->perm_arena && res->n_perm < res->perm_cap) {
                uint8_t *dst = res->perm_arena + (size_t)res->n_perm * res->len_perm;
                for (int q = 0; q < last->n; q++) {
                    /* colIndex() of the image of the orbit start; the image of an
                     * orbit under an automorphism is an orbit, addressed by its index */
                    dst[q] = colIndex[last->start[orbitOf[permCol[last->start[q]]]]];
                }
            } else if (res->perm_arena) {
                res->perm_overflow = 1;
            }
            res->n_perm++;
        }
        if (!row_permut) {
            uint8_t idx = 0;
            while (idx == perm[idx])
                idx++;
            if (g.stab_aut > idx) {
                or_group t = g;
                t.order = 1;
                g_ugo(&t, n, orb);
                part_order *= t.order;
            }
        }
        g_aa(&g, n, perm, orb, row_permut, 1);
        if (row_permut && (out_info & OR_SAVE_AUT_ROWS)) {
            /* t_outRowPermute: savePermutation() keeps every row automorphism */
            if (res->perm_arena && res->n_perm < res->perm_cap)
                memcpy(res->perm_arena + (size_t)res->n_perm * n, perm, n);
            res->n_perm++;
        }
        nRow = OR_IMAX;
    }

    if (row_permut) {
        g_ugo(&g, n, orb);
        res->aut_lo = (uint64_t)g.order;
        res->aut_hi = (uint64_t)(g.order >> 64);
    } else {
        or_group t = g;
        t.order = 1;
        g_ugo(&t, n, orb);
        part_order *= t.order;
        res->aut_lo = (uint64_t)part_order;
        res->aut_hi = (uint64_t)(part_order >> 64);
    }
    if (res->perm_arena && res->n_perm > res->perm_cap)
        res->perm_overflow = 1;
    return 0;
}

/* CanonizeMatrix(), MatrixCanonChecker.cpp:420-496 for k == 0, numClasses == 0:
 * repeat TestCanonicity(v, t_saveRowPermutations); on rejection move the rows as
 * permRow() says and rebuild the column orbits of the moved rows and below. */
int or_bibd_canonize(uint8_t *M, int nrows, int b, or_bibd_result *res)
{
    or_bibd_normalize(M, nrows, b);
    int calls = 0;
    uint8_t tmp[64 * OR_BMAX];
    for (;;) {
        uint8_t *arena = res->perm_arena;
        int cap = res->perm_cap;
        int rc = or_bibd_test(M, nrows, b, OR_SAVE_ROW_PERM, 0, res);
        res->perm_arena = arena;
        res->perm_cap = cap;
        calls++;
        if (rc < 0)
            return rc;
        if (res->canonical)
            return calls;
        /* row i of the new matrix is old row permRow[i] (cycle walk :461-475) */
        memcpy(tmp, M, (size_t)nrows * b);
        int first = -1;
        for (int i = 0; i < nrows; i++) {
            memcpy(M + i * b, tmp + res->witness[i] * b, b);
            if (first < 0 && res->witness[i] != i)
                first = i;
        }
        /* GenerateBinaryColumnOrbits from the first moved row on (:476-488);
         * rows above `first` are unchanged and already 1s-first */
        (void)first;
        or_bibd_normalize(M, nrows, b);
    }
}

/* =====================================================================
 * runCanonizer(): the canonical binary matrix of a k-system
 * (Source/CDTools.cpp:5-52).  createCanonizer(v, k) sets up a C_InSys of v+1 rows
 * and b = numDays*v/k columns whose first row colours the columns by day
 * (prepareFirstMatrixRow, Source/matrix.h:192-197: numDays groups of v/k columns,
 * values numDays-1 down to 0); runCanonizer() fills rows 1..v from the k-system
 * (convertToBinaryMatrix, matrix.h:198-209: column = one group of one day, row
 * 1+p = player p), keeps only the first dayNumb days when fewer are given
 * (adjustData: the columns of the first days dropped, the rank set to dayNumb,
 * no class permutations), and calls CanonizeMatrix(k, NULL, numClasses)
 * (Source/MatrixCanonChecker.cpp:420-564) with numClasses = numDays for a complete
 * matrix.  The result is rows 1..v of the canonised matrix.
 * ===================================================================== */

static int or_cmp_desc_len;
static int or_row_cmp_desc(const void *a, const void *b)
{
    return memcmp(b, a, (size_t)or_cmp_desc_len);   /* compareRows(), MatrixCanonChecker.cpp:389-392 */
}

/* sortRowsUpdateColumnOrbits(), MatrixCanonChecker.cpp:394-418: rows from..v-1 in
 * decreasing order, then GenerateBinaryColumnOrbits() for each of them */
static void or_sort_rows_update(uint8_t *M, int v, int b, int from)
{
    or_cmp_desc_len = b;
    qsort(M + (size_t)from * b, (size_t)(v - from), (size_t)b, or_row_cmp_desc);
    or_normalize_rows(M, v, b, from);
}

/* the TestCanonicity() loop of CanonizeMatrix() (:450-494) for a matrix whose first
 * row is never moved (nRowStart = 1, k > 0); returns the number of calls */
static int or_canonize_rank(uint8_t *M, int v, int b, int rank)
{
    or_bibd_result res;
    memset(&res, 0, sizeof(res));
    uint8_t tmp[(OR_KS_NPMAX + 1) * OR_BMAX];
    int calls = 0;
    for (;;) {
        if (or_test_rank(M, v, b, rank, OR_SAVE_ROW_PERM, 0, &res) < 0)
            return -1;
        calls++;
        if (res.canonical)
            return calls;
        /* row i of the new matrix is old row permRow()[i] (:458-475) */
        memcpy(tmp, M, (size_t)v * b);
        int first = -1;
        for (int i = 1; i < v; i++) {
            memcpy(M + (size_t)i * b, tmp + (size_t)res.witness[i] * b, (size_t)b);
            if (first < 0 && res.witness[i] != i)
                first = i;
        }
        if (first < 0)
            return -1;      /* a rejection always moves a row */
        /* GenerateBinaryColumnOrbits() from the first moved row on (:476-486), then,
         * k > 0, sortRowsUpdateColumnOrbits() from there (:488-492) */
        or_normalize_rows(M, v, b, first);
        or_sort_rows_update(M, v, b, first);
    }
}

int or_ksys_binary_canonize(const uint8_t *R, int np, int k, int day_numb, uint8_t *out, long *class_steps)
{
    if (k < 2 || np < 2 * k || np % k || (np - 1) % (k - 1) || np > OR_KS_NPMAX)
        return -1;
    const int num_days = (np - 1) / (k - 1);
    const int g = np / k;                           /* groups (columns) of one day */
    if (day_numb <= 0)
        day_numb = num_days;
    if (day_numb < 2 || day_numb > num_days || day_numb * g > OR_BMAX)
        return -1;
    const int num_classes = day_numb == num_days ? num_days : 0;
    const int rank = day_numb;
    const int v = np + 1, b = day_numb * g;
    uint8_t M[(OR_KS_NPMAX + 1) * OR_BMAX];
    memset(M, 0, sizeof(M));
    for (int c = 0; c < b; c++)
        M[c] = (uint8_t)(day_numb - 1 - c / g);     /* the day colours, highest first */
    for (int d = 0; d < day_numb; d++)
        for (int j = 0; j < g; j++)
            for (int n = 0; n < k; n++)
                M[(size_t)(1 + R[d * np + j * k + n]) * b + d * g + j] = 1;
    /* k > 0: rows sorted and made 1s-first inside the day groups (:440-451) */
    or_sort_rows_update(M, v, b, 1);

    const size_t len_data = (size_t)np * b;         /* rows 1..v of the matrix */
    uint8_t comp[OR_KS_NPMAX * OR_BMAX];
    int have_comp = 0, cmp = 1;
    uint8_t idx = OR_IMAX;
    uint8_t cperm[OR_KS_NPMAX], corb[OR_KS_NPMAX];
    or_group cg;
    memset(&cg, 0, sizeof(cg));
    cg.order = 1;
    long steps = 0;
    for (;;) {
        if (or_canonize_rank(M, v, b, rank) < 0)
            return -2;
        if (!num_classes)
            break;
        steps++;
        if (have_comp) {
            const int c = memcmp(M + b, comp, len_data);
            cmp = (c > 0) - (c < 0);
            if (!cmp) {
                /* the same matrix again: an automorphism on the classes */
                g_aa(&cg, (unsigned)num_classes, cperm, corb, 1, 1);
                idx = OR_IMAX;
            } else if (cmp < 0) {
                memcpy(M + b, comp, len_data);
            }
        } else {
            have_comp = 1;
        }
        if (cmp == 1) {
            /* initOrbits(), CanonicityChecker.h:78-87: identity, trivial orbits */
            cg.stab = cg.stab_aut = (unsigned)num_classes - 1;
            for (int i = 0; i < num_classes; i++)
                cperm[i] = corb[i] = (uint8_t)i;
            memcpy(comp, M + b, len_data);
        }
        idx = g_np(&cg, cperm, corb, (uint8_t)num_classes, idx, 0);
        if (idx == OR_EMAX)
            break;
        /* The reference passes lenPerm as the next index; next_permutation() then takes
         * its branch for an index past the last element, which reverses nothing and
         * continues as a plain next permutation (ELEMENT_MAX, no stabiliser). */
        idx = OR_EMAX;
        int i = 0;
        while (cperm[i] == i)
            i++;
        /* the column groups of rows 1..v in the order of the class permutation (:526-535) */
        for (; i < num_classes; i++)
            for (int r = 1; r < v; r++)
                memcpy(M + (size_t)r * b + (size_t)i * g, comp + (size_t)(r - 1) * b + (size_t)cperm[i] * g,
                       (size_t)g);
        or_sort_rows_update(M, v, b, 1);
    }
    memcpy(out, M + b, len_data);
    if (class_steps)
        *class_steps = steps;
    return b;
}

/* =====================================================================
 * k-system checker: alldata::cnvCheckNew() plain path
 * (k-Factorization/TripleSys/Source/cnv.cpp:211-351), with
 * m_pCheckFunc == NULL, USE_EQUAL 0, no automorphism-group reuse, no nested
 * groups, no row precalculation.  ProcessMatrix follows kmProcessMatrix
 * (kmSupport.cpp:220-313), whose result sign and setPlayerIndex arguments
 * equal those of the group-size-2 variant kmProcessMatrix2 (:601-700).
 * ===================================================================== */
#define OR_NPMAX 64

typedef struct {
    int np, g, ng, nrows, gfact;
    const uint8_t *R;
    uint8_t groups[24 * 4];   /* cnvInit(): in-group orders, cnv.cpp:45-64 */
    int player_index;
    uint64_t n_aut;
    uint8_t *arena;
    int cap, overflow;
    int full;
    uint64_t cand;
    uint64_t tr_ind;
} or_ks;

/* sorted-set insertion of an automorphism (CStorageIdx::updateRepo, Storage.h:181-196) */
static void or_ks_add_aut(or_ks *k, const uint8_t *tr)
{
    const int np = k->np;
    if (!k->arena || k->n_aut >= (uint64_t)k->cap) {
        /* cannot check for duplicates without storage; relabelings are distinct */
        if (k->arena)
            k->overflow = 1;
        k->n_aut++;
        return;
    }
    long lo = 0, hi = (long)k->n_aut;
    while (lo < hi) {
        long mid = (lo + hi) / 2;
        int c = memcmp(k->arena + mid * np, tr, np);
        if (c == 0)
            return;
        if (c < 0)
            lo = mid + 1;
        else
            hi = mid;
    }
    memmove(k->arena + (lo + 1) * np, k->arena + lo * np, (k->n_aut - lo) * np);
    memcpy(k->arena + lo * np, tr, np);
    k->n_aut++;
}

/* setPlayerIndexByPos / setPlayerIndex, kmSupport.cpp:314-356 */
static void or_ks_player_index(or_ks *k, const uint8_t *tr, int day_max, int day_cur,
                               const uint8_t *co, const uint8_t *ci, const uint8_t *ci_from)
{
    if (day_max > day_cur || !tr)
        return;
    const int np = k->np;
    const int imax = np - k->g - 1;
    int ip = 0;
    for (; ip < imax; ip++)
        if (co[ip] < ci[ip])
            break;
    uint8_t ttr[OR_NPMAX], tpr[OR_NPMAX];
    for (int i = 0; i < np; i++) {
        tpr[ci_from[i]] = (uint8_t)i;
        ttr[tr[i]] = (uint8_t)i;
    }
    int j = 0;
    for (int i = 0; i <= ip; i++) {
        int q = tpr[ttr[co[i]]];
        if (j < q)
            j = q;
    }
    int pi = day_cur * np + j;
    if (k->player_index > pi)
        k->player_index = pi;
}

static int or_sign(int c) { return (c > 0) - (c < 0); }

/* kmProcessMatrix(): relabel, sort each group, sort groups by first player,
 * sort rounds by their second entry, compare with the original round by round.
 * Returns -1 (relabelled matrix smaller), 0 (equal) or >0. */
static int or_ks_process(or_ks *k, const uint8_t *tr)
{
    const int np = k->np, g = k->g, nr = k->nrows, ng = k->ng;
    uint8_t tmp[OR_NPMAX * OR_NPMAX], srt[OR_NPMAX * OR_NPMAX];
    uint8_t ts[OR_NPMAX];
    const uint8_t *mi = k->R;
    for (int r = 0; r < nr; r++) {
        uint8_t row[OR_NPMAX];
        for (int i = 0; i < np; i++)
            row[i] = tr[mi[r * np + i]];
        /* sort inside each group (kmSortGroups*) */
        for (int q = 0; q < ng; q++) {
            uint8_t *p = row + q * g;
            for (int a = 1; a < g; a++)
                for (int c = a; c > 0 && p[c - 1] > p[c]; c--) {
                    uint8_t t = p[c];
                    p[c] = p[c - 1];
                    p[c - 1] = t;
                }
        }
        /* groups ordered by first element (kmSortGroupsByFirstValue) */
        const uint8_t *byFirst[OR_NPMAX];
        memset(byFirst, 0, sizeof(byFirst));
        for (int q = 0; q < ng; q++)
            byFirst[row[q * g]] = row + q * g;
        uint8_t *o = tmp + r * np;
        for (int v = 0; v < np; v++)
            if (byFirst[v]) {
                memcpy(o, byFirst[v], g);
                o += g;
            }
    }
    /* rounds ordered by their second entry (kmSortRowsBy2ndValue) */
    const uint8_t *by2[OR_NPMAX];
    uint8_t src[OR_NPMAX];
    memset(by2, 0, sizeof(by2));
    for (int r = 0; r < nr; r++) {
        by2[tmp[r * np + 1]] = tmp + r * np;
        src[tmp[r * np + 1]] = (uint8_t)r;
    }
    int j = 0;
    for (int v = 0; v < np && j < nr; v++)
        if (by2[v]) {
            memcpy(srt + j * np, by2[v], np);
            ts[j] = src[v];
            j++;
        }
    int day_max = ts[0];
    for (int i = 0; i < nr; i++) {
        int c = or_sign(memcmp(srt + i * np, mi + i * np, np));
        if (c < 0) {
            or_ks_player_index(k, tr, day_max, ts[i], srt + i * np, mi + i * np, mi + ts[i] * np);
            return -1;
        }
        if (c == 0) {
            if (day_max < ts[i])
                day_max = ts[i];
            continue;
        }
        return srt[i * np + 1] == mi[i * np + 1] ? 1 : 2;
    }
    return 0;
}

/* cnvCheckKm1(), cnv.cpp:65-167 (complete graph, m_DayIdx[d] == d) */
static int or_ks_km1(or_ks *k, const uint8_t *tr)
{
    const int np = k->np;
    int ret = 1, day = 0;
    uint8_t ttr[OR_NPMAX];
    if (!k->tr_ind && !k->n_aut) {
        or_ks_add_aut(k, k->R);   /* updateGroup(result()): round 0 is the identity */
        day = 1;
    }
    for (; day < k->nrows; day++) {
        const uint8_t *t = tr;
        if (day) {
            const uint8_t *resn = k->R + day * np;
            for (int i = np; i--;)
                ttr[resn[i]] = tr[i];
            t = ttr;
        }
        k->cand++;
        int icmp = or_ks_process(k, t);
        if (icmp == 0) {
            or_ks_add_aut(k, t);
            continue;
        }
        if (icmp < 0) {
            ret = -1;
            if (k->full)
                continue;
            break;
        }
    }
    return ret;
}

/* cnvCheckKm(), cnv.cpp:168-185 */
static int or_ks_km(or_ks *k, const uint8_t *a, const uint8_t *tg)
{
    uint8_t trmk[OR_NPMAX];
    for (int i = 0; i < k->ng; i++)
        for (int j = 0; j < k->g; j++)
            trmk[i * k->g + j] = (uint8_t)(a[i] + k->groups[tg[i] * k->g + j]);
    int ret = or_ks_km1(k, trmk) >= 0;
    k->tr_ind++;
    return ret;
}

/* cnvCheckTgNew(), cnv.cpp:186-210 */
static int or_ks_tg(or_ks *k, const uint8_t *a)
{
    uint8_t tg[OR_NPMAX];
    int ret = 1;
    memset(tg, 0, k->ng);
    for (;;) {
        if (!or_ks_km(k, a, tg)) {
            ret = 0;
            if (!k->full)
                break;
        }
        int i = k->ng;
        while (i-- && ++tg[i] >= k->gfact)
            tg[i] = 0;
        if (i < 0)
            break;
    }
    return ret;
}

int or_ksys_test(const uint8_t *R, int nrows, int np, int g, int full_aut, or_ksys_result *res)
{
    if (np > OR_NPMAX || g < 2 || g > 4 || np % g || nrows < 1 || nrows > np)
        return -1;
    or_ks k;
    memset(&k, 0, sizeof(k));
    k.np = np;
    k.g = g;
    k.ng = np / g;
    k.nrows = nrows;
    k.R = R;
    k.full = full_aut;
    k.arena = res->aut_arena;
    k.cap = res->aut_cap;
    /* cnvInit(): the g! in-group orders in odometer order */
    int gf = 1;
    for (int i = 2; i <= g; i++)
        gf *= i;
    k.gfact = gf;
    for (int i = 0; i < g; i++)
        k.groups[i] = (uint8_t)i;
    for (int p = 1; p < gf; p++) {
        uint8_t *cur = k.groups + p * g;
        memcpy(cur, cur - g, g);
        for (;;) {
            int j = g;
            while (cur[--j] >= g - 1)
                cur[j] = 0;
            cur[j]++;
            int ok = 1;
            unsigned m = 0;
            for (int q = 0; q < g; q++) {
                if (m & (1u << cur[q]))
                    ok = 0;
                m |= 1u << cur[q];
            }
            if (ok)
                break;
        }
    }
    /* cnvCheckNew(), cnv.cpp:211-217 */
    k.player_index = nrows * np - g - 1;

    /* canonizator(), cnv.cpp:271-316: Heap's permutations of the groups */
    uint8_t a[OR_NPMAX + 1], p[OR_NPMAX + 1];
    memset(a, 0, sizeof(a));
    memset(p, 0, sizeof(p));
    int ng = k.ng, ret = 1;
    for (int i = ng; i--;) {
        p[i] = (uint8_t)i;
        a[i] = (uint8_t)(i * g);
    }
    if (!or_ks_tg(&k, a))
        ret = 0;
    if (ret || k.full) {
        p[ng] = (uint8_t)ng;
        int i = 1;
        while (i < ng) {
            p[i]--;
            int j = (i % 2) ? p[i] : 0;
            uint8_t t = a[i];
            a[i] = a[j];
            a[j] = t;
            if (!or_ks_tg(&k, a)) {
                ret = 0;
                if (!k.full)
                    break;
            }
            i = 0;
            while (!p[++i])
                p[i] = (uint8_t)i;
        }
    }
    res->canonical = ret;
    res->player_index = k.player_index;
    res->n_aut = k.n_aut;
    res->aut_overflow = k.overflow;
    res->candidates = k.cand;
    return 0;
}

/* =====================================================================
 * Seeded generators
 * ===================================================================== */
uint64_t or_splitmix64(uint64_t *s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static uint32_t or_rand_below(uint64_t *s, uint32_t n)
{
    return (uint32_t)(((or_splitmix64(s) >> 32) * (uint64_t)n) >> 32);
}

/* Stinson's hill-climbing for STS(v) (D. R. Stinson, "Hill-climbing algorithms
 * for the construction of combinatorial designs", Ann. Discrete Math. 26, 1985):
 * pick a live point x and two points y, z not yet paired with x; if {y,z} is
 * uncovered add {x,y,z}, otherwise replace the block through {y,z} by {x,y,z}. */
static int or_sts_hillclimb_stream(int v, uint64_t *sp, uint8_t *blocks)
{
    const int b = v * (v - 1) / 6;
    int8_t cov[32][32];
    memset(cov, -1, sizeof(cov));
    int nb = 0, steps = 0;
    uint64_t s = *sp;
    while (nb < b) {
        steps++;
        int x;
        int cand[32], nc;
        for (;;) {
            x = (int)or_rand_below(&s, (uint32_t)v);
            nc = 0;
            for (int y = 0; y < v; y++)
                if (y != x && cov[x][y] < 0)
                    cand[nc++] = y;
            if (nc >= 2)
                break;
        }
        int iy = (int)or_rand_below(&s, (uint32_t)nc);
        int iz = (int)or_rand_below(&s, (uint32_t)(nc - 1));
        if (iz >= iy)
            iz++;
        int y = cand[iy], z = cand[iz];
        int slot = cov[y][z];
        if (slot < 0) {
            slot = nb++;
        } else {
            uint8_t *B = blocks + slot * 3;
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++)
                    if (i != j)
                        cov[B[i]][B[j]] = -1;
        }
        uint8_t *B = blocks + slot * 3;
        B[0] = (uint8_t)x;
        B[1] = (uint8_t)y;
        B[2] = (uint8_t)z;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
                if (i != j)
                    cov[B[i]][B[j]] = (int8_t)slot;
    }
    *sp = s;
    return steps;
}

int or_sts_hillclimb(int v, uint64_t seed, uint8_t *blocks)
{
    uint64_t s = seed;
    return or_sts_hillclimb_stream(v, &s, blocks);
}

/* item `index` of a seeded STS(v) batch: hill-climbing on the item's stream,
 * then Fisher-Yates row and column permutations from the same stream; row r is
 * point prow[r], column c is block pcol[c]; rows[r] bit c = incidence */
void or_sts_random_rows(int v, uint64_t seed, uint64_t index, uint64_t *rows)
{
    const int b = v * (v - 1) / 6;
    uint64_t s = seed ^ (index * 0xD1B54A32D192ED03ull);
    uint8_t blocks[64 * 3], prow[32], pcol[64], rowof[32];
    or_sts_hillclimb_stream(v, &s, blocks);
    for (int i = 0; i < v; i++)
        prow[i] = (uint8_t)i;
    for (int i = 0; i < b; i++)
        pcol[i] = (uint8_t)i;
    for (int k = v - 1; k >= 1; k--) {
        int j = (int)or_rand_below(&s, (uint32_t)(k + 1));
        uint8_t t = prow[k];
        prow[k] = prow[j];
        prow[j] = t;
    }
    for (int k = b - 1; k >= 1; k--) {
        int j = (int)or_rand_below(&s, (uint32_t)(k + 1));
        uint8_t t = pcol[k];
        pcol[k] = pcol[j];
        pcol[j] = t;
    }
    for (int r = 0; r < v; r++)
        rowof[prow[r]] = (uint8_t)r;
    for (int r = 0; r < v; r++)
        rows[r] = 0;
    for (int c = 0; c < b; c++)
        for (int a = 0; a < 3; a++)
            rows[rowof[blocks[pcol[c] * 3 + a]]] |= 1ull << c;
}

/* =====================================================================
 * Orderly enumerators (known-answer pins for the checkers).
 * ===================================================================== */
typedef struct {
    int v, b, r, k, lambda;
    uint8_t M[64 * OR_BMAX];
    uint8_t colw[OR_BMAX];
    or_design_cb cb;
    void *user;
    long found;
    uint64_t checks;
} or_benum;

static void or_benum_row(or_benum *e, int n);

/* choose how many 1s go into each orbit of level n (a row solution over the
 * column orbits, as CRowSolution holds them), then canonicity-check the rows */
static void or_benum_fill(or_benum *e, int n, const or_orbits *o, int q, int left, int *x)
{
    const int b = e->b;
    if (q == o->n) {
        if (left)
            return;
        /* intersections with the previous rows */
        uint8_t *row = e->M + n * b;
        memset(row, 0, b);
        for (int t = 0; t < o->n; t++)
            memset(row + o->start[t], 1, x[t]);
        for (int i = 0; i < n; i++) {
            int c = 0;
            for (int col = 0; col < b; col++)
                c += row[col] & e->M[i * b + col];
            if (c != e->lambda)
                return;
        }
        /* column weights must still be completable */
        for (int col = 0; col < b; col++) {
            int w = e->colw[col] + row[col];
            if (w > e->k || e->k - w > e->v - n - 1)
                return;
        }
        for (int col = 0; col < b; col++)
            e->colw[col] += row[col];
        or_bibd_result res;
        memset(&res, 0, sizeof(res));
        const int complete = n + 1 == e->v;
        e->checks++;
        or_bibd_test(e->M, n + 1, b, complete ? (OR_SAVE_ROW_PERM | OR_SAVE_ROW_TO_CHANGE) : 0, 0,
                     &res);
        if (res.canonical) {
            if (complete) {
                e->found++;
                if (e->cb)
                    e->cb(e->user, e->M, e->v, b, res.aut_lo, res.aut_hi);
            } else {
                or_benum_row(e, n + 1);
            }
        }
        for (int col = 0; col < b; col++)
            e->colw[col] -= row[col];
        return;
    }
    /* orbit q: columns share the pattern of rows 0..n-1 and hence the weight */
    const int w = e->colw[o->start[q]];
    int maxx = o->len[q];
    if (w >= e->k)
        maxx = 0;
    if (maxx > left)
        maxx = left;
    /* columns that need every remaining row are forced */
    int minx = (e->k - w == e->v - n) ? o->len[q] : 0;
    for (int xv = maxx; xv >= minx; xv--) {
        x[q] = xv;
        or_benum_fill(e, n, o, q + 1, left - xv, x);
    }
}

static void or_benum_row(or_benum *e, int n)
{
    or_orbits o;
    or_level_orbits(e->M, n, e->b, &o);
    int x[OR_BMAX];
    or_benum_fill(e, n, &o, 0, e->r, x);
}

long or_bibd_enumerate(int v, int b, int r, int k, int lambda, or_design_cb cb, void *user,
                       uint64_t *n_checks)
{
    if (v > 64 || b > OR_BMAX)
        return -1;
    or_benum *e = (or_benum *)calloc(1, sizeof(or_benum));
    e->v = v;
    e->b = b;
    e->r = r;
    e->k = k;
    e->lambda = lambda;
    e->cb = cb;
    e->user = user;
    /* row 0 is forced: r ones first */
    memset(e->M, 1, r);
    for (int c = 0; c < r; c++)
        e->colw[c] = 1;
    or_benum_row(e, 1);
    long f = e->found;
    if (n_checks)
        *n_checks = e->checks;
    free(e);
    return f;
}

typedef struct {
    int n;
    uint8_t R[OR_NPMAX * OR_NPMAX];
    uint8_t used[OR_NPMAX][OR_NPMAX];
    or_design_cb cb;
    void *user;
    long found;
    uint64_t checks;
} or_kenum;

static void or_kenum_round(or_kenum *e, int d);

/* build round d as a perfect matching of unused pairs, groups in increasing
 * order of their first player; player 0 is paired with d+1 (rounds sorted by
 * their second entry, as every canonical matrix is) */
static void or_kenum_match(or_kenum *e, int d, uint8_t *row, int pos, unsigned taken)
{
    const int n = e->n;
    if (pos == n) {
        e->checks++;
        or_ksys_result res;
        memset(&res, 0, sizeof(res));
        if (d >= 1) {
            or_ksys_test(e->R, d + 1, n, 2, 0, &res);
            if (!res.canonical)
                return;
        }
        if (d + 1 == n - 1) {
            e->found++;
            if (e->cb)
                e->cb(e->user, e->R, n - 1, n, res.n_aut, 0);
            return;
        }
        or_kenum_round(e, d + 1);
        return;
    }
    int a = 0;
    while (taken & (1u << a))
        a++;
    for (int c = a + 1; c < n; c++) {
        if ((taken & (1u << c)) || e->used[a][c])
            continue;
        if (a == 0 && c != d + 1)
            continue;
        row[pos] = (uint8_t)a;
        row[pos + 1] = (uint8_t)c;
        e->used[a][c] = e->used[c][a] = 1;
        or_kenum_match(e, d, row, pos + 2, taken | (1u << a) | (1u << c));
        e->used[a][c] = e->used[c][a] = 0;
    }
}

static void or_kenum_round(or_kenum *e, int d)
{
    or_kenum_match(e, d, e->R + d * e->n, 0, 0);
}

long or_ksys_enumerate(int n, or_design_cb cb, void *user, uint64_t *n_checks)
{
    if (n > 32 || n % 2)
        return -1;
    or_kenum *e = (or_kenum *)calloc(1, sizeof(or_kenum));
    e->n = n;
    e->cb = cb;
    e->user = user;
    for (int i = 0; i < n; i++)
        e->R[i] = (uint8_t)i;
    for (int i = 0; i < n; i += 2)
        e->used[i][i + 1] = e->used[i + 1][i] = 1;
    or_kenum_round(e, 1);
    long f = e->found;
    if (n_checks)
        *n_checks = e->checks;
    free(e);
    return f;
}
