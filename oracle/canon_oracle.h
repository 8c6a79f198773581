/*
 * canon_oracle.h -- CPU oracle for the canonicity-check hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * checker (andrei5055/Incidence-System-Enumeration) used as the parity checker
 * for the CUDA path.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it; the product library never links or calls it.
 *
 * Every function cites the reference file:line it follows.
 */
#ifndef CANON_ORACLE_H
#define CANON_ORACLE_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OR_EMAX 255u   /* ELEMENT_MAX, GroupOrder.h:9 */
#define OR_IMAX 254u   /* IDX_MAX,     GroupOrder.h:22 */

/* outInfo flags, Source/CanonicityChecker.h:27-32 */
#define OR_SAVE_NOTHING      0u
#define OR_SAVE_ROW_PERM     1u
#define OR_SAVE_ROW_TO_CHANGE 4u
/* Extension (no counterpart in the reference's TestCanonicity): keep searching
 * past a rejection (treated like a "greater" prune) so that |Aut| is also
 * known for non-canonical matrices. */
#define OR_FULL_AUT          0x100u
/* t_outRowPermute (designParam.h): keep every row automorphism of a complete
 * matrix in the PermutStorage arena (after the identity in slot 0). */
#define OR_SAVE_AUT_ROWS     0x200u

typedef struct {
    uint64_t trials;      /* permutations tried (next_permutation calls that returned a row) */
    uint64_t rows;        /* row comparisons (row x orbit loop entries) */
    uint64_t orbits;      /* column-orbit comparisons */
    uint64_t auts;        /* automorphisms found */
} or_stats;

typedef struct {
    int      canonical;       /* 1 = canonical */
    int      reject_row;      /* nRow at the first diff<0 (-1 if canonical) */
    int      row_to_change;   /* rowToChange(nRow) (CanonicityChecker.cpp:320-330), -1 if canonical */
    uint8_t  witness[64];     /* permRow() at rejection (first rejecting permutation) */
    uint64_t aut_lo, aut_hi;  /* |Aut| (row-permutation group order), 128 bit */
    int      n_perm;          /* permutations in the PermutStorage arena (slot 0 = identity) */
    int      len_perm;        /* lenPerm() of the arena */
    uint8_t *perm_arena;      /* caller buffer, n_perm*len_perm bytes (may be NULL) */
    int      perm_cap;        /* capacity of perm_arena in permutations */
    int      perm_overflow;   /* 1 if more permutations were produced than perm_cap */
    or_stats st;
} or_bibd_result;

/* ---- GroupOrder.h restatement (exposed for cross-checks against the reference) ---- */
typedef struct {
    unsigned stab;      /* m_nStabLength    (ushort) */
    unsigned stab_aut;  /* m_nStabLengthAut (ushort) */
    unsigned __int128 order;
} or_group;

uint8_t or_next_permutation(or_group *g, uint8_t *perm, const uint8_t *orb, uint8_t n,
                            uint8_t idx, uint8_t len_stab);
void or_add_automorphism(or_group *g, unsigned degree, const uint8_t *perm, uint8_t *orb,
                         int row_permut, int calc_group_order);
void or_update_group_order(or_group *g, unsigned degree, const uint8_t *orb);
/* substitute another implementation of the three functions above (same
 * signatures); NULL restores the restatement */
void or_set_group_impl(void *np_fn, void *aa_fn, void *ugo_fn);

/* ---- BIBD (rank-2 incidence matrix) checker ---- */
/* M: nrows x b bytes, row-major 0/1, columns in normal form (every row 1s-first
 * inside each column orbit of the rows above it).  Returns 0 on success, <0 on
 * invalid input. */
int or_bibd_is_normal(const uint8_t *M, int nrows, int b);
void or_bibd_normalize(uint8_t *M, int nrows, int b);        /* GenerateBinaryColumnOrbits rows 0..n-1 */
int or_bibd_test(const uint8_t *M, int nrows, int b, unsigned out_info, int len_stab,
                 or_bibd_result *res);
/* CanonizeMatrix(k=0): M is overwritten with the canonical form; returns the number of
 * TestCanonicity calls; res holds the final (canonical) call's result. */
int or_bibd_canonize(uint8_t *M, int nrows, int b, or_bibd_result *res);

/* ---- k-system (rows = rounds, numPlayers bytes each, groups of size g) ---- */
typedef struct {
    int      canonical;
    int      player_index;    /* m_playerIndex after the check (backjump position) */
    uint64_t n_aut;           /* orderOfGroup() */
    uint8_t *aut_arena;       /* caller buffer for automorphisms (sorted set), n_aut*np bytes */
    int      aut_cap;
    int      aut_overflow;
    uint64_t candidates;      /* relabelings compared */
} or_ksys_result;

int or_ksys_test(const uint8_t *R, int nrows, int np, int g, int full_aut, or_ksys_result *res);

/* runCanonizer() (Source/CDTools.cpp:5-52): the canonical binary matrix of a k-system
 * of np players in groups of k, its first day_numb rounds (<= 0: all); R holds the
 * rounds as result() does.  out: np x b bytes (b = day_numb * np / k, returned);
 * class_steps (optional): canonisations of the class loop.  <0 on invalid input. */
int or_ksys_binary_canonize(const uint8_t *R, int np, int k, int day_numb, uint8_t *out, long *class_steps);

/* ---- enumerators used to pin the oracle on the reference's known answers ---- */
typedef void (*or_design_cb)(void *user, const uint8_t *M, int v, int b, uint64_t aut_lo, uint64_t aut_hi);
/* orderly row-by-row generation of all BIBD(v,b,r,k,lambda); returns #canonical designs */
long or_bibd_enumerate(int v, int b, int r, int k, int lambda, or_design_cb cb, void *user,
                       uint64_t *n_checks);
/* all 1-factorizations of K_n (n even), rounds = n-1, canonical under cnvCheckNew */
long or_ksys_enumerate(int n, or_design_cb cb, void *user, uint64_t *n_checks);

/* ---- seeded generators (same streams as the product's data generator) ---- */
uint64_t or_splitmix64(uint64_t *state);
/* random STS(v) by Stinson's hill-climbing; blocks out[b*3]; returns #steps */
int or_sts_hillclimb(int v, uint64_t seed, uint8_t *blocks);
/* item `index` of a seeded batch: random STS(v) + random row/column permutation,
 * rows[r] bit c = incidence (the product's device generator draws the same stream) */
void or_sts_random_rows(int v, uint64_t seed, uint64_t index, uint64_t *rows);

#ifdef __cplusplus
}
#endif
#endif
