/*
 * canon_gb300.h -- C ABI of the GB300 canonicity-check engine.
 *
 * Drop-in for the canonicity test of andrei5055/Incidence-System-Enumeration:
 *   - CCanonicityChecker<T,S>::TestCanonicity()      Source/CanonicityChecker.h:58,255-586
 *     (callers Source/Enumerator.cpp:364 complete, :446-447 partial,
 *      Source/MatrixCanonChecker.cpp:456 canonize)
 *   - CMatrixCanonChecker::CanonizeMatrix()          Source/MatrixCanonChecker.cpp:420-564
 *   - alldata::cnvCheckNew()                         k-Factorization/TripleSys/Source/cnv.cpp:211-351
 *     (caller k-Factorization/TripleSys/Source/checkCurrentResult.cpp:91)
 *   - the GPU seam TestCanonicityOnGPU() / CGPU_CanonChecker   Source/Enumerator.h:220-228,
 *     Source/MatrixCanonChecker.h:204-350, Source/CanonicityChecker.cu:123-156
 * Results are written in the reference's layouts: the witness is permRow(),
 * the automorphisms of partial matrices are permutations of column orbits laid
 * out as CPermutStorage (Source/PermutStorage.h:8-110: numPerm x lenPerm
 * bytes, slot 0 the identity), k-system automorphisms as CGroupInfo entries
 * (k-Factorization/TripleSys/Include/groupInfo.h:121-125).
 *
 * Ownership: input batches are caller-owned host memory, read during the
 * submit call.  Results live in library-owned pinned buffers and stay valid
 * until the next canon_sync() or canon_destroy() on the same context.
 * Errors: every call returns a CANON_* status; nothing calls exit().
 * Threading: one context per host thread; a context owns one CUDA stream.
 */
#ifndef CANON_GB300_H
#define CANON_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define CANON_OK        0
#define CANON_EINVAL   -1   /* bad argument or malformed matrix */
#define CANON_ENOMEM   -2   /* allocation failed / capacity exceeded */
#define CANON_ECUDA    -3   /* CUDA runtime error */
#define CANON_ETIMEOUT -4   /* a search hit its trial budget (per-item status says which) */
#define CANON_ENODEV   -5   /* no usable GPU */
#define CANON_ESIZE    -6   /* batch larger than CANON_NOALLOC_MAX_ITEMS (canon_check_bibd_noalloc) */

/* ---- per-item status bits (canon_results.status[i]) ---- */
#define CANON_ST_OK        0u
#define CANON_ST_BADINPUT  1u   /* matrix not in the required form */
#define CANON_ST_TIMEOUT   2u   /* trial budget exhausted: verdict invalid */
#define CANON_ST_PERM_OVF  4u   /* automorphism arena too small: list truncated */

/* ---- batch flags ---- */
/* Complete matrix: TestCanonicity(v, .., t_saveRowPermutations | t_saveRowToChange)
 * (Enumerator.cpp:696): witness permRow(), rowToChange() and |Aut| are reported.
 * Without it the check is the partial one, t_saveNothing (Enumerator.cpp:446-447);
 * |Aut| of the partial matrix is still reported (an addition). */
#define CANON_COMPLETE    0x1u
/* Input rows are an arbitrary 0/1 matrix: bring the columns into the orbit
 * normal form first (GenerateBinaryColumnOrbits, MatrixCanonChecker.cpp:186-263).
 * Without it the matrix must already be in normal form (as the enumerator
 * builds it, MatrixCanonChecker.cpp:14-93). */
#define CANON_RAW         0x2u
/* Keep searching after the first rejection (treated like a "greater" prune) so
 * that |Aut| is also reported for non-canonical matrices.  No counterpart in the
 * reference's BIBD checker; the k-system analogue is m_doNotExitEarlyIfNotCanonical
 * (cnv.cpp:159-160). */
#define CANON_FULL_AUT    0x4u
/* Store automorphisms: column-orbit permutations for partial BIBD checks
 * (CanonicityChecker.h:427-451), every row automorphism for complete ones
 * (t_outRowPermute), relabelings for k-systems (updateGroup, cnv.cpp:127-133). */
#define CANON_SAVE_AUTS   0x8u
/* Complete matrices only: |Aut| of a rejected matrix is taken from its canonical
 * form, reached the way CanonizeMatrix() does (MatrixCanonChecker.cpp:420-496:
 * move the rows as the witness says, renormalise the columns, check again until
 * canonical).  The flag, witness and row_to_change stay those of the first check.
 * Much cheaper than CANON_FULL_AUT on non-canonical matrices. */
#define CANON_AUT_CANON   0x10u
/* Run the check in the reference's own search order throughout (next_permutation()
 * with its orbit pruning), so that canon_results.trials equals the number of
 * permutations the reference tries.  Without it (and without CANON_SAVE_AUTS, which
 * implies it) the verdict and |Aut| come from a lex-max search over the same tree
 * and only the witness is taken from the reference order: every output except
 * `trials` is identical, and the check is several times faster. */
#define CANON_REFERENCE_ORDER 0x20u
/* Only the canonical flag (and |Aut| of canonical matrices) is wanted, as in an
 * enumerator that keeps the canonical matrices of a level: a matrix that the
 * lex-max search rejects gets no witness search, so witness, reject_row and
 * row_to_change are undefined for it (trials counts the short search only).
 * Ignored with CANON_SAVE_AUTS or CANON_REFERENCE_ORDER. */
#define CANON_VERDICT_ONLY 0x40u

/* ---- context ---- */
typedef struct canon_ctx canon_ctx;

typedef struct {
    int      device;          /* CUDA device ordinal */
    uint32_t max_items;       /* capacity: matrices per sync (0 = 1<<21) */
    uint32_t max_words;       /* capacity: 64-bit input words per sync (0 = 16*max_items) */
    uint32_t aut_cap;         /* automorphisms kept per matrix when CANON_SAVE_AUTS (0 = 64) */
    uint64_t max_trials;      /* per-matrix trial budget (0 = 1<<28) */
    uint32_t options;         /* CANON_OPT_* bits (0 = none) */
} canon_cfg;

/* canon_enumerate_bibd prunes the children of every parent with the parent's
 * automorphisms (the grouping of row solutions by CRowSolution::sortSolutionsByGroup(),
 * Source/RowSolution.h:325-383): the same designs from fewer candidates, at the price of
 * one automorphism search per parent of the shallow levels, whose latency outweighs the
 * saving on the families measured; hence an option. */
#define CANON_OPT_AUT_PRUNE 0x1u
/* canon_sync copies back only `canonical` and `status`, the two arrays a caller that
 * keeps the canonical matrices of a level reads (Enumerator.cpp:446-447 keeps a
 * partial matrix when TestCanonicity() returns true): 2 bytes per item instead of
 * 51.  The other result arrays are not updated and their contents are undefined. */
#define CANON_OPT_VERDICT_SYNC 0x2u
/* canon_enumerate_ksys runs level by level with host-sized launches (reading every
 * level's size back) instead of replaying its captured CUDA graph.  Same output. */
#define CANON_OPT_NO_GRAPH 0x4u
/* The MLP's GEMMs (forward, the hidden-layer gradient, the weight gradients) run on the
 * warp-level mma.sync and FP32 paths instead of tcgen05 (the results agree to BF16
 * rounding of the operands). */
#define CANON_OPT_MLP_WARP_MMA 0x8u

/* BIBD / incidence-system batch: n matrices of b columns (b <= 63), v rows each
 * (v <= 16), row j of matrix i at rows[i*v + j] with bit c = column c.
 * nrows[i] (optional, NULL = all v) is the number of filled rows of matrix i. */
typedef struct {
    uint32_t        n;
    uint32_t        v;
    uint32_t        b;
    uint32_t        flags;
    const uint64_t *rows;
    const uint8_t  *nrows;
} canon_bibd_batch;

/* k-system batch (group size 2): n matrices of np players (np <= 12, even),
 * `rounds` rounds each, round j of matrix i at data[(i*rounds + j)*np ..]
 * as the reference's result() rows (pairs ascending, ordered by first player,
 * round 0 = 0 1 2 .. np-1).  nrows[i] (optional) = rounds filled. */
typedef struct {
    uint32_t       n;
    uint32_t       np;
    uint32_t       rounds;
    uint32_t       flags;
    const uint8_t *data;
    const uint8_t *nrows;
} canon_ksys_batch;

/* Results of every batch submitted since the previous sync, in submission
 * order (BIBD and k-system items share one index space). */
typedef struct {
    uint32_t        n;              /* items */
    const uint8_t  *canonical;      /* [n] 1 = canonical */
    const uint8_t  *status;         /* [n] CANON_ST_* bits */
    const uint8_t  *reject_row;     /* [n] BIBD: nRow of the first diff<0 (255 if canonical) */
    const uint8_t  *row_to_change;  /* [n] BIBD: rowToChange(); k-sys: 255 */
    const int32_t  *player_index;   /* [n] k-sys: m_playerIndex; BIBD: -1 */
    const uint8_t  *witness;        /* [n*16] permRow() at rejection (BIBD), 0xFF-filled if canonical */
    const uint64_t *aut;            /* [2n] |Aut| as (lo, hi) pairs */
    const uint64_t *trials;         /* [n] permutations / relabelings tried */
    const uint16_t *n_auts;         /* [n] automorphisms stored (CANON_SAVE_AUTS) incl. slot 0 */
    const uint8_t  *len_aut;        /* [n] bytes per stored automorphism */
    const uint8_t  *auts;           /* [n*aut_cap*64] arena, item i at i*aut_cap*64 */
    uint32_t        aut_cap;
    float           kernel_ms;      /* device time of the check kernels (CUDA events) */
} canon_results;

/* Learned search order: BF16 MLP 64 -> H -> H -> 1.  NULL weights = plain order. */
typedef struct {
    uint32_t        in_dim;         /* 64 */
    uint32_t        hidden;         /* 128 */
    const uint16_t *w1, *w2, *w3;   /* bf16, row-major [out][in] */
    const float    *b1, *b2, *b3;
} canon_mlp_weights;

/* Creates a context on cfg->device.  Replaces the per-thread CGPU_CanonChecker
 * set-up (MatrixCanonChecker.h:204-247, CanonicityChecker.cu:17-67). */
canon_ctx *canon_create(const canon_cfg *cfg);
void       canon_destroy(canon_ctx *ctx);
const char *canon_last_error(const canon_ctx *ctx);

/* Queue a batch of incidence matrices: one TestCanonicity() per matrix. */
int canon_submit_bibd(canon_ctx *ctx, const canon_bibd_batch *batch);
/* Queue a batch of k-system matrices: one cnvCheckNew(0, nrows) per matrix. */
int canon_submit_ksys(canon_ctx *ctx, const canon_ksys_batch *batch);
/* Queue a batch of k-system matrices with groups of group_size players: one
 * cnvCheckNew(0, nrows) per matrix on the reference's general path (kmProcessMatrix,
 * k-Factorization/TripleSys/Source/kmSupport.cpp:220-313), e.g. Kirkman triple systems.
 * group_size 2 is canon_submit_ksys; 3 and 4 take np <= 16 players (a multiple of the
 * group size, 2 groups at least), rounds as result() rows (players ascending inside a
 * group, groups ordered by first player, round 0 = 0 1 .. np-1).  Every relabeling,
 * (np/g)! * (g!)^(np/g) per round, is tried on the GPU.  Outputs as for group size 2;
 * with CANON_SAVE_AUTS the automorphisms of a canonical matrix are stored as a sorted set
 * (none for a rejected one; beyond aut_cap, CANON_ST_PERM_OVF and aut_cap of them, not
 * necessarily the first in the reference's order).  Such batches form a queue of their
 * own: no incidence or group-size-2 batch may be queued with them before canon_sync. */
int canon_submit_ksys_groups(canon_ctx *ctx, const canon_ksys_batch *batch, uint32_t group_size);
/* Copy the queued input to the GPU, run the checks, wait, expose the results. */
int canon_sync(canon_ctx *ctx, canon_results *out);
/* Work split of the k-system check (cnvCheckNew): the candidates of a matrix
 * (ng! * 2^ng * rounds relabelings) are cut into segments of `cands` candidates
 * (rounded up to a multiple of 32) that different warps take, so that a batch of a
 * few hundred matrices fills the GPU.  0 (the default) chooses the segment per launch
 * from the batch size; CANON_KSYS_WHOLE keeps one warp per matrix.  Every output is
 * the same either way.  Batches that store automorphisms (CANON_SAVE_AUTS) and mixed
 * batches always run one warp per matrix. */
#define CANON_KSYS_WHOLE 0xFFFFFFFFu
int canon_set_ksys_segment(canon_ctx *ctx, uint32_t cands);
/* Install (or with NULL remove) the learned ordering network. */
int canon_set_ordering(canon_ctx *ctx, const canon_mlp_weights *w);

/* CanonizeMatrix(k = 0) for a batch of complete incidence matrices, in place on
 * host memory (rows as in canon_bibd_batch, all v rows filled).  aut_out[2n]
 * (optional) receives |Aut|.  MatrixCanonChecker.cpp:420-564. */
int canon_canonize_bibd(canon_ctx *ctx, uint32_t n, uint32_t v, uint32_t b, uint64_t *rows,
                        uint64_t *aut_out);

/* ---- device-resident entry points (inputs already in HBM) ---- */
/* Same check as canon_submit_bibd + canon_sync for device pointers, all items
 * with v rows; launched on `stream` (a cudaStream_t, NULL = the context's).
 * Output arrays are device pointers (any may be NULL except canonical).
 * flags: CANON_COMPLETE, CANON_RAW, CANON_FULL_AUT, CANON_AUT_CANON, CANON_REFERENCE_ORDER,
 * CANON_VERDICT_ONLY.  A variant kept by canon_tune_bibd for (v, b, flags) is used. */
int canon_check_bibd_device(canon_ctx *ctx, uint32_t n, uint32_t v, uint32_t b, uint32_t flags,
                            const uint64_t *d_rows, uint8_t *d_canonical, uint8_t *d_witness16,
                            uint64_t *d_aut, uint8_t *d_status, uint64_t *d_trials, void *stream);
/* Seeded STS(v) batch on the device (Stinson hill-climbing + uniform row and
 * column permutations); if canon_odd, odd items are replaced by their
 * canonical form.  rows: device pointer [n*v]. */
/* ---- autotuning per design shape ----
 * Times the check variants that give identical outputs for (v, b, flags) on n
 * device-resident matrices, verifies them against the one-pass variant and keeps
 * the fastest for later canon_check_bibd_device calls with the same (v, b, flags)
 * on this context (without a learned order):
 *   CANON_VARIANT_SINGLE   one pass: short reference-order search, lex-max search
 *                          when it does not decide;
 *   CANON_VARIANT_TWO_PASS lex-max pass for all, witness pass for the rejected
 *                          (not with CANON_SAVE_AUTS / CANON_REFERENCE_ORDER);
 *   CANON_VARIANT_SPLIT    the lex-max search split over one thread per (matrix,
 *                          first row) (CANON_VERDICT_ONLY without |Aut| flags);
 *   CANON_VARIANT_CONVERGED two passes, the lex-max pass laid out so that the
 *                          threads of a warp evaluate their nodes together (one
 *                          pass over all columns per node and thread), its column
 *                          loads staged 4 columns ahead;
 *   CANON_VARIANT_CONVERGED_D2 / _D8 the same with the loads staged 2 / 8 columns
 *                          ahead (the shared-memory staging depth; 15 x 35 shapes).
 * ms[i]: the variant's device time, -1 when it does not apply, -2 when its
 * outputs differed (never chosen). */
#define CANON_VARIANT_SINGLE    0
#define CANON_VARIANT_TWO_PASS  1
#define CANON_VARIANT_SPLIT     2
#define CANON_VARIANT_CONVERGED 3
#define CANON_VARIANT_CONVERGED_D2 4
#define CANON_VARIANT_CONVERGED_D8 5
typedef struct {
    int   variant;      /* the variant kept */
    float ms[6];
} canon_tune_result;
int canon_tune_bibd(canon_ctx *ctx, uint32_t n, uint32_t v, uint32_t b, uint32_t flags, const uint64_t *d_rows,
                    canon_tune_result *out);
int canon_generate_sts_device(canon_ctx *ctx, uint32_t n, uint32_t v, uint64_t seed, int canon_odd,
                              uint64_t *d_rows, void *stream);
/* ---- measurement ----
 * Lex-max nodes visited per matrix by the search of the resident check's first pass
 * (its verdict and |Aut|), for n device-resident matrices: the work measure of the
 * check's integer roofline.  d_orders (optional, n device words): the first-row order
 * of every matrix, nibble-packed (nibble q = the row tried q-th); without it the
 * search runs in the learned order when one is installed (canon_set_ordering), as
 * canon_check_bibd_device runs it, else in the plain order.  d_nodes: n device words. */
int canon_lexmax_nodes_bibd(canon_ctx *ctx, uint32_t n, uint32_t v, uint32_t b, uint32_t flags,
                            const uint64_t *d_rows, uint64_t *d_nodes, const uint64_t *d_orders);
/* 32-bit integer lane operations per second that this GPU sustains on independent
 * XOR / ADD / shift chains (the peak of the check's integer roofline). */
int canon_measure_int_peak(canon_ctx *ctx, double *lane_ops_per_s);
/* Device memory helpers so callers without a CUDA toolchain can hold batches in HBM. */
void *canon_device_alloc(canon_ctx *ctx, size_t bytes);
int   canon_device_free(canon_ctx *ctx, void *p);
int   canon_memcpy_d2h(canon_ctx *ctx, void *dst, const void *src, size_t bytes);
int   canon_memcpy_h2d(canon_ctx *ctx, void *dst, const void *src, size_t bytes);
/* Device time (ms, CUDA events on the launching stream) of the last kernel issued by
 * canon_check_bibd_device / canon_sync. */
float canon_last_kernel_ms(const canon_ctx *ctx);
/* Number of kernels this context launched since creation. */
uint64_t canon_kernel_launches(const canon_ctx *ctx);
int canon_stream_sync(canon_ctx *ctx);

/* ---- frontier-batched orderly enumeration (the callers of the check) ---- */
typedef struct {
    uint64_t checks;      /* matrices checked on the GPU */
    uint64_t designs;     /* canonical complete matrices */
    uint32_t levels;      /* rows / rounds added */
    uint32_t batches;     /* canon_sync calls */
    double   seconds;     /* wall time */
    double   kernel_ms;   /* device time of the checks */
    /* per level: matrices with l+1 rows (rounds) checked, and their device time;
     * level_checks[v-1] counts the complete matrices constructed */
    uint64_t level_checks[16];
    double   level_kernel_ms[16];
    double   gen_seconds; /* time spent generating the candidates (host wall time, or
                             device time of the generation kernels) */
    uint64_t trials;      /* k-systems: relabelings tried by all checks (cnvCheckNew candidates) */
    double   level_gen_ms[16]; /* BIBDs and groups of 3 or 4: per level, the wall time of generating its candidates */
} canon_enum_stats;

/* Called for every canonical complete matrix: BIBD rows as rows x uint64 (cast to
 * bytes), k-systems as rows x cols bytes in result() form; |Aut| as (lo, hi). */
typedef void (*canon_design_cb)(void *user, const uint8_t *matrix, uint32_t rows, uint32_t cols,
                                uint64_t aut_lo, uint64_t aut_hi);

/* All BIBD(v, b, r, k, lambda) up to isomorphism by orderly generation, level by
 * level, every level's partial matrices checked in batches on the GPU: the work of
 * CEnumerator::Enumerate() with C_InSysEnumerator/CBIBD_Enumerator
 * (Source/Enumerator.cpp:540-1024; checks at :446-447 and :364).  v <= 16, b <= 63. */
int canon_enumerate_bibd(canon_ctx *ctx, uint32_t v, uint32_t b, uint32_t r, uint32_t k, uint32_t lambda,
                         canon_design_cb cb, void *user, canon_enum_stats *stats);
/* All 1-factorizations of K_np up to isomorphism, round by round with every level in
 * HBM: the next rounds of all canonical parents are generated on the GPU (the round
 * construction of processOneDay()/getNextPlayer(), k-Factorization/TripleSys/Source/
 * TripleSys.cpp:487-775), checked there and the canonical ones kept: the work of
 * alldata::Run() for group size 2 with the check at every level (TripleSys.cpp:80-775,
 * check at checkCurrentResult.cpp:91).  np even, <= 12. */
int canon_enumerate_ksys(canon_ctx *ctx, uint32_t np, canon_design_cb cb, void *user, canon_enum_stats *stats);
/* All k-systems of np players in groups of g = 3 or 4 with (np - 1) / (g - 1) rounds
 * (resolvable designs with blocks of g, e.g. the Kirkman triple systems of 15 players)
 * up to isomorphism, by orderly generation: the next rounds of every canonical parent are
 * built on the host cores (every partition into groups that repeats no pair, in result()
 * form, ordered by second entry), checked in batches on the GPU (canon_submit_ksys_groups)
 * and the canonical ones kept: alldata::Run() for group size 3 or 4 with the check at
 * every level (k-Factorization/TripleSys/Source/TripleSys.cpp:80-775).  g = 2 is
 * canon_enumerate_ksys.  np <= 16; the context's queue must be empty. */
int canon_enumerate_ksys_groups(canon_ctx *ctx, uint32_t np, uint32_t g, canon_design_cb cb, void *user,
                                canon_enum_stats *stats);

/* ---- seeded inputs of an uneven batched check ----
 * n partial BIBD(v, b, r, k, lambda) incidence matrices made by random backtracking of
 * their rows, as an orderly enumerator meets them (the row constraints of
 * C_InSysEnumerator's row solutions, Source/Enumerator.cpp:726-975, with MakeRow,
 * Source/MatrixCanonChecker.cpp:14-93, drawn at random): item i has nrows[i] rows,
 * uniform in [min_rows, max_rows]; each row has weight r, lambda columns in common
 * with every earlier row, no column above k ones and no column left unable to reach
 * k ones with the rows below.  A level without an admissible row drops the row above
 * and draws it again, so dead ends that no complete design extends are included.
 * A Steiner triple system (k = 3, lambda = 1) with v-1 or v rows filled is a complete
 * design (v-1 admissible rows determine the last), which row-by-row backtracking
 * reaches only rarely: such items, and any whose search budget runs out, are the
 * first rows of a complete random STS(v) (Stinson's hill-climbing, uniform row and
 * column permutation); *n_from_complete (optional) counts them.
 * rows: n*v words (unfilled rows 0), bit c = column c.  Item i uses its own random
 * stream (seed, i); the work is spread over the host cores.  CANON_ETIMEOUT if an
 * item's search budget ran out (its nrows is then 0).  Host only. */
int canon_generate_partial_bibd(uint32_t v, uint32_t b, uint32_t r, uint32_t k, uint32_t lambda, uint32_t n,
                                uint64_t seed, uint32_t min_rows, uint32_t max_rows, uint64_t *rows,
                                uint8_t *nrows, uint32_t *n_from_complete);
/* n partial 1-factorizations of K_np (np even, <= 12), the same way round by round:
 * round 0 is (0 1)(2 3)..., every further round a random perfect matching of pairs not
 * used before, in result() form (pairs ascending, ordered by first player), the
 * rounds ordered by the partner of player 0.  data: n*(np-1)*np bytes, item i's round d at (i*(np-1) + d)*np. */
int canon_generate_partial_ksys(uint32_t np, uint32_t n, uint64_t seed, uint32_t min_rounds, uint32_t max_rounds,
                                uint8_t *data, uint8_t *nrows);

/* ---- the canonical binary matrix of k-systems (the reference's plugin) ----
 * createCanonizer / runCanonizer / releaseCanonizer replace the reference's exported
 * plugin of the same names and signatures (k-Factorization/Utils/Include/CDTools.h:9-11,
 * Source/CDTools.cpp:5-52).  runCanonizer() writes the first iDay rounds of a k-system
 * (all numDays = (v-1)/(k-1) rounds when iDay <= 0; rounds as result() holds them) as a
 * binary matrix -- one column per group of each day, row p = player p
 * (convertToBinaryMatrix, Source/matrix.h:198-209) -- and returns its canonical form,
 * the matrix CanonizeMatrix(k, NULL, numClasses) converges to
 * (Source/MatrixCanonChecker.cpp:420-564): the lexicographically greatest matrix over
 * permutations of the players, of the groups inside each day and, when all days are
 * given, of the days.  v rows of iDay*v/k bytes, owned by the canonizer and valid until
 * its next call; NULL on error.  Group size k = 2, 3 or 4, v <= 16 a multiple of k with
 * (v-1) a multiple of k-1 and at least 3 groups a day (k = 2: v even, 6 <= v <= 16;
 * k = 3: v = 9 or 15; k = 4: v = 16); the canonizer holds a context on GPU 0.  Not
 * thread-safe per canonizer (as the reference's). */
void *createCanonizer(int v, int k);
void releaseCanonizer(void *pCanonizer);
const unsigned char *runCanonizer(void *pCanonizer, const unsigned char *pMatrix, int k, int iDay);
/* The same for n k-systems at once: data = n x days x np bytes (host), out = n x np x
 * (days*np/2) bytes (host), aut_out[n] (optional) = the number of player labelings that
 * reach the canonical form (the order of its automorphism group).  One GPU thread per
 * k-system. */
int canon_canonize_ksys_binary(canon_ctx *ctx, uint32_t n, uint32_t np, uint32_t days, const uint8_t *data,
                               uint8_t *out, uint64_t *aut_out);
/* The same with groups of k = 2, 3 or 4 players (out = n x np x (days*np/k) bytes); the
 * shapes createCanonizer takes. */
int canon_canonize_ksys_binary_groups(canon_ctx *ctx, uint32_t n, uint32_t np, uint32_t k, uint32_t days,
                                      const uint8_t *data, uint8_t *out, uint64_t *aut_out);

/* ---- result tables (the reference's text output of a finished run) ----
 * Per complete design: simple[i] = no two equal columns (no replicated blocks) and
 * transitive[i] = Aut(D) transitive on the points, the properties that the
 * reference counts as Ns and Ndt (CGroupsInfo, Source/GroupsInfo.h:4-11; the
 * transitivity test groupIsTransitive(), Source/CanonicityChecker.cpp:292-304).
 * Transitivity comes from the lex-max search on the GPU: the rows that start a
 * labeling reaching the canonical form form one orbit of Aut(D).  Host rows
 * (n*v words); either output may be NULL. */
int canon_design_properties(canon_ctx *ctx, uint32_t n, uint32_t v, uint32_t b, const uint64_t *rows,
                            uint8_t *simple, uint8_t *transitive);
/* The |Aut(D)| table that closes a BIBD run (CGroupsInfo::printGroupInfo,
 * Source/GroupsInfo.cpp:72-150, in the layout of Results/BIBDs/V = v/<v>_<k>_<l>.txt):
 * one line per group order with Nd / Ns / Ndt / Nst, the totals and the run's
 * counters.  aut[i] = |Aut| of design i; simple / transitive may be NULL (all 0).
 * Host only.  Writes at most cap bytes including the final 0 and returns the full
 * length (snprintf convention). */
size_t canon_report_bibd(uint32_t v, uint32_t b, uint32_t r, uint32_t k, uint32_t lambda, uint32_t n,
                         const uint64_t *aut, const uint8_t *simple, const uint8_t *transitive,
                         uint64_t fully_constructed, double seconds, char *buf, size_t cap);
/* The cycle descriptor of one k-system matrix (alldata::matrixStatOutput,
 * k-Factorization/TripleSys/Source/p1fCheck.cpp:499-515, without its "Cycles:"
 * prefix): for every pair of rounds the cycle lengths of their union, the cycle
 * sets in increasing order, each as "count(l1:l2:...) ".  rounds x np bytes in
 * result() form.  Host only; snprintf convention. */
size_t canon_ksys_cycles(uint32_t np, uint32_t rounds, const uint8_t *matrix, char *buf, size_t cap);
/* The |Aut(M)| x cycles table of a k-system run (MatrixDB::printRecord and
 * DescrStorage::reportResult, k-Factorization/TripleSys/Include/MatrixDB.h, in the
 * layout of K_Results.txt, without its time stamp): n matrices of rounds x np
 * bytes, aut[i] = |Aut(M)|.  Host only; snprintf convention. */
size_t canon_report_ksys(uint32_t np, uint32_t rounds, uint32_t n, const uint8_t *matrices, const uint64_t *aut,
                         char *buf, size_t cap);

/* ---- the learned search order (no counterpart in the reference) ----
 * A BF16 MLP 64 -> 128 -> 128 -> 1 (ReLU) scores each row of a matrix as the first
 * row of the labeling that reaches its canonical form.  With weights installed by
 * canon_set_ordering, canon_check_bibd_device tries the rows at the first level of
 * the lex-max search in decreasing score; verdicts, |Aut| and witnesses do not
 * change, only the search order.  Parameters travel as one flat FP32 vector of
 * CANON_MLP_PARAMS floats: w1[128][64] | b1[128] | w2[128][128] | b2[128] | w3[128] | b3. */
#define CANON_MLP_PARAMS (128 * 64 + 128 + 128 * 128 + 128 + 128 + 1)
/* 64 BF16 features of every row of n device-resident matrices (d_feat: n*v*64 BF16). */
int canon_mlp_features(canon_ctx *ctx, uint32_t n, uint32_t v, uint32_t b, const uint64_t *d_rows, void *d_feat);
/* Training labels from the exact search: for every matrix the rows that start a
 * labeling reaching its canonical form (bit x of d_first_rows[i]), and the number
 * of lex-max nodes visited (d_nodes, optional) in the order given by d_orders
 * (optional, n nibble-packed orders; NULL = plain). */
int canon_label_first_rows(canon_ctx *ctx, uint32_t n, uint32_t v, uint32_t b, uint32_t flags, const uint64_t *d_rows,
                           uint16_t *d_first_rows, uint64_t *d_nodes, const uint64_t *d_orders);
/* Logits of n feature rows (device) under `params` (host, CANON_MLP_PARAMS floats). */
int canon_mlp_forward(canon_ctx *ctx, uint64_t n, const void *d_x, const float *params, float *d_logits);
/* Gradient of the mean binary cross-entropy over n rows (labels 0/1, device) with
 * respect to `params`, into grad (host, CANON_MLP_PARAMS floats); loss (host) = the mean. */
int canon_mlp_grad(canon_ctx *ctx, uint64_t n, const void *d_x, const float *d_labels, const float *params,
                   float *grad, float *loss);
/* Adam training (lr, batches of `batch` rows, `epochs` passes) of params in place
 * (host); epoch_loss (host, optional) gets the mean loss of every epoch. */
int canon_mlp_train(canon_ctx *ctx, uint64_t n, const void *d_x, const float *d_labels, uint32_t epochs,
                    uint32_t batch, float lr, float *params, float *epoch_loss);

/* ---- checking without allocating ---- */
/* Device output arrays of canon_check_bibd_noalloc (one entry per matrix, same
 * meaning as the canon_results fields).  auts may be NULL unless CANON_SAVE_AUTS
 * is set, in which case it holds aut_cap*64 bytes per matrix. */
typedef struct {
    uint8_t  *canonical;
    uint8_t  *status;
    uint8_t  *reject_row;
    uint8_t  *row_to_change;
    int32_t  *player_index;
    uint8_t  *witness;      /* 16 bytes per matrix */
    uint64_t *aut;          /* (lo, hi) per matrix */
    uint64_t *trials;
    uint16_t *n_auts;
    uint8_t  *len_aut;
    uint8_t  *auts;
    uint32_t  aut_cap;
} canon_device_outputs;

#define CANON_NOALLOC_MAX_ITEMS 65536u

/* The batched TestCanonicity() check of canon_submit_bibd + canon_sync for
 * device-resident matrices, for callers that cannot call cudaMalloc: a host
 * application whose device memory belongs to another allocator or pool (a
 * framework's caching allocator, a fixed arena sized at start-up), or a latency
 * path where the implicit device synchronisation of cudaMalloc/cudaFree is not
 * acceptable.  It needs no context and allocates nothing: its scratch (one
 * 16-byte work descriptor per matrix and a work counter) is a static device
 * array of 1 MiB + 256 bytes that every GPU loading this library holds until
 * the process exits.  Hence at most CANON_NOALLOC_MAX_ITEMS matrices per call;
 * larger batches are refused with CANON_ESIZE.  Rows and per-matrix filled-row
 * counts (d_nrows, NULL = all v) are device pointers laid out as in
 * canon_bibd_batch; `out` holds device pointers.  Launched on `stream`
 * (a cudaStream_t, NULL = the default stream) and not waited for.
 * Unlike canon_submit_bibd, which refuses a whole batch with CANON_EINVAL when a
 * filled-row count is 0 or above v, the counts are only read on the GPU here: such
 * a matrix gets status CANON_ST_BADINPUT (canonical 0) and the others are checked.
 * The first call on a device looks up the scratch's device address (once per
 * device, with that device current), so make that first call before any stream
 * capture.  All calls share the one scratch array: calls whose work overlaps on
 * the GPU race, so issue them on one stream or wait in between.  The work
 * counter is cleared by every call.  max_trials 0 = 1<<28.
 * No counterpart in the reference. */
int canon_check_bibd_noalloc(uint32_t n, uint32_t v, uint32_t b, uint32_t flags, const uint64_t *d_rows,
                             const uint8_t *d_nrows, const canon_device_outputs *out, uint64_t max_trials,
                             void *stream);

#ifdef __cplusplus
}
#endif
#endif /* CANON_GB300_H */
