// canon_internal.h -- shared definitions of the device kernels and the C-ABI layer.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace canon {

constexpr unsigned VMAX = 16;        // rows of an incidence matrix (nibble-packed permutations)
constexpr unsigned BMAX = 63;        // columns (one uint64 per row, bit b is the orbit sentinel)
constexpr unsigned KS_NPMAX = 12;    // k-system players (group size 2, <= 6 groups)
constexpr unsigned EMAX = 255;       // ELEMENT_MAX
constexpr unsigned IMAX = 254;       // IDX_MAX

// one work item: a matrix to check (16 bytes)
struct Item {
    uint32_t data_off;   // BIBD: offset in uint64 words; k-sys: offset in bytes
    uint8_t  kind;       // 0 = BIBD, 1 = k-system
    uint8_t  nrows;      // rows / rounds filled
    uint8_t  ncols;      // b / numPlayers
    uint8_t  flags;      // CANON_* batch flags
    uint32_t out_idx;    // output slot
    uint32_t pad;
};

enum : uint8_t { KIND_BIBD = 0, KIND_KSYS = 1 };

// structure-of-arrays outputs, all indexed by Item::out_idx
struct Outputs {
    uint8_t  *canonical;
    uint8_t  *status;
    uint8_t  *reject_row;
    uint8_t  *row_to_change;
    int32_t  *player_index;
    uint8_t  *witness;      // 16 bytes per item
    uint64_t *aut;          // 2 per item
    uint64_t *trials;
    uint16_t *n_auts;
    uint8_t  *len_aut;
    uint8_t  *auts;         // aut_cap * 64 bytes per item
    uint32_t  aut_cap;
};

// flags (same values as the public CANON_* flags)
constexpr uint32_t F_COMPLETE = 0x1, F_RAW = 0x2, F_FULL_AUT = 0x4, F_SAVE_AUTS = 0x8, F_AUT_CANON = 0x10,
                   F_REFERENCE_ORDER = 0x20, F_VERDICT_ONLY = 0x40;
constexpr uint8_t ST_BADINPUT = 1, ST_TIMEOUT = 2, ST_PERM_OVF = 4;

// launchers (stream-ordered; return cudaGetLastError())
// d_ticket: one device word of scratch (the work-stealing counter), reset by the launcher
cudaError_t launch_bibd_check(const Item *d_items, uint32_t n_items, const uint64_t *d_words,
                              Outputs out, uint64_t max_trials, unsigned *d_ticket, int num_sms,
                              cudaStream_t s);
// the same check in two passes (lex-max search for all, witness for the rejected) for items that all
// want |Aut| (CANON_AUT_CANON or CANON_FULL_AUT) without the reference order; d_ticket: two words
cudaError_t launch_bibd_check_two_pass(const Item *d_items, uint32_t n_items, const uint64_t *d_words,
                                       Outputs out, uint64_t max_trials, unsigned *d_ticket, int num_sms,
                                       cudaStream_t s, uint32_t max_b = 63, uint32_t max_v = 16);
cudaError_t launch_bibd_check_uniform(uint32_t n, uint32_t v, uint32_t b, uint32_t flags,
                                      const uint64_t *d_rows, uint8_t *d_canonical,
                                      uint8_t *d_witness16, uint64_t *d_aut, uint8_t *d_status,
                                      uint64_t *d_trials, uint64_t max_trials, unsigned *d_ticket,
                                      int num_sms, cudaStream_t s, const uint64_t *d_orders = nullptr,
                                      int variant = -1);
// check variants with identical outputs (canon_tune_bibd): one pass, two passes,
// the search split by first row (verdict only), two passes with the first pass in
// the converged layout (canon_bibd_conv.cuh)
enum : int {
    VARIANT_SINGLE = 0,
    VARIANT_TWO_PASS = 1,
    VARIANT_SPLIT = 2,
    VARIANT_CONVERGED = 3,
    VARIANT_CONVERGED_D2 = 4,   // the converged pass staging its column loads 2 (8) columns ahead
    VARIANT_CONVERGED_D8 = 5,
    N_VARIANTS = 6
};
// one share of a lex-max search split by first row (bibd_split_kernel)
struct SplitPart {
    uint64_t leaves;
    uint8_t orbit0, improved, status, orbit1, pad[4];
};
// levels of the split search for n matrices of v rows: 2 (threads per matrix and
// first two rows) while n * v * v <= 2^20 and v >= 3, else 1
inline uint32_t split_levels(uint64_t n, uint32_t v) { return (v >= 3 && n * v * v <= (1ull << 20)) ? 2u : 1u; }
// verdict (and |Aut| of the canonical) of n matrices with v rows, one thread per
// (matrix, first row[, second row]); d_parts: n*v*v parts (n*v when one level),
// d_stop: n words of scratch.  Outputs other than the flag, |Aut| and status are
// not produced.
cudaError_t launch_bibd_check_split(uint32_t n, uint32_t v, uint32_t b, uint32_t flags, const uint64_t *d_rows,
                                    uint8_t *d_canonical, uint64_t *d_aut, uint8_t *d_status, SplitPart *d_parts,
                                    unsigned *d_stop, uint64_t max_trials, unsigned *d_ticket, int num_sms,
                                    cudaStream_t s);
cudaError_t launch_bibd_labels(uint32_t n, uint32_t v, uint32_t b, uint32_t flags, const uint64_t *d_rows,
                               uint16_t *d_first_rows, uint64_t *d_nodes, const uint64_t *d_orders,
                               uint64_t max_nodes, unsigned *d_ticket, int num_sms, cudaStream_t s);
// per-matrix node counts of the lex-max pass of the resident check (the search of
// bibd_max_kernel, same tree): the work measure of the check's integer roofline
cudaError_t launch_bibd_lexmax_nodes(uint32_t n, uint32_t v, uint32_t b, uint32_t flags, const uint64_t *d_rows,
                                     uint64_t *d_nodes, uint64_t max_nodes, unsigned *d_ticket, int num_sms,
                                     cudaStream_t s, const uint64_t *d_orders = nullptr);
// automorphisms (row permutations, nibble-packed) of n canonical matrices, at most gcap
// each: d_gens n*gcap words, d_ngens n bytes
cudaError_t launch_bibd_autgen(uint32_t n, uint32_t v, uint32_t b, const uint64_t *d_rows, uint64_t *d_gens,
                               uint8_t *d_ngens, uint32_t gcap, uint64_t max_nodes, unsigned *d_ticket,
                               int num_sms, cudaStream_t s);
// integer-pipe throughput probe: *ops = 32-bit lane operations of the launch
cudaError_t launch_int_peak(uint32_t iters, int num_sms, uint32_t *d_sink, cudaStream_t s, uint64_t *ops);
// order of the rows as first-row candidates by decreasing score (scores: n x v floats)
cudaError_t launch_order_by_score(uint32_t n, uint32_t v, const float *d_scores, uint64_t *d_orders,
                                  cudaStream_t s);

namespace mlp {
// flat FP32 parameter vector: w1[128][64] | b1[128] | w2[128][128] | b2[128] | w3[128] | b3[1]
constexpr int N_PARAMS = 128 * 64 + 128 + 128 * 128 + 128 + 128 + 1;
cudaError_t forward(long n, const void *x, const void *w1, const float *b1, const void *w2, const float *b2,
                    const void *w3, const float *b3, float *y, void *h1, void *h2, int num_sms, cudaStream_t s);
// the same forward pass on tcgen05 (x 16-byte aligned); *err is raised if a wait for
// the tensor cores timed out
cudaError_t forward_tc(long n, const void *x, const void *w1, const float *b1, const void *w2, const float *b2,
                       const void *w3, const float *b3, float *y, void *h1, void *h2, unsigned *err, int num_sms,
                       cudaStream_t s);
// the backward pass with dH1 = dH2 W2 on tcgen05 (h1, h2, dh1, dh2 16-byte aligned)
cudaError_t backward_tc(long n, const float *logit, const float *label, const void *h1, const void *h2,
                        const void *w3, const void *w2t, float *dy, float *dh2, float *dh1, float *loss,
                        unsigned *err, int num_sms, cudaStream_t s);
cudaError_t backward(long n, const float *logit, const float *label, const void *h1, const void *h2,
                     const void *w3, const void *w2t, float *dy, float *dh2, float *dh1, float *loss,
                     int num_sms, cudaStream_t s);
cudaError_t weight_grads(long n, const float *dh1, const float *dh2, const float *dy, const void *x,
                         const void *h1, const void *h2, float *grad, int num_sms, cudaStream_t s);
// the same weight gradients as GEMMs over the batch rows on tcgen05 (dh1, dh2 16-byte aligned)
cudaError_t weight_grads_tc(long n, const float *dh1, const float *dh2, const float *dy, const void *x,
                            const void *h1, const void *h2, float *grad, unsigned *err, int num_sms,
                            cudaStream_t s);
cudaError_t adam(int count, float *p, const float *grad, float *m, float *v, float lr, int step, void *w1,
                 void *w2, void *w2t, void *w3, cudaStream_t s);
cudaError_t features(uint32_t n, uint32_t v, uint32_t b, uint32_t flags, const uint64_t *rows, void *feat,
                     cudaStream_t s);
}  // namespace mlp
cudaError_t launch_bibd_canonize(uint32_t n, uint32_t v, uint32_t b, uint64_t *d_rows,
                                 uint64_t *d_aut, uint8_t *d_status, uint32_t stride_items,
                                 uint32_t first_item, uint64_t max_trials, unsigned *d_ticket,
                                 int num_sms, cudaStream_t s);
// check of a device-resident batch with the scratch in static device memory (no allocation)
cudaError_t launch_bibd_check_noalloc(uint32_t n, uint32_t v, uint32_t b, uint32_t flags,
                                      const uint64_t *d_rows, const uint8_t *d_nrows, Outputs out,
                                      uint64_t max_trials, cudaStream_t s);
cudaError_t launch_sts_generate(uint32_t n, uint32_t v, uint64_t seed, uint64_t *d_rows,
                                int num_sms, cudaStream_t s);
cudaError_t launch_ksys_check(const Item *d_items, uint32_t n_items, const uint8_t *d_bytes,
                              Outputs out, unsigned *d_ticket, int num_sms, cudaStream_t s);
// one persistent launch over a mixed batch: k-system items (warp each) then incidence items (thread each);
// d_ticket: two device words
// (max_b, max_v: the widest incidence item, which sizes the per-thread state)
cudaError_t launch_mixed_check(const Item *d_bitems, uint32_t nb, const Item *d_kitems, uint32_t nk,
                               const uint64_t *d_words, const uint8_t *d_bytes, Outputs out,
                               uint64_t max_trials, unsigned *d_ticket, int num_sms, cudaStream_t s,
                               uint32_t max_b = 63, uint32_t max_v = 16);
cudaError_t ksys_upload_tables();
// per-item state of the segmented k-system check: the first rejection as
// (candidate << 32 | player index), all ones while none; automorphisms counted;
// ill-formed rounds
struct KsysSeg {
    unsigned long long key;
    unsigned n_aut;
    unsigned bad;
};
// the k-system check with every item's candidates split into segments of seg_cands
// (a multiple of 32; 0 = chosen on the device by ksys_auto_segment) taken by different
// warps; d_state holds n_items + 1 entries (the last is the work counter); total_max =
// the most candidates of any item; d_n (optional) = the item count in device memory
// (at most n_items).  Automorphisms are not stored.
cudaError_t launch_ksys_check_split(const Item *d_items, uint32_t n_items, const uint8_t *d_bytes, Outputs out,
                                   uint32_t seg_cands, uint64_t total_max, KsysSeg *d_state, int num_sms,
                                   cudaStream_t s, const uint64_t *d_n = nullptr);
// the check of k-systems with groups of 3 or 4 (np <= 16; Item::pad holds the group
// size), split into segments of seg_cands relabelings over warps; automorphisms are stored
// (CANON_SAVE_AUTS) for canonical matrices, unordered (canon_sync sorts them)
cudaError_t launch_kgen_check(const Item *d_items, uint32_t n_items, const uint8_t *d_bytes, Outputs out,
                              uint32_t seg_cands, uint64_t total_max, KsysSeg *d_state, int num_sms,
                              cudaStream_t s);
// relabelings of one check with groups of g: (np/g)! * (g!)^(np/g) * rounds
inline uint64_t kgen_candidates(uint32_t np, uint32_t g, uint32_t rounds) {
    uint64_t t = 1, gf = 1;
    for (uint32_t i = 2; i <= g; ++i)
        gf *= i;
    for (uint32_t i = 2; i <= np / g; ++i)
        t *= i;
    for (uint32_t i = 0; i < np / g; ++i)
        t *= gf;
    return t * rounds;
}
// warps of the segmented k-system kernel resident on one SM (128-thread blocks)
constexpr uint32_t KSYS_RESIDENT_WARPS_PER_SM = 64;
// Candidates per segment for n items of at most `total` candidates each: about 8
// warp tasks per resident warp, segments of at least 256 candidates (fewer cost more
// in set-up, the rounds' tables, than they spread); a segment that covers the whole
// item is one warp per matrix.  The same rule on the host and on the device.
__host__ __device__ inline uint32_t ksys_auto_segment(uint64_t n, uint64_t total, uint32_t resident_warps) {
    uint64_t seg = total * n / (8ull * (resident_warps ? resident_warps : 1));
    seg &= ~31ull;
    if (seg < 256)
        seg = 256;
    const uint64_t whole = (total + 31) & ~31ull;
    return (uint32_t)(seg < whole ? seg : whole);
}
// candidates of one k-system check: ng! * 2^ng * rounds
inline uint64_t ksys_candidates(uint32_t np, uint32_t rounds) {
    uint64_t f = 1;
    for (uint32_t i = 2; i <= np / 2; ++i)
        f *= i;
    return (f << (np / 2)) * rounds;
}

}  // namespace canon
