// canon_ctx.h -- the context behind the C ABI's opaque canon_ctx handle.
#pragma once
#include <map>
#include <string>
#include <vector>

#include "../../include/canon_gb300.h"
#include "canon_internal.h"

struct canon_ctx {
    int device = 0;
    int num_sms = 0;
    canon_cfg cfg{};
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // queued host input (pinned)
    canon::Item *h_bitems = nullptr, *h_kitems = nullptr;
    uint64_t *h_words = nullptr;
    uint8_t *h_bytes = nullptr;
    uint32_t n_bitems = 0, n_kitems = 0, n_words = 0, n_bytes = 0;
    uint32_t max_bytes = 0;
    // what the queued batches need, kept at submit so that canon_sync reads no item:
    // widest incidence shape, whether every incidence item takes the two-pass check,
    // whether any item stores automorphisms
    uint32_t q_max_b = 0, q_max_v = 0;
    bool q_two_pass = true, q_want_auts = false;
    // the queued input is copied to the GPU at submit; a call that borrows the device
    // staging in between (canon_canonize_bibd) makes canon_sync copy it all again
    bool q_reupload = false;
    // k-system items queued: widest players and filled rounds (the segmented check's size)
    uint32_t q_ks_np = 0, q_ks_nr = 0;
    // queued k-systems with groups of 3 or 4 (a queue of their own), the most relabelings of one
    bool q_ks_groups = false;
    uint64_t q_ks_total = 0;
    // candidates per warp task of the k-system check (canon_set_ksys_segment):
    // 0 = chosen per launch, CANON_KSYS_WHOLE = one warp per matrix
    uint32_t ksys_seg = 0;
    canon::KsysSeg *d_kseg = nullptr;
    size_t kseg_cap = 0;
    // the captured k-system enumeration (canon_levels.cu) and its level capacity
    void *ksys_graph = nullptr;
    uint64_t ksys_graph_cap = 1ull << 16;
    // device buffers
    canon::Item *d_bitems = nullptr, *d_kitems = nullptr;
    uint64_t *d_words = nullptr;
    uint8_t *d_bytes = nullptr;
    unsigned *d_ticket = nullptr;      // work-stealing counters (2 words)
    unsigned *d_tc_err = nullptr;      // raised when a tensor-core forward pass gave up waiting
    canon::Outputs d_out{}, h_out{};
    std::vector<uint8_t> item_kind;   // per out_idx
    // learned order: installed weights (device) and lazily grown scratch
    bool order_on = false;
    float *d_mlp = nullptr;            // flat FP32 parameters (canon::mlp::N_PARAMS)
    uint16_t *d_w1 = nullptr, *d_w2 = nullptr, *d_w2t = nullptr, *d_w3 = nullptr;   // BF16 copies
    float *d_adam_m = nullptr, *d_adam_v = nullptr, *d_grad = nullptr, *d_loss = nullptr;
    void *d_scratch = nullptr;
    size_t scratch_bytes = 0;
    uint64_t *d_orders = nullptr;
    size_t d_orders_bytes = 0;
    // autotuned check variant per (v, b, flags) (canon_tune_bibd), and the split
    // variant's scratch
    std::map<uint32_t, int> tuned;
    canon::SplitPart *d_split_parts = nullptr;
    unsigned *d_split_stop = nullptr;
    size_t split_cap = 0;              // matrices x rows the scratch holds
    std::string err;
    float last_ms = 0.f;
    uint64_t launches = 0;
};

namespace canon {
// candidates per warp task for a k-system check of n items of np players and
// `rounds` rounds (0 = one warp per matrix)
uint32_t ksys_segment(const canon_ctx *c, uint64_t n, uint32_t np, uint32_t rounds);
uint32_t kgen_segment(const canon_ctx *c, uint64_t n, uint64_t total);
// the largest batch of matrices of `words` 64-bit words (BIBD) or `bytes` bytes
// (k-systems) each that one canon_submit_* call can queue on an empty context
uint32_t batch_capacity(const canon_ctx *c, uint32_t words, uint32_t bytes);
// frees the captured k-system enumeration of a context
void ksys_graph_release(canon_ctx *c);
}  // namespace canon
