// canon_api.cu -- the C ABI (include/canon_gb300.h) over the sm_103a kernels.
//
// A context owns one CUDA stream, pinned host staging for queued batches and
// device buffers sized at creation.  canon_submit_* appends a batch to the host
// staging (on host threads) and queues its copy to the GPU at once, so the copy
// of one batch runs while the next is packed; canon_sync launches the check
// kernels on the context's stream, copies the result arrays back and waits.  This
// replaces CGPU_CanonChecker (Source/MatrixCanonChecker.h:204-350), which
// marshalled one C++ checker object per matrix onto the device heap and launched
// TestCanonicity<<<1, nMatr>>> (Source/CanonicityChecker.cu:152-156).
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <string>
#include <vector>

#include "../../include/canon_gb300.h"
#include "canon_internal.h"
#include "canon_ctx.h"
#include "canon_hostpool.h"
#include "canon_pack.h"

using canon::Item;
using canon::Outputs;


namespace {

int fail(canon_ctx *c, int code, const std::string &msg) {
    if (c)
        c->err = msg;
    return code;
}

int cuda_fail(canon_ctx *c, cudaError_t e, const char *what) {
    return fail(c, CANON_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename T>
cudaError_t dev_alloc(T **p, size_t count) {
    return cudaMalloc((void **)p, count * sizeof(T) + 16);
}
template <typename T>
cudaError_t host_alloc(T **p, size_t count) {
    return cudaMallocHost((void **)p, count * sizeof(T) + 16);
}

cudaError_t alloc_outputs(Outputs &o, size_t n, uint32_t aut_cap, bool device) {
    o.aut_cap = aut_cap;
    cudaError_t e;
#define CANON_ALLOC(field, count)                                               \
    e = device ? dev_alloc(&o.field, (count)) : host_alloc(&o.field, (count)); \
    if (e != cudaSuccess)                                                       \
        return e;
    CANON_ALLOC(canonical, n)
    CANON_ALLOC(status, n)
    CANON_ALLOC(reject_row, n)
    CANON_ALLOC(row_to_change, n)
    CANON_ALLOC(player_index, n)
    CANON_ALLOC(witness, n * 16)
    CANON_ALLOC(aut, n * 2)
    CANON_ALLOC(trials, n)
    CANON_ALLOC(n_auts, n)
    CANON_ALLOC(len_aut, n)
    CANON_ALLOC(auts, n * (size_t)aut_cap * 64)
#undef CANON_ALLOC
    return cudaSuccess;
}

void free_outputs(Outputs &o, bool device) {
    void *ptrs[] = {o.canonical, o.status, o.reject_row, o.row_to_change, o.player_index, o.witness,
                    o.aut,       o.trials, o.n_auts,     o.len_aut,       o.auts};
    for (void *p : ptrs)
        if (p)
            device ? cudaFree(p) : cudaFreeHost(p);
    o = Outputs{};
}

uint16_t to_bf16(float f) {
    // round to nearest even (NaN kept quiet)
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7F800000u) == 0x7F800000u && (u & 0x7FFFFFu))
        return (uint16_t)((u >> 16) | 0x40u);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

constexpr int P_W1 = 0, P_B1 = 128 * 64, P_W2 = P_B1 + 128, P_B2 = P_W2 + 128 * 128, P_W3 = P_B2 + 128,
              P_B3 = P_W3 + 128;

cudaError_t ensure_mlp(canon_ctx *c) {
    if (c->d_mlp)
        return cudaSuccess;
    cudaError_t e = dev_alloc(&c->d_mlp, canon::mlp::N_PARAMS);
    if (e == cudaSuccess)
        e = dev_alloc(&c->d_w1, 128 * 64);
    if (e == cudaSuccess)
        e = dev_alloc(&c->d_w2, 128 * 128);
    if (e == cudaSuccess)
        e = dev_alloc(&c->d_w2t, 128 * 128);
    if (e == cudaSuccess)
        e = dev_alloc(&c->d_w3, 128);
    if (e == cudaSuccess)
        e = dev_alloc(&c->d_adam_m, canon::mlp::N_PARAMS);
    if (e == cudaSuccess)
        e = dev_alloc(&c->d_adam_v, canon::mlp::N_PARAMS);
    if (e == cudaSuccess)
        e = dev_alloc(&c->d_grad, canon::mlp::N_PARAMS);
    if (e == cudaSuccess)
        e = dev_alloc(&c->d_loss, 1);
    return e;
}

// upload flat FP32 parameters and their BF16 copies (W2 also transposed)
cudaError_t upload_params(canon_ctx *c, const float *p) {
    cudaError_t e = ensure_mlp(c);
    if (e != cudaSuccess)
        return e;
    std::vector<uint16_t> w1(128 * 64), w2(128 * 128), w2t(128 * 128), w3(128);
    for (int i = 0; i < 128 * 64; ++i)
        w1[i] = to_bf16(p[P_W1 + i]);
    for (int o = 0; o < 128; ++o)
        for (int i = 0; i < 128; ++i) {
            w2[o * 128 + i] = to_bf16(p[P_W2 + o * 128 + i]);
            w2t[i * 128 + o] = w2[o * 128 + i];
        }
    for (int i = 0; i < 128; ++i)
        w3[i] = to_bf16(p[P_W3 + i]);
    cudaStream_t s = c->stream;
    cudaMemcpyAsync(c->d_mlp, p, canon::mlp::N_PARAMS * 4, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(c->d_w1, w1.data(), w1.size() * 2, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(c->d_w2, w2.data(), w2.size() * 2, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(c->d_w2t, w2t.data(), w2t.size() * 2, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(c->d_w3, w3.data(), w3.size() * 2, cudaMemcpyHostToDevice, s);
    return cudaStreamSynchronize(s);
}

cudaError_t ensure_scratch(canon_ctx *c, size_t bytes) {
    if (c->scratch_bytes >= bytes)
        return cudaSuccess;
    if (c->d_scratch)
        cudaFree(c->d_scratch);
    c->d_scratch = nullptr;
    c->scratch_bytes = 0;
    cudaError_t e = cudaMalloc(&c->d_scratch, bytes);
    if (e == cudaSuccess)
        c->scratch_bytes = bytes;
    return e;
}

// the forward pass of the installed weights: on tcgen05 (at least one 128-row tile,
// 16-byte aligned rows), or the warp-level mma.sync path (CANON_OPT_MLP_WARP_MMA,
// fewer rows, or unaligned buffers)
cudaError_t mlp_forward_installed(canon_ctx *c, long n, const void *x, float *y, void *h1, void *h2, cudaStream_t s) {
    const auto a16 = [](const void *p) { return ((uintptr_t)p & 15u) == 0; };
    if (!(c->cfg.options & CANON_OPT_MLP_WARP_MMA) && c->d_tc_err && n >= 128 && a16(x) && a16(h1) && a16(h2))
        return canon::mlp::forward_tc(n, x, c->d_w1, c->d_mlp + P_B1, c->d_w2, c->d_mlp + P_B2, c->d_w3,
                                      c->d_mlp + P_B3, y, h1, h2, c->d_tc_err, c->num_sms, s);
    return canon::mlp::forward(n, x, c->d_w1, c->d_mlp + P_B1, c->d_w2, c->d_mlp + P_B2, c->d_w3, c->d_mlp + P_B3, y,
                               h1, h2, c->num_sms, s);
}

// after the stream is synchronised: did a tensor-core forward pass give up waiting?
// (the flag is cleared)
bool tc_timed_out(canon_ctx *c) {
    if (!c->d_tc_err)
        return false;
    unsigned f = 0;
    if (cudaMemcpy(&f, c->d_tc_err, sizeof(f), cudaMemcpyDeviceToHost) != cudaSuccess)
        return true;
    if (f)
        cudaMemset(c->d_tc_err, 0, sizeof(f));
    return f != 0;
}

// orders of the first-row candidates for n matrices (chunked: features, scores, sort)
cudaError_t compute_orders(canon_ctx *c, uint32_t n, uint32_t v, uint32_t b, const uint64_t *d_rows,
                           uint64_t *d_orders, cudaStream_t s) {
    const uint32_t chunk = 1u << 16;
    const size_t feat_bytes = (size_t)chunk * v * 64 * 2, score_bytes = (size_t)chunk * v * 4;
    cudaError_t e = ensure_scratch(c, feat_bytes + score_bytes + 256);
    if (e != cudaSuccess)
        return e;
    void *feat = c->d_scratch;
    float *scores = reinterpret_cast<float *>(static_cast<char *>(c->d_scratch) + feat_bytes);
    for (uint32_t off = 0; off < n; off += chunk) {
        const uint32_t cnt = (n - off < chunk) ? n - off : chunk;
        e = canon::mlp::features(cnt, v, b, 0, d_rows + (size_t)off * v, feat, s);
        if (e == cudaSuccess)
            e = mlp_forward_installed(c, (long)cnt * v, feat, scores, nullptr, nullptr, s);
        if (e == cudaSuccess)
            e = canon::launch_order_by_score(cnt, v, scores, d_orders + off, s);
        if (e != cudaSuccess)
            return e;
    }
    return cudaSuccess;
}

}  // namespace

namespace {

}  // namespace

extern "C" {

canon_ctx *canon_create(const canon_cfg *cfg) {
    canon_ctx *c = new canon_ctx();
    if (cfg)
        c->cfg = *cfg;
    if (!c->cfg.max_items)
        c->cfg.max_items = 1u << 21;
    if (!c->cfg.max_words)
        c->cfg.max_words = 16u * c->cfg.max_items;
    if (!c->cfg.aut_cap)
        c->cfg.aut_cap = 64;
    if (!c->cfg.max_trials)
        c->cfg.max_trials = 1ull << 28;
    c->max_bytes = c->cfg.max_words * 8u;
    // level capacity of the captured k-system enumeration: the context's item
    // capacity, at most 64K matrices (it grows when a level does not fit)
    c->ksys_graph_cap = std::min<uint64_t>(std::max<uint64_t>(c->cfg.max_items, 256), 1ull << 16);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= c->cfg.device || c->cfg.device < 0) {
        c->err = "no CUDA device";
        delete c;
        return nullptr;
    }
    c->device = c->cfg.device;
    cudaError_t e = cudaSetDevice(c->device);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device);
    if (e == cudaSuccess)
        e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaEventCreate(&c->ev0);
    if (e == cudaSuccess)
        e = cudaEventCreate(&c->ev1);
    const size_t n = c->cfg.max_items;
    if (e == cudaSuccess)
        e = host_alloc(&c->h_bitems, n);
    if (e == cudaSuccess)
        e = host_alloc(&c->h_kitems, n);
    if (e == cudaSuccess)
        e = host_alloc(&c->h_words, c->cfg.max_words);
    if (e == cudaSuccess)
        e = host_alloc(&c->h_bytes, c->max_bytes);
    if (e == cudaSuccess)
        e = dev_alloc(&c->d_bitems, n);
    if (e == cudaSuccess)
        e = dev_alloc(&c->d_kitems, n);
    if (e == cudaSuccess)
        e = dev_alloc(&c->d_words, c->cfg.max_words);
    if (e == cudaSuccess)
        e = dev_alloc(&c->d_bytes, c->max_bytes);
    if (e == cudaSuccess)
        e = dev_alloc(&c->d_ticket, 2);
    if (e == cudaSuccess)
        e = dev_alloc(&c->d_tc_err, 1);
    if (e == cudaSuccess)
        e = cudaMemset(c->d_tc_err, 0, sizeof(unsigned));
    if (e == cudaSuccess)
        e = alloc_outputs(c->d_out, n, c->cfg.aut_cap, true);
    if (e == cudaSuccess)
        e = alloc_outputs(c->h_out, n, c->cfg.aut_cap, false);
    if (e == cudaSuccess)
        e = canon::ksys_upload_tables();
    if (e != cudaSuccess) {
        std::fprintf(stderr, "canon_create: %s\n", cudaGetErrorString(e));
        canon_destroy(c);
        return nullptr;
    }
    c->item_kind.reserve(1024);
    return c;
}

void canon_destroy(canon_ctx *c) {
    if (c) {
        cudaFree(c->d_split_parts);
        cudaFree(c->d_split_stop);
        cudaFree(c->d_kseg);
    }
    if (c && c->ksys_graph) {
        cudaSetDevice(c->device);
        canon::ksys_graph_release(c);
    }
    if (!c)
        return;
    cudaSetDevice(c->device);
    if (c->stream)
        cudaStreamSynchronize(c->stream);
    free_outputs(c->d_out, true);
    free_outputs(c->h_out, false);
    void *dptrs[] = {c->d_bitems, c->d_kitems, c->d_words, c->d_bytes, c->d_ticket, c->d_tc_err, c->d_mlp, c->d_w1, c->d_w2,
                     c->d_w2t, c->d_w3, c->d_adam_m, c->d_adam_v, c->d_grad, c->d_loss, c->d_scratch,
                     c->d_orders};
    for (void *p : dptrs)
        if (p)
            cudaFree(p);
    void *hptrs[] = {c->h_bitems, c->h_kitems, c->h_words, c->h_bytes};
    for (void *p : hptrs)
        if (p)
            cudaFreeHost(p);
    if (c->ev0)
        cudaEventDestroy(c->ev0);
    if (c->ev1)
        cudaEventDestroy(c->ev1);
    if (c->stream)
        cudaStreamDestroy(c->stream);
    delete c;
}

const char *canon_last_error(const canon_ctx *c) { return c ? c->err.c_str() : "null context"; }

int canon_submit_bibd(canon_ctx *c, const canon_bibd_batch *bt) {
    if (!c || !bt)
        return fail(c, CANON_EINVAL, "null argument");
    if (!bt->n)
        return CANON_OK;
    if (!bt->rows || bt->v < 1 || bt->v > canon::VMAX || bt->b < 1 || bt->b > canon::BMAX)
        return fail(c, CANON_EINVAL, "bibd batch: need rows, 1 <= v <= 16, 1 <= b <= 63");
    if (bt->flags & ~0x7Fu)
        return fail(c, CANON_EINVAL, "bibd batch: unknown flags");
    if (c->q_ks_groups)
        return fail(c, CANON_EINVAL, "groups of 3 or 4 are queued: canon_sync them before other batches");
    const uint32_t total = c->n_bitems + c->n_kitems;
    if ((uint64_t)total + bt->n > c->cfg.max_items)
        return fail(c, CANON_ENOMEM, "item capacity exceeded (canon_cfg.max_items)");
    if ((uint64_t)c->n_words + (uint64_t)bt->n * bt->v > c->cfg.max_words)
        return fail(c, CANON_ENOMEM, "word capacity exceeded (canon_cfg.max_words)");
    // packed on host threads, which check the filled-row counts; a refused batch leaves
    // the queue as it was (its bytes past the queue's end are overwritten by the next batch)
    const bool ok = canon::pack_items_by_rows(
        bt->n, bt->nrows, bt->v, c->h_bitems + c->n_bitems,
        [&](uint64_t lo, uint64_t hi) {
            std::memcpy(c->h_words + c->n_words + lo * bt->v, bt->rows + lo * bt->v,
                        (size_t)(hi - lo) * bt->v * sizeof(uint64_t));
        },
        [&](uint64_t i, uint32_t nr) {
            Item it{};
            it.data_off = c->n_words + (uint32_t)i * bt->v;
            it.kind = canon::KIND_BIBD;
            it.nrows = (uint8_t)nr;
            it.ncols = (uint8_t)bt->b;
            it.flags = (uint8_t)bt->flags;
            it.out_idx = total + (uint32_t)i;
            return it;
        });
    if (!ok)
        return fail(c, CANON_EINVAL, "bibd batch: nrows out of range");
    cudaError_t e = cudaSetDevice(c->device);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(c->d_words + c->n_words, c->h_words + c->n_words, (size_t)bt->n * bt->v * 8,
                            cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(c->d_bitems + c->n_bitems, c->h_bitems + c->n_bitems, (size_t)bt->n * sizeof(Item),
                            cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "bibd batch upload");
    const uint8_t f = (uint8_t)bt->flags;
    c->q_two_pass = c->q_two_pass && (f & (canon::F_AUT_CANON | canon::F_FULL_AUT)) &&
                    !(f & (canon::F_SAVE_AUTS | canon::F_REFERENCE_ORDER));
    c->q_want_auts = c->q_want_auts || (f & canon::F_SAVE_AUTS);
    c->q_max_b = std::max(c->q_max_b, bt->b);
    // the widest filled-row count decides the kernel's row capacity, as the rows read
    uint32_t mv = bt->v;
    if (bt->nrows) {
        mv = 0;
        for (uint32_t i = 0; i < bt->n && mv < bt->v; ++i)
            mv = std::max<uint32_t>(mv, bt->nrows[i]);
    }
    c->q_max_v = std::max(c->q_max_v, mv);
    c->n_words += bt->n * bt->v;
    c->n_bitems += bt->n;
    c->item_kind.insert(c->item_kind.end(), bt->n, canon::KIND_BIBD);
    return CANON_OK;
}

// queues a checked k-system batch with groups of g (Item::pad)
static int submit_ksys_items(canon_ctx *c, const canon_ksys_batch *bt, uint32_t g) {
    const uint32_t total = c->n_bitems + c->n_kitems;
    const uint64_t bytes = (uint64_t)bt->n * bt->rounds * bt->np;
    if ((uint64_t)total + bt->n > c->cfg.max_items)
        return fail(c, CANON_ENOMEM, "item capacity exceeded (canon_cfg.max_items)");
    if ((uint64_t)c->n_bytes + bytes > c->max_bytes)
        return fail(c, CANON_ENOMEM, "byte capacity exceeded (8 * canon_cfg.max_words)");
    const uint64_t per = (uint64_t)bt->rounds * bt->np;
    const bool ok = canon::pack_items_by_rows(
        bt->n, bt->nrows, bt->rounds, c->h_kitems + c->n_kitems,
        [&](uint64_t lo, uint64_t hi) {
            std::memcpy(c->h_bytes + c->n_bytes + lo * per, bt->data + lo * per, (size_t)((hi - lo) * per));
        },
        [&](uint64_t i, uint32_t nr) {
            Item it{};
            it.data_off = c->n_bytes + (uint32_t)(i * per);
            it.kind = canon::KIND_KSYS;
            it.nrows = (uint8_t)nr;
            it.ncols = (uint8_t)bt->np;
            it.flags = (uint8_t)bt->flags;
            it.out_idx = total + (uint32_t)i;
            it.pad = g;
            return it;
        });
    if (!ok)
        return fail(c, CANON_EINVAL, "ksys batch: nrows out of range");
    cudaError_t e = cudaSetDevice(c->device);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(c->d_bytes + c->n_bytes, c->h_bytes + c->n_bytes, (size_t)bytes, cudaMemcpyHostToDevice,
                            c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(c->d_kitems + c->n_kitems, c->h_kitems + c->n_kitems, (size_t)bt->n * sizeof(Item),
                            cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "ksys batch upload");
    c->q_want_auts = c->q_want_auts || (bt->flags & canon::F_SAVE_AUTS);
    c->q_ks_np = std::max(c->q_ks_np, bt->np);
    uint32_t mr = bt->rounds;
    if (bt->nrows) {
        mr = 0;
        for (uint32_t i = 0; i < bt->n && mr < bt->rounds; ++i)
            mr = std::max<uint32_t>(mr, bt->nrows[i]);
    }
    c->q_ks_nr = std::max(c->q_ks_nr, mr);
    if (g > 2) {
        c->q_ks_groups = true;
        c->q_ks_total = std::max(c->q_ks_total, canon::kgen_candidates(bt->np, g, mr));
    }
    c->n_bytes += (uint32_t)bytes;
    c->n_kitems += bt->n;
    c->item_kind.insert(c->item_kind.end(), bt->n, canon::KIND_KSYS);
    return CANON_OK;
}

int canon_submit_ksys(canon_ctx *c, const canon_ksys_batch *bt) {
    if (!c || !bt)
        return fail(c, CANON_EINVAL, "null argument");
    if (!bt->n)
        return CANON_OK;
    if (!bt->data || bt->np < 4 || bt->np > canon::KS_NPMAX || (bt->np & 1u) || bt->rounds < 1 ||
        bt->rounds >= bt->np)
        return fail(c, CANON_EINVAL, "ksys batch: need data, even 4 <= np <= 12, 1 <= rounds < np");
    if (bt->flags & ~0xFu)
        return fail(c, CANON_EINVAL, "ksys batch: unknown flags");
    if (c->q_ks_groups)
        return fail(c, CANON_EINVAL, "groups of 3 or 4 are queued: canon_sync them before other batches");
    return submit_ksys_items(c, bt, 2);
}

int canon_submit_ksys_groups(canon_ctx *c, const canon_ksys_batch *bt, uint32_t group_size) {
    if (!c || !bt)
        return fail(c, CANON_EINVAL, "null argument");
    if (group_size == 2)
        return canon_submit_ksys(c, bt);
    if (group_size != 3 && group_size != 4)
        return fail(c, CANON_EINVAL, "ksys batch: group size 2, 3 or 4");
    if (!bt->n)
        return CANON_OK;
    if (!bt->data || bt->np > 16 || bt->np % group_size || bt->np / group_size < 2 || bt->rounds < 1 ||
        bt->rounds >= bt->np)
        return fail(c, CANON_EINVAL,
                    "ksys batch: need data, np <= 16 a multiple of the group size (2 groups at least), "
                    "1 <= rounds < np");
    if (bt->flags & ~0xFu)
        return fail(c, CANON_EINVAL, "ksys batch: unknown flags");
    if (c->n_bitems || (c->n_kitems && !c->q_ks_groups))
        return fail(c, CANON_EINVAL, "groups of 3 or 4 are checked in a queue of their own: canon_sync first");
    return submit_ksys_items(c, bt, group_size);
}

int canon_sync(canon_ctx *c, canon_results *r) {
    if (!c || !r)
        return fail(c, CANON_EINVAL, "null argument");
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "cudaSetDevice");
    const uint32_t n = c->n_bitems + c->n_kitems;
    const bool verdict_sync = c->cfg.options & CANON_OPT_VERDICT_SYNC;
    std::memset(r, 0, sizeof(*r));
    if (n) {
        cudaStream_t s = c->stream;
        if (c->q_reupload) {
            // the device staging was borrowed after the batches were queued: copy them again
            if (c->n_bitems)
                cudaMemcpyAsync(c->d_bitems, c->h_bitems, c->n_bitems * sizeof(Item), cudaMemcpyHostToDevice, s);
            if (c->n_kitems)
                cudaMemcpyAsync(c->d_kitems, c->h_kitems, c->n_kitems * sizeof(Item), cudaMemcpyHostToDevice, s);
            if (c->n_words)
                cudaMemcpyAsync(c->d_words, c->h_words, c->n_words * sizeof(uint64_t), cudaMemcpyHostToDevice, s);
            if (c->n_bytes)
                cudaMemcpyAsync(c->d_bytes, c->h_bytes, c->n_bytes, cudaMemcpyHostToDevice, s);
            e = cudaGetLastError();
            if (e != cudaSuccess)
                return cuda_fail(c, e, "canon_sync upload");
        }
        cudaEventRecord(c->ev0, s);
        if (c->n_bitems && c->n_kitems) {
            // uneven batch: one persistent launch for both kinds, sized by the widest
            // incidence item
            e = canon::launch_mixed_check(c->d_bitems, c->n_bitems, c->d_kitems, c->n_kitems, c->d_words,
                                          c->d_bytes, c->d_out, c->cfg.max_trials, c->d_ticket, c->num_sms, s,
                                          c->q_max_b, c->q_max_v);
            if (e != cudaSuccess)
                return cuda_fail(c, e, "mixed check launch");
            ++c->launches;
        } else if (c->n_bitems) {
            // items that all want |Aut| without the reference order take the two-pass check
            const bool two_pass = c->q_two_pass;
            e = two_pass ? canon::launch_bibd_check_two_pass(c->d_bitems, c->n_bitems, c->d_words, c->d_out,
                                                             c->cfg.max_trials, c->d_ticket, c->num_sms, s, c->q_max_b,
                                                             c->q_max_v)
                         : canon::launch_bibd_check(c->d_bitems, c->n_bitems, c->d_words, c->d_out,
                                                    c->cfg.max_trials, c->d_ticket, c->num_sms, s);
            if (e != cudaSuccess)
                return cuda_fail(c, e, "bibd check launch");
            c->launches += two_pass ? 2 : 1;
        } else if (c->n_kitems) {
            const uint32_t seg =
                c->q_ks_groups ? canon::kgen_segment(c, c->n_kitems, c->q_ks_total)
                : c->q_want_auts ? 0u
                                 : canon::ksys_segment(c, c->n_kitems, c->q_ks_np, c->q_ks_nr);
            if (seg) {
                if (c->kseg_cap < (size_t)c->n_kitems + 1) {
                    cudaFree(c->d_kseg);
                    c->d_kseg = nullptr;
                    c->kseg_cap = 0;
                    e = cudaMalloc(&c->d_kseg, ((size_t)c->n_kitems + 1) * sizeof(canon::KsysSeg));
                    if (e != cudaSuccess)
                        return cuda_fail(c, e, "k-system segment state");
                    c->kseg_cap = (size_t)c->n_kitems + 1;
                }
                e = c->q_ks_groups
                        ? canon::launch_kgen_check(c->d_kitems, c->n_kitems, c->d_bytes, c->d_out, seg,
                                                   c->q_ks_total, c->d_kseg, c->num_sms, s)
                        : canon::launch_ksys_check_split(c->d_kitems, c->n_kitems, c->d_bytes, c->d_out, seg,
                                                         canon::ksys_candidates(c->q_ks_np, c->q_ks_nr),
                                                         c->d_kseg, c->num_sms, s);
                c->launches += 3;
            } else {
                e = canon::launch_ksys_check(c->d_kitems, c->n_kitems, c->d_bytes, c->d_out, c->d_ticket + 1,
                                             c->num_sms, s);
                ++c->launches;
            }
            if (e != cudaSuccess)
                return cuda_fail(c, e, "ksys check launch");
        }
        cudaEventRecord(c->ev1, s);
        const Outputs &d = c->d_out, &h = c->h_out;
#define CANON_D2H(field, count) \
    cudaMemcpyAsync(h.field, d.field, (size_t)(count) * sizeof(*h.field), cudaMemcpyDeviceToHost, s)
        CANON_D2H(canonical, n);
        CANON_D2H(status, n);
        if (!verdict_sync) {
            CANON_D2H(reject_row, n);
            CANON_D2H(row_to_change, n);
            CANON_D2H(player_index, n);
            CANON_D2H(witness, n * 16);
            CANON_D2H(aut, n * 2);
            CANON_D2H(trials, n);
            CANON_D2H(n_auts, n);
            CANON_D2H(len_aut, n);
        }
#undef CANON_D2H
        const bool want_auts = c->q_want_auts && !verdict_sync;
        if (want_auts)
            cudaMemcpyAsync(h.auts, d.auts, (size_t)n * c->cfg.aut_cap * 64, cudaMemcpyDeviceToHost, s);
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess)
            return cuda_fail(c, e, "canon_sync");
        cudaEventElapsedTime(&c->last_ms, c->ev0, c->ev1);
        if (want_auts) {
            // k-system automorphisms form a sorted set, as CGroupInfo::updateRepo keeps them
            for (uint32_t i = 0; i < c->n_kitems; ++i) {
                const Item &it = c->h_kitems[i];
                if (!(it.flags & canon::F_SAVE_AUTS))
                    continue;
                const uint32_t o = it.out_idx, na = h.n_auts[o], np = it.ncols;
                uint8_t *base = h.auts + (size_t)o * c->cfg.aut_cap * 64;
                std::vector<std::vector<uint8_t>> v(na);
                for (uint32_t k = 0; k < na; ++k)
                    v[k].assign(base + k * 64, base + k * 64 + np);
                std::sort(v.begin(), v.end());
                for (uint32_t k = 0; k < na; ++k)
                    std::memcpy(base + k * 64, v[k].data(), np);
            }
        }
    }
    r->n = n;
    r->canonical = c->h_out.canonical;
    r->status = c->h_out.status;
    r->reject_row = c->h_out.reject_row;
    r->row_to_change = c->h_out.row_to_change;
    r->player_index = c->h_out.player_index;
    r->witness = c->h_out.witness;
    r->aut = c->h_out.aut;
    r->trials = c->h_out.trials;
    r->n_auts = c->h_out.n_auts;
    r->len_aut = c->h_out.len_aut;
    r->auts = c->h_out.auts;
    r->aut_cap = c->cfg.aut_cap;
    r->kernel_ms = c->last_ms;
    c->n_bitems = c->n_kitems = c->n_words = c->n_bytes = 0;
    c->q_max_b = c->q_max_v = c->q_ks_np = c->q_ks_nr = 0;
    c->q_ks_total = 0;
    c->q_ks_groups = false;
    c->q_two_pass = true;
    c->q_want_auts = c->q_reupload = false;
    c->item_kind.clear();
    // any item out of trial budget: eight status bytes at a time
    uint64_t any = 0;
    uint32_t i = 0;
    for (; i + 8 <= n; i += 8) {
        uint64_t w;
        std::memcpy(&w, c->h_out.status + i, 8);
        any |= w;
    }
    for (; i < n; ++i)
        any |= c->h_out.status[i];
    if (any & 0x0202020202020202ull) {
        c->err = "a search hit the trial budget (canon_cfg.max_trials)";
        return CANON_ETIMEOUT;
    }
    return CANON_OK;
}

int canon_set_ksys_segment(canon_ctx *c, uint32_t cands) {
    if (!c)
        return CANON_EINVAL;
    c->ksys_seg = cands;
    return CANON_OK;
}

int canon_set_ordering(canon_ctx *c, const canon_mlp_weights *w) {
    if (!c)
        return CANON_EINVAL;
    if (!w) {
        c->order_on = false;
        return CANON_OK;
    }
    if (w->in_dim != 64 || w->hidden != 128 || !w->w1 || !w->w2 || !w->w3 || !w->b1 || !w->b2 || !w->b3)
        return fail(c, CANON_EINVAL, "ordering: need in_dim 64, hidden 128 and all weights");
    // BF16 weights -> the flat FP32 vector the kernels read
    std::vector<float> p(canon::mlp::N_PARAMS);
    auto f32 = [](uint16_t h) {
        uint32_t u = (uint32_t)h << 16;
        float f;
        std::memcpy(&f, &u, 4);
        return f;
    };
    for (int i = 0; i < 128 * 64; ++i)
        p[P_W1 + i] = f32(w->w1[i]);
    for (int i = 0; i < 128 * 128; ++i)
        p[P_W2 + i] = f32(w->w2[i]);
    for (int i = 0; i < 128; ++i) {
        p[P_W3 + i] = f32(w->w3[i]);
        p[P_B1 + i] = w->b1[i];
        p[P_B2 + i] = w->b2[i];
    }
    p[P_B3] = w->b3[0];
    cudaSetDevice(c->device);
    cudaError_t e = upload_params(c, p.data());
    if (e != cudaSuccess)
        return cuda_fail(c, e, "ordering upload");
    c->order_on = true;
    return CANON_OK;
}

int canon_canonize_bibd(canon_ctx *c, uint32_t n, uint32_t v, uint32_t b, uint64_t *rows, uint64_t *aut_out) {
    if (!c || !rows)
        return fail(c, CANON_EINVAL, "null argument");
    if (v < 1 || v > canon::VMAX || b < 1 || b > canon::BMAX)
        return fail(c, CANON_EINVAL, "canonize: need 1 <= v <= 16, 1 <= b <= 63");
    if (!n)
        return CANON_OK;
    if ((uint64_t)n * v > c->cfg.max_words || n > c->cfg.max_items)
        return fail(c, CANON_ENOMEM, "canonize: batch exceeds context capacity");
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    // borrows the device staging of queued batches: canon_sync copies them again
    if (c->n_words)
        c->q_reupload = true;
    cudaMemcpyAsync(c->d_words, rows, (size_t)n * v * 8, cudaMemcpyHostToDevice, s);
    cudaEventRecord(c->ev0, s);
    cudaError_t e = canon::launch_bibd_canonize(n, v, b, c->d_words, c->d_out.aut, c->d_out.status, 1, 0,
                                                c->cfg.max_trials, c->d_ticket, c->num_sms, s);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "canonize launch");
    ++c->launches;
    cudaEventRecord(c->ev1, s);
    cudaMemcpyAsync(rows, c->d_words, (size_t)n * v * 8, cudaMemcpyDeviceToHost, s);
    if (aut_out)
        cudaMemcpyAsync(aut_out, c->d_out.aut, (size_t)n * 16, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(c->h_out.status, c->d_out.status, n, cudaMemcpyDeviceToHost, s);
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "canonize");
    cudaEventElapsedTime(&c->last_ms, c->ev0, c->ev1);
    for (uint32_t i = 0; i < n; ++i)
        if (c->h_out.status[i])
            return fail(c, (c->h_out.status[i] & canon::ST_TIMEOUT) ? CANON_ETIMEOUT : CANON_EINVAL,
                        "canonize: an item failed");
    return CANON_OK;
}

namespace {

uint32_t tune_key(uint32_t v, uint32_t b, uint32_t flags) { return v | (b << 8) | (flags << 16); }

// the split variant's scratch, grown to n matrices of v rows
cudaError_t split_scratch(canon_ctx *c, size_t n, uint32_t v) {
    const size_t need = n * v * (canon::split_levels(n, v) == 2 ? v : 1);
    if (need <= c->split_cap && c->d_split_stop)
        return cudaSuccess;
    cudaFree(c->d_split_parts);
    cudaFree(c->d_split_stop);
    c->d_split_parts = nullptr;
    c->d_split_stop = nullptr;
    c->split_cap = 0;
    cudaError_t e = cudaMalloc((void **)&c->d_split_parts, need * sizeof(canon::SplitPart));
    if (e == cudaSuccess)
        e = cudaMalloc((void **)&c->d_split_stop, need * sizeof(unsigned) + 64);   // need >= n
    if (e == cudaSuccess)
        c->split_cap = need;
    return e;
}

// one resident check in the given variant (-1: the default rule)
cudaError_t run_variant(canon_ctx *c, int variant, uint32_t n, uint32_t v, uint32_t b, uint32_t flags,
                        const uint64_t *d_rows, uint8_t *d_canonical, uint8_t *d_witness16, uint64_t *d_aut,
                        uint8_t *d_status, uint64_t *d_trials, const uint64_t *orders, cudaStream_t s) {
    if (variant == canon::VARIANT_SPLIT) {
        cudaError_t e = split_scratch(c, n, v);
        if (e != cudaSuccess)
            return e;
        c->launches += 2;
        return canon::launch_bibd_check_split(n, v, b, flags, d_rows, d_canonical, d_aut, d_status,
                                              c->d_split_parts, c->d_split_stop, c->cfg.max_trials, c->d_ticket,
                                              c->num_sms, s);
    }
    const bool ref = flags & (CANON_SAVE_AUTS | CANON_REFERENCE_ORDER);
    const bool two = !ref && (variant < 0 ? (flags & (CANON_AUT_CANON | CANON_FULL_AUT)) != 0
                                          : (variant == canon::VARIANT_TWO_PASS ||
                                             variant == canon::VARIANT_CONVERGED ||
                                             variant == canon::VARIANT_CONVERGED_D2 ||
                                             variant == canon::VARIANT_CONVERGED_D8));
    c->launches += two ? ((d_witness16 || d_trials) ? 2 : 1) : 1;
    return canon::launch_bibd_check_uniform(n, v, b, flags, d_rows, d_canonical, d_witness16, d_aut, d_status,
                                            d_trials, c->cfg.max_trials, c->d_ticket, c->num_sms, s, orders,
                                            variant);
}

}  // namespace

int canon_check_bibd_device(canon_ctx *c, uint32_t n, uint32_t v, uint32_t b, uint32_t flags,
                            const uint64_t *d_rows, uint8_t *d_canonical, uint8_t *d_witness16, uint64_t *d_aut,
                            uint8_t *d_status, uint64_t *d_trials, void *stream) {
    if (!c || !d_rows || !d_canonical)
        return fail(c, CANON_EINVAL, "null argument");
    if (v < 1 || v > canon::VMAX || b < 1 || b > canon::BMAX || (flags & ~0x77u))
        return fail(c, CANON_EINVAL,
                    "check: need 1 <= v <= 16, 1 <= b <= 63, flags in COMPLETE|RAW|FULL_AUT|AUT_CANON|"
                    "REFERENCE_ORDER|VERDICT_ONLY");
    cudaSetDevice(c->device);
    cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
    uint64_t *orders = nullptr;
    cudaEventRecord(c->ev0, s);
    if (c->order_on) {
        // learned order of the first rows: features, scores and the sort are part of the timed check
        const size_t need = (size_t)n * 8 + 256;
        cudaError_t e0 = cudaSuccess;
        if (!c->d_orders_bytes || c->d_orders_bytes < need) {
            if (c->d_orders)
                cudaFree(c->d_orders);
            c->d_orders = nullptr;
            c->d_orders_bytes = 0;
            e0 = cudaMalloc((void **)&c->d_orders, need);
            if (e0 == cudaSuccess)
                c->d_orders_bytes = need;
        }
        if (e0 == cudaSuccess)
            e0 = compute_orders(c, n, v, b, d_rows, c->d_orders, s);
        if (e0 != cudaSuccess)
            return cuda_fail(c, e0, "learned order");
        orders = c->d_orders;
        c->launches += 3 * ((n + 65535) / 65536);
    }
    int variant = -1;
    if (!orders) {
        const auto it = c->tuned.find(tune_key(v, b, flags));
        if (it != c->tuned.end())
            variant = it->second;
    }
    const cudaError_t e = run_variant(c, variant, n, v, b, flags, d_rows, d_canonical, d_witness16, d_aut,
                                      d_status, d_trials, orders, s);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "check launch");
    cudaEventRecord(c->ev1, s);
    return CANON_OK;
}

int canon_tune_bibd(canon_ctx *c, uint32_t n, uint32_t v, uint32_t b, uint32_t flags, const uint64_t *d_rows,
                    canon_tune_result *out) {
    if (!c || !d_rows || !out || !n)
        return fail(c, CANON_EINVAL, "tune: null argument or empty sample");
    if (v < 1 || v > canon::VMAX || b < 1 || b > canon::BMAX || (flags & ~0x77u))
        return fail(c, CANON_EINVAL, "tune: bad shape or flags");
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    const bool ref = flags & (CANON_SAVE_AUTS | CANON_REFERENCE_ORDER);
    const bool verdict = flags & CANON_VERDICT_ONLY;
    const bool want_aut = flags & (CANON_AUT_CANON | CANON_FULL_AUT);
    constexpr int NV = canon::N_VARIANTS;
    const bool small = v <= 15 && b <= 35;     // the instance the staging-depth variants exist for
    bool applies[NV] = {true, !ref, verdict && !ref && !want_aut, !ref, !ref && small, !ref && small};
    // outputs of every variant, compared with the one-pass variant's on the host
    struct Out {
        uint8_t *can = nullptr, *wit = nullptr, *st = nullptr;
        uint64_t *aut = nullptr;
    } o[NV];
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < NV && e == cudaSuccess; ++k) {
        if (!applies[k])
            continue;
        e = cudaMalloc((void **)&o[k].can, n);
        if (e == cudaSuccess)
            e = cudaMalloc((void **)&o[k].st, n);
        if (e == cudaSuccess)
            e = cudaMalloc((void **)&o[k].aut, (size_t)n * 16);
        if (e == cudaSuccess && !verdict)
            e = cudaMalloc((void **)&o[k].wit, (size_t)n * 16);
    }
    std::vector<uint8_t> can0(n), st0(n), wit0(verdict ? 0 : (size_t)n * 16), can1(n), st1(n),
        wit1(verdict ? 0 : (size_t)n * 16);
    std::vector<uint64_t> aut0((size_t)n * 2), aut1((size_t)n * 2);
    float ms[NV];
    for (int k = 0; k < NV; ++k)
        ms[k] = -1.f;
    int best = -1;
    for (int k = 0; k < NV && e == cudaSuccess; ++k) {
        if (!applies[k])
            continue;
        // one untimed run, then two timed ones
        e = run_variant(c, k, n, v, b, flags, d_rows, o[k].can, o[k].wit, o[k].aut, o[k].st, nullptr, nullptr, s);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(s);
        float t = 0.f;
        for (int rep = 0; rep < 2 && e == cudaSuccess; ++rep) {
            cudaEventRecord(c->ev0, s);
            e = run_variant(c, k, n, v, b, flags, d_rows, o[k].can, o[k].wit, o[k].aut, o[k].st, nullptr, nullptr,
                            s);
            cudaEventRecord(c->ev1, s);
            if (e == cudaSuccess)
                e = cudaEventSynchronize(c->ev1);
            float dt = 0.f;
            cudaEventElapsedTime(&dt, c->ev0, c->ev1);
            t += dt;
        }
        if (e != cudaSuccess)
            break;
        ms[k] = t / 2.f;
        // identical outputs, or the variant is not kept
        std::vector<uint8_t> &cn = k ? can1 : can0, &sn = k ? st1 : st0, &wn = k ? wit1 : wit0;
        std::vector<uint64_t> &an = k ? aut1 : aut0;
        e = cudaMemcpy(cn.data(), o[k].can, n, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess)
            e = cudaMemcpy(sn.data(), o[k].st, n, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess)
            e = cudaMemcpy(an.data(), o[k].aut, (size_t)n * 16, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess && !verdict)
            e = cudaMemcpy(wn.data(), o[k].wit, (size_t)n * 16, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess)
            break;
        bool same = true;
        for (uint32_t i = 0; k && same && i < n; ++i) {
            same = can1[i] == can0[i] && st1[i] == st0[i];
            if (same && (can0[i] || want_aut))
                same = aut1[2 * i] == aut0[2 * i] && aut1[2 * i + 1] == aut0[2 * i + 1];
            if (same && !verdict && !can0[i])
                same = std::memcmp(&wit1[(size_t)i * 16], &wit0[(size_t)i * 16], v) == 0;
        }
        if (!same)
            ms[k] = -2.f;
        else if (best < 0 || ms[k] < ms[best])
            best = k;
    }
    for (int k = 0; k < NV; ++k) {
        cudaFree(o[k].can);
        cudaFree(o[k].st);
        cudaFree(o[k].aut);
        cudaFree(o[k].wit);
    }
    if (e != cudaSuccess)
        return cuda_fail(c, e, "tune");
    c->tuned[tune_key(v, b, flags)] = best;
    out->variant = best;
    for (int k = 0; k < NV; ++k)
        out->ms[k] = ms[k];
    return CANON_OK;
}

int canon_lexmax_nodes_bibd(canon_ctx *c, uint32_t n, uint32_t v, uint32_t b, uint32_t flags,
                            const uint64_t *d_rows, uint64_t *d_nodes, const uint64_t *d_orders) {
    if (!c || !d_rows || !d_nodes)
        return fail(c, CANON_EINVAL, "null argument");
    if (v < 1 || v > canon::VMAX || b < 1 || b > canon::BMAX)
        return fail(c, CANON_EINVAL, "nodes: need 1 <= v <= 16, 1 <= b <= 63");
    cudaSetDevice(c->device);
    const uint64_t *orders = d_orders;
    cudaError_t e = cudaSuccess;
    if (!orders && c->order_on) {
        // the learned first-row order, as canon_check_bibd_device applies it
        const size_t need = (size_t)n * 8 + 256;
        if (!c->d_orders_bytes || c->d_orders_bytes < need) {
            if (c->d_orders)
                cudaFree(c->d_orders);
            c->d_orders = nullptr;
            c->d_orders_bytes = 0;
            e = cudaMalloc((void **)&c->d_orders, need);
            if (e == cudaSuccess)
                c->d_orders_bytes = need;
        }
        if (e == cudaSuccess)
            e = compute_orders(c, n, v, b, d_rows, c->d_orders, c->stream);
        orders = c->d_orders;
    }
    if (e == cudaSuccess)
        e = canon::launch_bibd_lexmax_nodes(n, v, b, flags, d_rows, d_nodes, c->cfg.max_trials, c->d_ticket,
                                            c->num_sms, c->stream, orders);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    ++c->launches;
    return e == cudaSuccess ? CANON_OK : cuda_fail(c, e, "nodes");
}

int canon_measure_int_peak(canon_ctx *c, double *lane_ops_per_s) {
    if (!c || !lane_ops_per_s)
        return fail(c, CANON_EINVAL, "null argument");
    cudaSetDevice(c->device);
    uint32_t *sink = nullptr;
    cudaError_t e = cudaMalloc((void **)&sink, 16);
    uint64_t ops = 0;
    float best = 0.f;
    // one untimed launch, then the fastest of five
    for (int rep = 0; rep < 6 && e == cudaSuccess; ++rep) {
        cudaEventRecord(c->ev0, c->stream);
        e = canon::launch_int_peak(1u << 16, c->num_sms, sink, c->stream, &ops);
        cudaEventRecord(c->ev1, c->stream);
        if (e == cudaSuccess)
            e = cudaEventSynchronize(c->ev1);
        float ms = 0.f;
        if (e == cudaSuccess)
            e = cudaEventElapsedTime(&ms, c->ev0, c->ev1);
        if (e == cudaSuccess && rep > 0 && ms > 0.f && (best == 0.f || ms < best))
            best = ms;
        ++c->launches;
    }
    cudaFree(sink);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "int peak");
    *lane_ops_per_s = best > 0.f ? (double)ops / (best * 1e-3) : 0.0;
    return CANON_OK;
}

int canon_generate_sts_device(canon_ctx *c, uint32_t n, uint32_t v, uint64_t seed, int canon_odd, uint64_t *d_rows,
                              void *stream) {
    if (!c || !d_rows)
        return fail(c, CANON_EINVAL, "null argument");
    if (v > canon::VMAX || v < 3 || (v % 6 != 1 && v % 6 != 3))
        return fail(c, CANON_EINVAL, "generate: STS(v) needs v = 1 or 3 mod 6, 3 <= v <= 15");
    cudaSetDevice(c->device);
    cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
    cudaError_t e = canon::launch_sts_generate(n, v, seed, d_rows, c->num_sms, s);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "generate launch");
    ++c->launches;
    if (canon_odd) {
        e = canon::launch_bibd_canonize(n, v, v * (v - 1) / 6, d_rows, nullptr, nullptr, 2, 1, c->cfg.max_trials,
                                        c->d_ticket, c->num_sms, s);
        if (e != cudaSuccess)
            return cuda_fail(c, e, "canonize launch");
        ++c->launches;
    }
    return CANON_OK;
}

void *canon_device_alloc(canon_ctx *c, size_t bytes) {
    if (!c)
        return nullptr;
    cudaSetDevice(c->device);
    void *p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
        c->err = "cudaMalloc failed";
        return nullptr;
    }
    return p;
}

int canon_device_free(canon_ctx *c, void *p) {
    if (!c)
        return CANON_EINVAL;
    cudaSetDevice(c->device);
    cudaError_t e = cudaFree(p);
    return e == cudaSuccess ? CANON_OK : cuda_fail(c, e, "cudaFree");
}

int canon_memcpy_d2h(canon_ctx *c, void *dst, const void *src, size_t bytes) {
    if (!c)
        return CANON_EINVAL;
    cudaSetDevice(c->device);
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? CANON_OK : cuda_fail(c, e, "d2h");
}

int canon_memcpy_h2d(canon_ctx *c, void *dst, const void *src, size_t bytes) {
    if (!c)
        return CANON_EINVAL;
    cudaSetDevice(c->device);
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? CANON_OK : cuda_fail(c, e, "h2d");
}

float canon_last_kernel_ms(const canon_ctx *c) {
    if (!c)
        return 0.f;
    float ms = 0.f;
    if (cudaEventSynchronize(c->ev1) == cudaSuccess && cudaEventElapsedTime(&ms, c->ev0, c->ev1) == cudaSuccess)
        return ms;
    return c->last_ms;
}

uint64_t canon_kernel_launches(const canon_ctx *c) { return c ? c->launches : 0; }

int canon_stream_sync(canon_ctx *c) {
    if (!c)
        return CANON_EINVAL;
    cudaSetDevice(c->device);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? CANON_OK : cuda_fail(c, e, "stream sync");
}

int canon_mlp_features(canon_ctx *c, uint32_t n, uint32_t v, uint32_t b, const uint64_t *d_rows, void *d_feat) {
    if (!c || !d_rows || !d_feat || v < 1 || v > canon::VMAX || b < 1 || b > canon::BMAX)
        return fail(c, CANON_EINVAL, "features: bad arguments");
    cudaSetDevice(c->device);
    cudaError_t e = canon::mlp::features(n, v, b, 0, d_rows, d_feat, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    ++c->launches;
    return e == cudaSuccess ? CANON_OK : cuda_fail(c, e, "features");
}

int canon_label_first_rows(canon_ctx *c, uint32_t n, uint32_t v, uint32_t b, uint32_t flags, const uint64_t *d_rows,
                           uint16_t *d_first_rows, uint64_t *d_nodes, const uint64_t *d_orders) {
    if (!c || !d_rows || v < 1 || v > canon::VMAX || b < 1 || b > canon::BMAX)
        return fail(c, CANON_EINVAL, "labels: bad arguments");
    cudaSetDevice(c->device);
    cudaEventRecord(c->ev0, c->stream);
    cudaError_t e = canon::launch_bibd_labels(n, v, b, flags, d_rows, d_first_rows, d_nodes, d_orders,
                                              c->cfg.max_trials, c->d_ticket, c->num_sms, c->stream);
    cudaEventRecord(c->ev1, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    ++c->launches;
    return e == cudaSuccess ? CANON_OK : cuda_fail(c, e, "labels");
}

int canon_design_properties(canon_ctx *c, uint32_t n, uint32_t v, uint32_t b, const uint64_t *rows,
                            uint8_t *simple, uint8_t *transitive) {
    if (!c || (n && !rows) || v < 1 || v > canon::VMAX || b < 1 || b > canon::BMAX)
        return fail(c, CANON_EINVAL, "design properties: bad arguments");
    if (!n)
        return CANON_OK;
    if (simple) {
        for (uint32_t i = 0; i < n; ++i) {
            std::vector<uint32_t> colpat(b, 0u);
            for (uint32_t r = 0; r < v; ++r)
                for (uint32_t col = 0; col < b; ++col)
                    colpat[col] |= (uint32_t)((rows[(size_t)i * v + r] >> col) & 1u) << r;
            std::sort(colpat.begin(), colpat.end());
            simple[i] = std::adjacent_find(colpat.begin(), colpat.end()) == colpat.end();
        }
    }
    if (!transitive)
        return CANON_OK;
    cudaSetDevice(c->device);
    uint64_t *d_rows = nullptr;
    uint16_t *d_first = nullptr;
    cudaError_t e = cudaMalloc(&d_rows, (size_t)n * v * sizeof(uint64_t));
    if (e == cudaSuccess)
        e = cudaMalloc(&d_first, (size_t)n * sizeof(uint16_t));
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_rows, rows, (size_t)n * v * sizeof(uint64_t), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) {
        e = canon::launch_bibd_labels(n, v, b, canon::F_RAW | canon::F_COMPLETE, d_rows, d_first, nullptr, nullptr,
                                      c->cfg.max_trials, c->d_ticket, c->num_sms, c->stream);
        ++c->launches;
    }
    std::vector<uint16_t> first(n);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(first.data(), d_first, (size_t)n * sizeof(uint16_t), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    cudaFree(d_rows);
    cudaFree(d_first);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "design properties");
    const unsigned all = (v >= 16) ? 0xFFFFu : ((1u << v) - 1u);
    for (uint32_t i = 0; i < n; ++i)
        transitive[i] = first[i] == all;
    return CANON_OK;
}

int canon_mlp_forward(canon_ctx *c, uint64_t n, const void *d_x, const float *params, float *d_logits) {
    if (!c || !d_x || !d_logits || !params)
        return fail(c, CANON_EINVAL, "forward: bad arguments");
    cudaSetDevice(c->device);
    cudaError_t e = upload_params(c, params);
    if (e == cudaSuccess)
        e = mlp_forward_installed(c, (long)n, d_x, d_logits, nullptr, nullptr, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    ++c->launches;
    if (e == cudaSuccess && tc_timed_out(c))
        return fail(c, CANON_ETIMEOUT, "forward: a wait for the tensor cores timed out");
    return e == cudaSuccess ? CANON_OK : cuda_fail(c, e, "forward");
}

// one forward + backward over rows [0, n) of (d_x, d_labels) into c->d_grad (zeroed first)
static cudaError_t mlp_grad_pass(canon_ctx *c, long n, const void *d_x, const float *d_labels) {
    const size_t act = (size_t)n * 128;
    cudaError_t e = ensure_scratch(c, (size_t)n * 4 + act * 2 * 2 + (size_t)n * 4 + act * 4 * 2 + 1024);
    if (e != cudaSuccess)
        return e;
    // the per-row arrays of 128 values first (256- or 512-byte rows), so every one starts
    // 16-byte aligned (the tensor-core passes move them 16 bytes at a time), then the
    // per-row scalars
    char *base = static_cast<char *>(c->d_scratch);
    void *h1 = base;
    void *h2 = base + act * 2;
    float *dh2 = reinterpret_cast<float *>(base + act * 4);
    float *dh1 = dh2 + act;
    float *logit = dh1 + act;
    float *dy = logit + n;
    cudaStream_t s = c->stream;
    e = cudaMemsetAsync(c->d_grad, 0, canon::mlp::N_PARAMS * 4, s);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(c->d_loss, 0, 4, s);
    if (e == cudaSuccess)
        e = mlp_forward_installed(c, n, d_x, logit, h1, h2, s);
    if (e == cudaSuccess) {
        if (!(c->cfg.options & CANON_OPT_MLP_WARP_MMA) && c->d_tc_err && n >= 128)
            e = canon::mlp::backward_tc(n, logit, d_labels, h1, h2, c->d_w3, c->d_w2t, dy, dh2, dh1, c->d_loss,
                                        c->d_tc_err, c->num_sms, s);
        else
            e = canon::mlp::backward(n, logit, d_labels, h1, h2, c->d_w3, c->d_w2t, dy, dh2, dh1, c->d_loss,
                                     c->num_sms, s);
    }
    if (e == cudaSuccess) {
        if (!(c->cfg.options & CANON_OPT_MLP_WARP_MMA) && c->d_tc_err && n >= 128 &&
            ((uintptr_t)d_x & 15u) == 0)
            e = canon::mlp::weight_grads_tc(n, dh1, dh2, dy, d_x, h1, h2, c->d_grad, c->d_tc_err, c->num_sms, s);
        else
            e = canon::mlp::weight_grads(n, dh1, dh2, dy, d_x, h1, h2, c->d_grad, c->num_sms, s);
    }
    c->launches += 6;
    return e;
}

int canon_mlp_grad(canon_ctx *c, uint64_t n, const void *d_x, const float *d_labels, const float *params, float *grad,
                   float *loss) {
    if (!c || !d_x || !d_labels || !params || !grad || !n)
        return fail(c, CANON_EINVAL, "grad: bad arguments");
    cudaSetDevice(c->device);
    cudaError_t e = upload_params(c, params);
    if (e == cudaSuccess)
        e = mlp_grad_pass(c, (long)n, d_x, d_labels);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(grad, c->d_grad, canon::mlp::N_PARAMS * 4, cudaMemcpyDeviceToHost, c->stream);
    float l = 0.f;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&l, c->d_loss, 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    if (loss)
        *loss = l / (float)n;
    if (e == cudaSuccess && tc_timed_out(c))
        return fail(c, CANON_ETIMEOUT, "grad: a wait for the tensor cores timed out");
    return e == cudaSuccess ? CANON_OK : cuda_fail(c, e, "grad");
}

int canon_mlp_train(canon_ctx *c, uint64_t n, const void *d_x, const float *d_labels, uint32_t epochs,
                    uint32_t batch, float lr, float *params, float *epoch_loss) {
    if (!c || !d_x || !d_labels || !params || !n || !batch)
        return fail(c, CANON_EINVAL, "train: bad arguments");
    cudaSetDevice(c->device);
    cudaError_t e = upload_params(c, params);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "train upload");
    e = cudaMemsetAsync(c->d_adam_m, 0, canon::mlp::N_PARAMS * 4, c->stream);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(c->d_adam_v, 0, canon::mlp::N_PARAMS * 4, c->stream);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "train reset");
    int step = 0;
    for (uint32_t ep = 0; ep < epochs; ++ep) {
        double lsum = 0.0;
        for (uint64_t off = 0; off < n; off += batch) {
            const long cnt = (long)((n - off < batch) ? n - off : batch);
            e = mlp_grad_pass(c, cnt, static_cast<const char *>(d_x) + off * 128, d_labels + off);
            if (e == cudaSuccess)
                e = canon::mlp::adam(canon::mlp::N_PARAMS, c->d_mlp, c->d_grad, c->d_adam_m, c->d_adam_v, lr, ++step,
                                     c->d_w1, c->d_w2, c->d_w2t, c->d_w3, c->stream);
            float l = 0.f;
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(&l, c->d_loss, 4, cudaMemcpyDeviceToHost, c->stream);
            if (e == cudaSuccess)
                e = cudaStreamSynchronize(c->stream);
            if (e != cudaSuccess)
                return cuda_fail(c, e, "train step");
            lsum += l;
            ++c->launches;
        }
        if (epoch_loss)
            epoch_loss[ep] = (float)(lsum / (double)n);
    }
    e = cudaMemcpyAsync(params, c->d_mlp, canon::mlp::N_PARAMS * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess && tc_timed_out(c))
        return fail(c, CANON_ETIMEOUT, "train: a wait for the tensor cores timed out");
    return e == cudaSuccess ? CANON_OK : cuda_fail(c, e, "train");
}

int canon_check_bibd_noalloc(uint32_t n, uint32_t v, uint32_t b, uint32_t flags, const uint64_t *d_rows,
                             const uint8_t *d_nrows, const canon_device_outputs *out, uint64_t max_trials,
                             void *stream) {
    if (n > CANON_NOALLOC_MAX_ITEMS)
        return CANON_ESIZE;
    if (!out || !d_rows || v < 1 || v > canon::VMAX || b < 1 || b > canon::BMAX || (flags & ~0x7Fu))
        return CANON_EINVAL;
    if (!out->canonical || !out->status || !out->reject_row || !out->row_to_change || !out->player_index ||
        !out->witness || !out->aut || !out->trials || !out->n_auts || !out->len_aut)
        return CANON_EINVAL;
    if ((flags & canon::F_SAVE_AUTS) && (!out->auts || !out->aut_cap))
        return CANON_EINVAL;
    if (!n)
        return CANON_OK;
    Outputs o{};
    o.canonical = out->canonical;
    o.status = out->status;
    o.reject_row = out->reject_row;
    o.row_to_change = out->row_to_change;
    o.player_index = out->player_index;
    o.witness = out->witness;
    o.aut = out->aut;
    o.trials = out->trials;
    o.n_auts = out->n_auts;
    o.len_aut = out->len_aut;
    o.auts = (flags & canon::F_SAVE_AUTS) ? out->auts : nullptr;
    o.aut_cap = (flags & canon::F_SAVE_AUTS) ? out->aut_cap : 0;
    const cudaError_t e = canon::launch_bibd_check_noalloc(n, v, b, flags, d_rows, d_nrows, o,
                                                           max_trials ? max_trials : (1ull << 28),
                                                           (cudaStream_t)stream);
    return e == cudaSuccess ? CANON_OK : CANON_ECUDA;
}

}  // extern "C"

namespace canon {

// Candidates per warp task of a k-system check.  A matrix whose rounds are all
// canonical tries every one of its ng! * 2^ng * rounds relabelings, so a batch of
// fewer matrices than the GPU holds warps leaves it mostly idle with one warp per
// matrix; ksys_auto_segment cuts the candidates into segments.
uint32_t ksys_segment(const canon_ctx *c, uint64_t n, uint32_t np, uint32_t rounds) {
    if (c->ksys_seg == CANON_KSYS_WHOLE || !n || !np || !rounds)
        return 0;
    const uint64_t total = ksys_candidates(np, rounds);
    const uint64_t seg = c->ksys_seg ? (((uint64_t)c->ksys_seg + 31u) & ~31ull)
                                     : ksys_auto_segment(n, total, (uint32_t)(c->num_sms > 0 ? c->num_sms : 1) *
                                                                       KSYS_RESIDENT_WARPS_PER_SM);
    return seg >= total ? 0u : (uint32_t)seg;
}

// Candidates per warp task of the check with groups of 3 or 4 (always segmented: a
// canonical KTS(15) tries 6,531,840 relabelings); CANON_KSYS_WHOLE = one segment per item.
// The automatic size is capped at KGEN_SEGMENT_MAX: in an enumeration level most matrices
// are rejected within their first relabelings, so the work is the few canonical ones, and
// a segment sized as if every matrix tried all its relabelings would leave each of those to
// a handful of warps (a level of 13,824 matrices of 16 players: 2.8M-relabeling segments).
constexpr uint64_t KGEN_SEGMENT_MAX = 65536;
uint32_t kgen_segment(const canon_ctx *c, uint64_t n, uint64_t total) {
    const uint64_t whole = (total + 31) & ~31ull;
    uint64_t seg = c->ksys_seg == CANON_KSYS_WHOLE ? whole
                   : c->ksys_seg ? (((uint64_t)c->ksys_seg + 31u) & ~31ull)
                                 : std::min<uint64_t>(
                                       KGEN_SEGMENT_MAX,
                                       ksys_auto_segment(n, total, (uint32_t)(c->num_sms > 0 ? c->num_sms : 1) *
                                                                       KSYS_RESIDENT_WARPS_PER_SM));
    return (uint32_t)(seg < whole ? seg : whole);
}

// The largest batch of matrices with `words` 64-bit words (BIBD) or `bytes` bytes
// (k-systems) each that one canon_submit_* call can queue on an empty context.
uint32_t batch_capacity(const canon_ctx *c, uint32_t words, uint32_t bytes) {
    uint64_t n = c->cfg.max_items;
    if (words && c->cfg.max_words / words < n)
        n = c->cfg.max_words / words;
    if (bytes && c->max_bytes / bytes < n)
        n = c->max_bytes / bytes;
    return (uint32_t)n;
}

}  // namespace canon
