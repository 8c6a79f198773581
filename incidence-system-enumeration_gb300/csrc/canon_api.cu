// canon_api.cu -- the C ABI (include/canon_gb300.h) over the sm_103a kernels.
//
// A context owns one CUDA stream, pinned host staging for queued batches and
// device buffers sized at creation.  canon_submit_* only appends to the host
// staging; canon_sync copies everything to the GPU in two copies (items, data),
// launches the check kernels on the context's stream, copies the result arrays
// back and waits.  This replaces CGPU_CanonChecker (Source/MatrixCanonChecker.h:
// 204-350), which marshalled one C++ checker object per matrix onto the device
// heap and launched TestCanonicity<<<1, nMatr>>> (Source/CanonicityChecker.cu:152-156).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/canon_gb300.h"
#include "canon_internal.h"

using canon::Item;
using canon::Outputs;

struct canon_ctx {
    int device = 0;
    int num_sms = 0;
    canon_cfg cfg{};
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // queued host input (pinned)
    Item *h_bitems = nullptr, *h_kitems = nullptr;
    uint64_t *h_words = nullptr;
    uint8_t *h_bytes = nullptr;
    uint32_t n_bitems = 0, n_kitems = 0, n_words = 0, n_bytes = 0;
    uint32_t max_bytes = 0;
    // device buffers
    Item *d_bitems = nullptr, *d_kitems = nullptr;
    uint64_t *d_words = nullptr;
    uint8_t *d_bytes = nullptr;
    unsigned *d_ticket = nullptr;      // work-stealing counters (2 words)
    Outputs d_out{}, h_out{};
    std::vector<uint8_t> item_kind;   // per out_idx
    std::string err;
    float last_ms = 0.f;
    uint64_t launches = 0;
};

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
    if (!c)
        return;
    cudaSetDevice(c->device);
    if (c->stream)
        cudaStreamSynchronize(c->stream);
    free_outputs(c->d_out, true);
    free_outputs(c->h_out, false);
    void *dptrs[] = {c->d_bitems, c->d_kitems, c->d_words, c->d_bytes, c->d_ticket};
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
    if (bt->flags & ~0x3Fu)
        return fail(c, CANON_EINVAL, "bibd batch: unknown flags");
    const uint32_t total = c->n_bitems + c->n_kitems;
    if ((uint64_t)total + bt->n > c->cfg.max_items)
        return fail(c, CANON_ENOMEM, "item capacity exceeded (canon_cfg.max_items)");
    if ((uint64_t)c->n_words + (uint64_t)bt->n * bt->v > c->cfg.max_words)
        return fail(c, CANON_ENOMEM, "word capacity exceeded (canon_cfg.max_words)");
    for (uint32_t i = 0; i < bt->n; ++i) {
        const uint32_t nr = bt->nrows ? bt->nrows[i] : bt->v;
        if (nr < 1 || nr > bt->v)
            return fail(c, CANON_EINVAL, "bibd batch: nrows out of range");
    }
    std::memcpy(c->h_words + c->n_words, bt->rows, (size_t)bt->n * bt->v * sizeof(uint64_t));
    for (uint32_t i = 0; i < bt->n; ++i) {
        Item it{};
        it.data_off = c->n_words + i * bt->v;
        it.kind = canon::KIND_BIBD;
        it.nrows = (uint8_t)(bt->nrows ? bt->nrows[i] : bt->v);
        it.ncols = (uint8_t)bt->b;
        it.flags = (uint8_t)bt->flags;
        it.out_idx = total + i;
        c->h_bitems[c->n_bitems + i] = it;
    }
    c->n_words += bt->n * bt->v;
    c->n_bitems += bt->n;
    c->item_kind.insert(c->item_kind.end(), bt->n, canon::KIND_BIBD);
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
    const uint32_t total = c->n_bitems + c->n_kitems;
    const uint64_t bytes = (uint64_t)bt->n * bt->rounds * bt->np;
    if ((uint64_t)total + bt->n > c->cfg.max_items)
        return fail(c, CANON_ENOMEM, "item capacity exceeded (canon_cfg.max_items)");
    if ((uint64_t)c->n_bytes + bytes > c->max_bytes)
        return fail(c, CANON_ENOMEM, "byte capacity exceeded (8 * canon_cfg.max_words)");
    for (uint32_t i = 0; i < bt->n; ++i) {
        const uint32_t nr = bt->nrows ? bt->nrows[i] : bt->rounds;
        if (nr < 1 || nr > bt->rounds)
            return fail(c, CANON_EINVAL, "ksys batch: nrows out of range");
    }
    std::memcpy(c->h_bytes + c->n_bytes, bt->data, bytes);
    for (uint32_t i = 0; i < bt->n; ++i) {
        Item it{};
        it.data_off = c->n_bytes + i * bt->rounds * bt->np;
        it.kind = canon::KIND_KSYS;
        it.nrows = (uint8_t)(bt->nrows ? bt->nrows[i] : bt->rounds);
        it.ncols = (uint8_t)bt->np;
        it.flags = (uint8_t)bt->flags;
        it.out_idx = total + i;
        c->h_kitems[c->n_kitems + i] = it;
    }
    c->n_bytes += (uint32_t)bytes;
    c->n_kitems += bt->n;
    c->item_kind.insert(c->item_kind.end(), bt->n, canon::KIND_KSYS);
    return CANON_OK;
}

int canon_sync(canon_ctx *c, canon_results *r) {
    if (!c || !r)
        return fail(c, CANON_EINVAL, "null argument");
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "cudaSetDevice");
    const uint32_t n = c->n_bitems + c->n_kitems;
    std::memset(r, 0, sizeof(*r));
    if (n) {
        cudaStream_t s = c->stream;
        if (c->n_bitems)
            cudaMemcpyAsync(c->d_bitems, c->h_bitems, c->n_bitems * sizeof(Item), cudaMemcpyHostToDevice, s);
        if (c->n_kitems)
            cudaMemcpyAsync(c->d_kitems, c->h_kitems, c->n_kitems * sizeof(Item), cudaMemcpyHostToDevice, s);
        if (c->n_words)
            cudaMemcpyAsync(c->d_words, c->h_words, c->n_words * sizeof(uint64_t), cudaMemcpyHostToDevice, s);
        if (c->n_bytes)
            cudaMemcpyAsync(c->d_bytes, c->h_bytes, c->n_bytes, cudaMemcpyHostToDevice, s);
        cudaEventRecord(c->ev0, s);
        if (c->n_bitems && c->n_kitems) {
            // uneven batch: one persistent launch for both kinds
            e = canon::launch_mixed_check(c->d_bitems, c->n_bitems, c->d_kitems, c->n_kitems, c->d_words,
                                          c->d_bytes, c->d_out, c->cfg.max_trials, c->d_ticket, c->num_sms, s);
            if (e != cudaSuccess)
                return cuda_fail(c, e, "mixed check launch");
            ++c->launches;
        } else if (c->n_bitems) {
            e = canon::launch_bibd_check(c->d_bitems, c->n_bitems, c->d_words, c->d_out, c->cfg.max_trials,
                                         c->d_ticket, c->num_sms, s);
            if (e != cudaSuccess)
                return cuda_fail(c, e, "bibd check launch");
            ++c->launches;
        } else if (c->n_kitems) {
            e = canon::launch_ksys_check(c->d_kitems, c->n_kitems, c->d_bytes, c->d_out, c->d_ticket + 1,
                                         c->num_sms, s);
            if (e != cudaSuccess)
                return cuda_fail(c, e, "ksys check launch");
            ++c->launches;
        }
        cudaEventRecord(c->ev1, s);
        const Outputs &d = c->d_out, &h = c->h_out;
#define CANON_D2H(field, count) \
    cudaMemcpyAsync(h.field, d.field, (size_t)(count) * sizeof(*h.field), cudaMemcpyDeviceToHost, s)
        CANON_D2H(canonical, n);
        CANON_D2H(status, n);
        CANON_D2H(reject_row, n);
        CANON_D2H(row_to_change, n);
        CANON_D2H(player_index, n);
        CANON_D2H(witness, n * 16);
        CANON_D2H(aut, n * 2);
        CANON_D2H(trials, n);
        CANON_D2H(n_auts, n);
        CANON_D2H(len_aut, n);
#undef CANON_D2H
        bool want_auts = false;
        for (uint32_t i = 0; i < c->n_bitems && !want_auts; ++i)
            want_auts = c->h_bitems[i].flags & canon::F_SAVE_AUTS;
        for (uint32_t i = 0; i < c->n_kitems && !want_auts; ++i)
            want_auts = c->h_kitems[i].flags & canon::F_SAVE_AUTS;
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
    c->item_kind.clear();
    int rc = CANON_OK;
    for (uint32_t i = 0; i < n; ++i)
        if (c->h_out.status[i] & canon::ST_TIMEOUT)
            rc = CANON_ETIMEOUT;
    if (rc != CANON_OK)
        c->err = "a search hit the trial budget (canon_cfg.max_trials)";
    return rc;
}

int canon_set_ordering(canon_ctx *c, const canon_mlp_weights *w) {
    if (!c)
        return CANON_EINVAL;
    if (w)
        return fail(c, CANON_EINVAL, "learned ordering is not available in this build");
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

int canon_check_bibd_device(canon_ctx *c, uint32_t n, uint32_t v, uint32_t b, uint32_t flags,
                            const uint64_t *d_rows, uint8_t *d_canonical, uint8_t *d_witness16, uint64_t *d_aut,
                            uint8_t *d_status, uint64_t *d_trials, void *stream) {
    if (!c || !d_rows || !d_canonical)
        return fail(c, CANON_EINVAL, "null argument");
    if (v < 1 || v > canon::VMAX || b < 1 || b > canon::BMAX || (flags & ~0x37u))
        return fail(c, CANON_EINVAL,
                    "check: need 1 <= v <= 16, 1 <= b <= 63, flags in COMPLETE|RAW|FULL_AUT|AUT_CANON|"
                    "REFERENCE_ORDER");
    cudaSetDevice(c->device);
    cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
    cudaEventRecord(c->ev0, s);
    cudaError_t e = canon::launch_bibd_check_uniform(n, v, b, flags, d_rows, d_canonical, d_witness16, d_aut,
                                                     d_status, d_trials, c->cfg.max_trials, c->d_ticket,
                                                     c->num_sms, s);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "check launch");
    ++c->launches;
    cudaEventRecord(c->ev1, s);
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

int canon_check_bibd_noalloc(uint32_t n, uint32_t v, uint32_t b, uint32_t flags, const uint64_t *d_rows,
                             const uint8_t *d_nrows, const canon_device_outputs *out, uint64_t max_trials,
                             void *stream) {
    if (n > CANON_NOALLOC_MAX_ITEMS)
        return CANON_ESIZE;
    if (!out || !d_rows || v < 1 || v > canon::VMAX || b < 1 || b > canon::BMAX || (flags & ~0x3Fu))
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
