// canon_kbin.cu -- the canonical binary matrix of k-systems on sm_103a, and the
// reference's plugin entry points createCanonizer / runCanonizer / releaseCanonizer
// (k-Factorization/Utils/Include/CDTools.h:9-11, Source/CDTools.cpp:5-52) on top of it.
//
// One thread owns one k-system: it writes the binary matrix as convertToBinaryMatrix()
// does (Source/matrix.h:198-209) and runs the lex-max search of canon_kbin_core.cuh,
// whose result is the matrix CanonizeMatrix(k, NULL, numClasses) converges to
// (Source/MatrixCanonChecker.cpp:420-564).  The search state (under 600 bytes) lives
// in the thread's local memory; the work is one search per k-system, as the plugin is
// called once per partial matrix.
#include <cstring>
#include <new>

#include "../../include/canon_gb300.h"
#include "canon_ctx.h"
#include "canon_kbin_core.cuh"

namespace {

constexpr int KB_TPB = 64;

// data: n k-systems of `days` rounds x np bytes (result() rows, groups of k);
// out: n x np x (days * np / k) bytes; aut (optional): labelings reaching the form
__global__ void __launch_bounds__(KB_TPB) kbin_kernel(uint32_t n, uint32_t np, uint32_t k, uint32_t days,
                                                      int free_days, const uint8_t *__restrict__ data, uint8_t *out,
                                                      uint64_t *aut, uint8_t *status, uint64_t max_nodes) {
    using namespace canon::kbin;
    const uint32_t g = np / k, b = days * g;
    for (uint32_t it = blockIdx.x * blockDim.x + threadIdx.x; it < n; it += gridDim.x * blockDim.x) {
        const uint8_t *R = data + (size_t)it * days * np;
        uint64_t rows[KB_VMAX] = {};
        bool ok = true;
        for (uint32_t d = 0; d < days; ++d) {
            unsigned seen = 0;
            for (uint32_t q = 0; q < np; ++q) {
                const uint32_t p = R[d * np + q];
                if (p >= np || ((seen >> p) & 1u)) {
                    ok = false;
                    break;
                }
                seen |= 1u << p;
                rows[p] |= 1ull << (d * g + q / k);
            }
        }
        uint8_t *o = out + (size_t)it * np * b;
        uint8_t st = 0;
        uint64_t leaves = 0;
        if (!ok) {
            st = canon::ST_BADINPUT;
        } else {
            Search S;
            S.sh = Shape{(int)np, (int)b, (int)g, (int)days, free_days != 0};
            const Result r = canonize(S, rows, max_nodes);
            if (r.timeout) {
                st = canon::ST_TIMEOUT;
            } else {
                leaves = r.leaves;
                for (uint32_t i = 0; i < np; ++i)
                    for (uint32_t c = 0; c < b; ++c)
                        o[i * b + c] = (uint8_t)((S.bound[i] >> c) & 1ull);
            }
        }
        if (st)
            for (uint32_t q = 0; q < np * b; ++q)
                o[q] = 0;
        if (aut)
            aut[it] = leaves;
        if (status)
            status[it] = st;
    }
}

int fail(canon_ctx *c, int rc, const char *msg) {
    if (c)
        c->err = msg;
    return rc;
}

}  // namespace

extern "C" {

int canon_canonize_ksys_binary_groups(canon_ctx *c, uint32_t n, uint32_t np, uint32_t k, uint32_t days,
                                      const uint8_t *data, uint8_t *out, uint64_t *aut_out) {
    if (!c || (n && (!data || !out)))
        return fail(c, CANON_EINVAL, "canonize k-system: null argument");
    if (k < 2 || k > 4 || np % k || (np - 1) % (k - 1) || np < 3 * k || np > (uint32_t)canon::kbin::KB_VMAX)
        return fail(c, CANON_EINVAL, "canonize k-system: need groups of 2, 3 or 4 and np <= 16 a multiple of "
                                     "the group size with (np-1) a multiple of k-1");
    const uint32_t num_days = (np - 1) / (k - 1);
    if (days < 2 || days > num_days || days * (np / k) > (uint32_t)canon::kbin::KB_BMAX)
        return fail(c, CANON_EINVAL, "canonize k-system: need 2 <= days <= (np-1)/(k-1), days * np/k <= 63");
    if (!n)
        return CANON_OK;
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    const uint32_t b = days * (np / k);
    const size_t in_bytes = (size_t)n * days * np, out_bytes = (size_t)n * np * b;
    uint8_t *d_in = nullptr, *d_out = nullptr, *d_st = nullptr;
    uint64_t *d_aut = nullptr;
    cudaError_t e = cudaMalloc((void **)&d_in, in_bytes);
    if (e == cudaSuccess)
        e = cudaMalloc((void **)&d_out, out_bytes);
    if (e == cudaSuccess)
        e = cudaMalloc((void **)&d_aut, (size_t)n * 8);
    if (e == cudaSuccess)
        e = cudaMalloc((void **)&d_st, n);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_in, data, in_bytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        int grid = (int)((n + KB_TPB - 1) / KB_TPB);
        const int cap = 8 * (c->num_sms > 0 ? c->num_sms : 1);
        if (grid > cap)
            grid = cap;
        cudaEventRecord(c->ev0, s);
        kbin_kernel<<<grid, KB_TPB, 0, s>>>(n, np, k, days, days == num_days ? 1 : 0, d_in, d_out, d_aut, d_st,
                                            c->cfg.max_trials);
        e = cudaGetLastError();
        cudaEventRecord(c->ev1, s);
        ++c->launches;
    }
    std::vector<uint8_t> st(n);
    std::vector<uint64_t> aut(n);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, d_out, out_bytes, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(aut.data(), d_aut, (size_t)n * 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(st.data(), d_st, n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    if (e == cudaSuccess)
        cudaEventElapsedTime(&c->last_ms, c->ev0, c->ev1);
    cudaFree(d_in);
    cudaFree(d_out);
    cudaFree(d_aut);
    cudaFree(d_st);
    if (e != cudaSuccess) {
        c->err = std::string("canonize k-system: ") + cudaGetErrorString(e);
        return CANON_ECUDA;
    }
    int rc = CANON_OK;
    for (uint32_t i = 0; i < n; ++i) {
        if (st[i] & canon::ST_BADINPUT)
            rc = fail(c, CANON_EINVAL, "canonize k-system: a round is not a partition of the players");
        else if (st[i] & canon::ST_TIMEOUT && rc == CANON_OK)
            rc = fail(c, CANON_ETIMEOUT, "canonize k-system: the search hit its node budget");
    }
    if (aut_out)
        std::memcpy(aut_out, aut.data(), (size_t)n * 8);
    return rc;
}

int canon_canonize_ksys_binary(canon_ctx *c, uint32_t n, uint32_t np, uint32_t days, const uint8_t *data,
                               uint8_t *out, uint64_t *aut_out) {
    if (c && (np & 1u))
        return fail(c, CANON_EINVAL, "canonize k-system: need np even in 6..16, 2 <= days <= np-1, "
                                     "days * np/2 <= 63");
    return canon_canonize_ksys_binary_groups(c, n, np, 2, days, data, out, aut_out);
}

// ---- the reference's plugin ----------------------------------------------------
// createCanonizer(v, k) prepares the canonizer of k-systems of v players in groups of
// k (the C_InSys of v+1 rows and numDays*v/k columns, CDTools.cpp:5-14); here, a
// context on the first GPU and a result buffer.  Groups of 2, 3 or 4.
struct KsysCanonizer {
    canon_ctx *ctx;
    int v, k, num_days;
    uint8_t *result;        // v x b bytes of the last call's canonical matrix
};

void *createCanonizer(int v, int k) {
    if (k < 2 || k > 4 || v < 3 * k || v > canon::kbin::KB_VMAX || (v % k) || (v - 1) % (k - 1))
        return nullptr;
    const int num_days = (v - 1) / (k - 1);
    if (num_days * (v / k) > canon::kbin::KB_BMAX)
        return nullptr;
    canon_cfg cfg{};
    cfg.device = 0;
    cfg.max_items = 16;
    canon_ctx *ctx = canon_create(&cfg);
    if (!ctx)
        return nullptr;
    KsysCanonizer *h = new (std::nothrow) KsysCanonizer{ctx, v, k, num_days, nullptr};
    if (h)
        h->result = new (std::nothrow) uint8_t[(size_t)v * num_days * (v / k)];
    if (!h || !h->result) {
        if (h)
            delete h;
        canon_destroy(ctx);
        return nullptr;
    }
    return h;
}

void releaseCanonizer(void *pCanonizer) {
    if (!pCanonizer)
        return;
    KsysCanonizer *h = static_cast<KsysCanonizer *>(pCanonizer);
    canon_destroy(h->ctx);
    delete[] h->result;
    delete h;
}

// runCanonizer(h, pMatrix, k, dayNumb): the canonical binary matrix of the first
// dayNumb rounds of pMatrix (all numDays rounds when dayNumb <= 0), as rows 1..v of
// the canonised C_InSys (CDTools.cpp:25-52): v rows of dayNumb*v/k bytes.  The
// returned buffer belongs to the canonizer and is overwritten by its next call;
// nullptr on error (the reference's convention).
const unsigned char *runCanonizer(void *pCanonizer, const unsigned char *pMatrix, int k, int iDay) {
    if (!pCanonizer || !pMatrix)
        return nullptr;
    KsysCanonizer *h = static_cast<KsysCanonizer *>(pCanonizer);
    if (k != h->k)
        return nullptr;
    const int days = iDay <= 0 ? h->num_days : iDay;
    if (days < 2 || days > h->num_days)
        return nullptr;
    const int rc = canon_canonize_ksys_binary_groups(h->ctx, 1, (uint32_t)h->v, (uint32_t)h->k, (uint32_t)days,
                                                     pMatrix, h->result, nullptr);
    return rc == CANON_OK ? h->result : nullptr;
}

}  // extern "C"
