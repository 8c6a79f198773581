// canon_levels.cu -- BIBD enumeration with every level resident in HBM.
//
// The reference enumerates depth-first and checks one partial matrix at a time
// (CEnumerator::Enumerate, Source/Enumerator.cpp:540-1024; checks at :446-447 for
// partial and :364 for complete matrices).  Here a whole level lives on the GPU:
//   1. rows_count_kernel: one thread per canonical parent counts its admissible
//      next rows (canon_rows.cuh) and keeps the first 16;
//   2. an exclusive scan turns the counts into output offsets;
//   3. rows_emit_kernel writes every child (the parent's rows and the new row),
//      parents in order, children in the generator's order (copied from the kept
//      rows, generated again only for parents with more than 16 children);
//   4. the check kernel flags the canonical children: bibd_uniform_kernel
//      (verdict only), or for small slices bibd_split_kernel, the lex-max search
//      split over one thread per (child, first row);
//   5. a scan of the flags and compact_kernel pack them into the next level.
// The host reads one count per level (and per slice when a level is split to
// bound memory) and, at the end, the complete designs.  Orderly generation makes
// the result independent of the visiting order: every prefix of a canonical
// matrix is canonical, so the canonical complete matrices are exactly those the
// depth-first search finds; the order is that of the host-generated levels.
#include <chrono>
#include <cstring>
#include <vector>

#include "../../include/canon_gb300.h"
#include "canon_ctx.h"
#include "canon_internal.h"
#include "canon_rows.cuh"

namespace {

constexpr int GEN_TPB = 128;
constexpr int SCAN_TPB = 256;
constexpr int SCAN_PER_THREAD = 16;
constexpr int SCAN_TILE = SCAN_TPB * SCAN_PER_THREAD;
// candidates checked per slice: bounds the device memory of one level
constexpr uint64_t SLICE_CAP = 1ull << 24;
// slices up to this size are checked with the search split by first row (one
// thread per matrix and first row): small levels are latency bound
constexpr uint64_t SPLIT_MAX = 1ull << 14;

template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t cap = 0;
    // at least n elements; the contents are not kept
    cudaError_t ensure(size_t n) {
        if (n <= cap)
            return cudaSuccess;
        cudaFree(p);
        p = nullptr;
        cap = 0;
        const size_t want = n + n / 4 + 1024;
        const cudaError_t e = cudaMalloc(&p, want * sizeof(T));
        if (e == cudaSuccess)
            cap = want;
        return e;
    }
    void swap(DevBuf &o) {
        T *tp = p;
        p = o.p;
        o.p = tp;
        const size_t tc = cap;
        cap = o.cap;
        o.cap = tc;
    }
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { cudaFree(p); }
};

// new rows kept per parent by the counting pass, so that the emitting pass only
// copies for parents with at most this many children
constexpr uint32_t ROW_CACHE = 16;

__global__ void __launch_bounds__(GEN_TPB) rows_count_kernel(canon::rows::Params d, const uint64_t *parents,
                                                             uint32_t n_par, int n, uint32_t *counts,
                                                             uint64_t *cache, unsigned *ticket) {
    for (;;) {
        const unsigned p = atomicAdd(ticket, 1u);
        if (p >= n_par)
            break;
        counts[p] = canon::rows::children<canon::rows::NEW_ROW>(d, parents + (size_t)p * n, n,
                                                               cache + (size_t)p * ROW_CACHE, ROW_CACHE);
    }
}

__global__ void __launch_bounds__(GEN_TPB) rows_emit_kernel(canon::rows::Params d, const uint64_t *parents,
                                                            uint32_t p0, uint32_t p1, int n,
                                                            const uint64_t *offsets, const uint32_t *counts,
                                                            const uint64_t *cache, uint64_t *out,
                                                            unsigned *ticket) {
    const uint64_t base = offsets[p0];
    for (;;) {
        const unsigned p = p0 + atomicAdd(ticket, 1u);
        if (p >= p1)
            break;
        const uint32_t cnt = counts[p];
        const uint64_t *par = parents + (size_t)p * n;
        uint64_t *dst = out + (offsets[p] - base) * (n + 1);
        if (cnt <= ROW_CACHE) {
            for (uint32_t j = 0; j < cnt; ++j) {
                for (int i = 0; i < n; ++i)
                    dst[(size_t)j * (n + 1) + i] = par[i];
                dst[(size_t)j * (n + 1) + n] = cache[(size_t)p * ROW_CACHE + j];
            }
        } else {
            canon::rows::children<canon::rows::CHILD>(d, par, n, dst, cnt);
        }
    }
}

// exclusive scan of one 256-thread block; *total gets the block's sum
__device__ uint64_t block_exclusive_scan(uint64_t x, uint64_t *total) {
    __shared__ uint64_t warp_sums[SCAN_TPB / 32];
    const unsigned lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    uint64_t incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= (unsigned)o)
            incl += y;
    }
    if (lane == 31)
        warp_sums[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        uint64_t w = lane < SCAN_TPB / 32 ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < SCAN_TPB / 32; o <<= 1) {
            const uint64_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
            if (lane >= (unsigned)o)
                w += y;
        }
        if (lane < SCAN_TPB / 32)
            warp_sums[lane] = w;
    }
    __syncthreads();
    const uint64_t res = (wid ? warp_sums[wid - 1] : 0) + incl - x;
    *total = warp_sums[SCAN_TPB / 32 - 1];
    __syncthreads();
    return res;
}

// pass 1: the sum of every tile of SCAN_TILE inputs
template <typename T>
__global__ void __launch_bounds__(SCAN_TPB) tile_sums_kernel(const T *in, uint64_t n, uint64_t *sums) {
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_PER_THREAD;
    uint64_t s = 0;
    for (int j = 0; j < SCAN_PER_THREAD; ++j)
        if (base + j < n)
            s += in[base + j];
    uint64_t total;
    block_exclusive_scan(s, &total);
    if (threadIdx.x == 0)
        sums[blockIdx.x] = total;
}

// pass 2 (one block): exclusive scan of the tile sums in place; sums[ntiles] = total
__global__ void __launch_bounds__(SCAN_TPB) scan_sums_kernel(uint64_t *sums, uint32_t ntiles) {
    uint64_t carry = 0;
    for (uint32_t b0 = 0; b0 < ntiles; b0 += SCAN_TPB) {
        const uint32_t i = b0 + threadIdx.x;
        const uint64_t x = i < ntiles ? sums[i] : 0;
        uint64_t total;
        const uint64_t ex = block_exclusive_scan(x, &total);
        if (i < ntiles)
            sums[i] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0)
        sums[ntiles] = carry;
}

// pass 3: exclusive offsets of every input; out[n] = total
template <typename T>
__global__ void __launch_bounds__(SCAN_TPB) tile_scan_kernel(const T *in, uint64_t n, const uint64_t *sums,
                                                             uint32_t ntiles, uint64_t *out) {
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_PER_THREAD;
    uint64_t v[SCAN_PER_THREAD];
    uint64_t s = 0;
    for (int j = 0; j < SCAN_PER_THREAD; ++j) {
        v[j] = (base + j < n) ? (uint64_t)in[base + j] : 0;
        s += v[j];
    }
    uint64_t total;
    uint64_t run = sums[blockIdx.x] + block_exclusive_scan(s, &total);
    for (int j = 0; j < SCAN_PER_THREAD; ++j) {
        if (base + j < n)
            out[base + j] = run;
        run += v[j];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
        out[n] = sums[ntiles];
}

// the canonical children of a slice into the next level (rows) and, for complete
// matrices, their |Aut|; a search that ran out of budget raises *timeout
__global__ void compact_kernel(uint64_t n_cand, int m, const uint64_t *cand, const uint8_t *canonical,
                               const uint8_t *status, const uint64_t *aut, const uint64_t *offs, uint64_t *dst,
                               uint64_t *aut_dst, unsigned *timeout) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_cand; i += stride) {
        if (status[i] & canon::ST_TIMEOUT)
            atomicOr(timeout, 1u);
        if (!canonical[i])
            continue;
        const uint64_t o = offs[i];
        for (int r = 0; r < m; ++r)
            dst[o * m + r] = cand[i * m + r];
        if (aut_dst) {
            aut_dst[2 * o] = aut[2 * i];
            aut_dst[2 * o + 1] = aut[2 * i + 1];
        }
    }
}

template <typename T>
cudaError_t exclusive_scan(const T *in, uint64_t n, uint64_t *out, DevBuf<uint64_t> &sums, cudaStream_t s) {
    const uint32_t ntiles = (uint32_t)((n + SCAN_TILE - 1) / SCAN_TILE);
    cudaError_t e = sums.ensure((size_t)ntiles + 1);
    if (e != cudaSuccess)
        return e;
    if (ntiles) {
        tile_sums_kernel<T><<<ntiles, SCAN_TPB, 0, s>>>(in, n, sums.p);
        scan_sums_kernel<<<1, SCAN_TPB, 0, s>>>(sums.p, ntiles);
        tile_scan_kernel<T><<<ntiles, SCAN_TPB, 0, s>>>(in, n, sums.p, ntiles, out);
    } else {
        cudaMemsetAsync(out, 0, sizeof(uint64_t), s);
    }
    return cudaGetLastError();
}

cudaError_t read_u64(const uint64_t *d, uint64_t *h, cudaStream_t s) {
    cudaError_t e = cudaMemcpyAsync(h, d, sizeof(uint64_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    return e;
}

int gen_grid(const void *kernel, int num_sms, uint64_t work) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, GEN_TPB, 0);
    if (per_sm < 1)
        per_sm = 1;
    uint64_t g = (uint64_t)per_sm * (num_sms > 0 ? num_sms : 1);
    const uint64_t need = (work + GEN_TPB - 1) / GEN_TPB;
    if (g > need)
        g = need;
    return (int)(g ? g : 1);
}

}  // namespace

extern "C" int canon_enumerate_bibd(canon_ctx *c, uint32_t v, uint32_t b, uint32_t r, uint32_t k, uint32_t lambda,
                                    canon_design_cb cb, void *user, canon_enum_stats *stats) {
    if (!c || v < 2 || v > canon::VMAX || b < 1 || b > canon::BMAX || r < 1 || r > b || k < 1 || k > v)
        return CANON_EINVAL;
    const auto t0 = std::chrono::steady_clock::now();
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    canon_enum_stats st{};
    const canon::rows::Params prm{(int)v, (int)b, (int)r, (int)k, (int)lambda};
    DevBuf<uint64_t> lev, next, cand, offs, coffs, sums, aut, aut_out, rcache;
    DevBuf<uint32_t> counts;
    DevBuf<uint8_t> can, status;
    DevBuf<unsigned> ticket, stop;
    DevBuf<canon::SplitPart> parts;
    cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventCreate(&e2);
    auto done = [&](int rc, const char *what, cudaError_t e) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaEventDestroy(e2);
        if (rc != CANON_OK) {
            c->err = std::string("enumerate: ") + what + (e != cudaSuccess ? std::string(": ") + cudaGetErrorString(e)
                                                                           : std::string());
        }
        return rc;
    };
    cudaError_t e = ticket.ensure(2);
    // level 1: row 0 is forced, r ones first
    const uint64_t row0 = (r >= 64) ? ~0ull : ((1ull << r) - 1ull);
    if (e == cudaSuccess)
        e = lev.ensure(1);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(lev.p, &row0, sizeof(uint64_t), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess)
        return done(CANON_ECUDA, "setup", e);
    uint64_t n_par = 1;
    uint32_t n = 1;
    while (n < v && n_par) {
        const uint32_t m = n + 1;
        const bool complete = m == v;
        // 1-2: children per parent and their offsets
        e = counts.ensure(n_par);
        if (e == cudaSuccess)
            e = offs.ensure(n_par + 1);
        if (e == cudaSuccess)
            e = rcache.ensure((size_t)n_par * ROW_CACHE);
        if (e != cudaSuccess)
            return done(CANON_ENOMEM, "level buffers", e);
        cudaEventRecord(e0, s);
        cudaMemsetAsync(ticket.p, 0, sizeof(unsigned), s);
        rows_count_kernel<<<gen_grid((const void *)rows_count_kernel, c->num_sms, n_par), GEN_TPB, 0, s>>>(
            prm, lev.p, (uint32_t)n_par, (int)n, counts.p, rcache.p, ticket.p);
        e = exclusive_scan(counts.p, n_par, offs.p, sums, s);
        uint64_t n_cand = 0;
        if (e == cudaSuccess)
            e = read_u64(offs.p + n_par, &n_cand, s);
        if (e != cudaSuccess)
            return done(CANON_ECUDA, "count", e);
        float ms = 0.f;
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        st.gen_seconds += ms * 1e-3;
        c->launches += 4;
        // the canonical children of all slices, packed
        e = next.ensure((size_t)(n_cand ? n_cand : 1) * m);
        if (e == cudaSuccess && complete)
            e = aut_out.ensure((size_t)(n_cand ? n_cand : 1) * 2);
        if (e != cudaSuccess)
            return done(CANON_ENOMEM, "next level", e);
        uint64_t n_next = 0;
        uint64_t p0 = 0;
        while (p0 < n_par) {
            // the largest slice of parents whose children fit SLICE_CAP (at least one parent)
            uint64_t base = 0, p1 = n_par, end = n_cand;
            e = read_u64(offs.p + p0, &base, s);
            if (e == cudaSuccess && n_cand - base > SLICE_CAP) {
                uint64_t lo = p0 + 1, hi = n_par;
                while (lo < hi) {
                    const uint64_t mid = (lo + hi + 1) / 2;
                    uint64_t at = 0;
                    e = read_u64(offs.p + mid, &at, s);
                    if (e != cudaSuccess)
                        break;
                    if (at - base <= SLICE_CAP)
                        lo = mid;
                    else
                        hi = mid - 1;
                }
                p1 = lo;
                if (e == cudaSuccess)
                    e = read_u64(offs.p + p1, &end, s);
            }
            if (e != cudaSuccess)
                return done(CANON_ECUDA, "slice", e);
            const uint64_t ns = end - base;
            e = cand.ensure((size_t)(ns ? ns : 1) * m);
            if (e == cudaSuccess)
                e = can.ensure(ns ? ns : 1);
            if (e == cudaSuccess)
                e = status.ensure(ns ? ns : 1);
            if (e == cudaSuccess)
                e = coffs.ensure(ns + 1);
            if (e == cudaSuccess && complete)
                e = aut.ensure((size_t)(ns ? ns : 1) * 2);
            if (e != cudaSuccess)
                return done(CANON_ENOMEM, "slice buffers", e);
            // 3: the children of parents [p0, p1)
            cudaEventRecord(e0, s);
            cudaMemsetAsync(ticket.p, 0, sizeof(unsigned), s);
            rows_emit_kernel<<<gen_grid((const void *)rows_emit_kernel, c->num_sms, p1 - p0), GEN_TPB, 0, s>>>(
                prm, lev.p, (uint32_t)p0, (uint32_t)p1, (int)n, offs.p, counts.p, rcache.p, cand.p, ticket.p);
            cudaEventRecord(e1, s);
            // 4: the verdicts
            if (ns <= SPLIT_MAX) {
                e = parts.ensure((size_t)(ns ? ns : 1) * m);
                if (e == cudaSuccess)
                    e = stop.ensure(ns ? ns : 1);
                if (e == cudaSuccess)
                    e = canon::launch_bibd_check_split((uint32_t)ns, m, b,
                                                       canon::F_VERDICT_ONLY | (complete ? canon::F_COMPLETE : 0u),
                                                       cand.p, can.p, complete ? aut.p : nullptr, status.p, parts.p,
                                                       stop.p, c->cfg.max_trials, c->d_ticket, c->num_sms, s);
            } else {
                e = canon::launch_bibd_check_uniform((uint32_t)ns, m, b,
                                                     canon::F_VERDICT_ONLY | (complete ? canon::F_COMPLETE : 0u),
                                                     cand.p, can.p, nullptr, complete ? aut.p : nullptr, status.p,
                                                     nullptr, c->cfg.max_trials, c->d_ticket, c->num_sms, s);
            }
            cudaEventRecord(e2, s);
            // 5: pack the canonical ones
            if (e == cudaSuccess)
                e = exclusive_scan(can.p, ns, coffs.p, sums, s);
            if (e == cudaSuccess) {
                cudaMemsetAsync(ticket.p + 1, 0, sizeof(unsigned), s);
                const int grid = (int)((ns + 255) / 256 < 4096 ? (ns + 255) / 256 : 4096);
                compact_kernel<<<grid ? grid : 1, 256, 0, s>>>(ns, (int)m, cand.p, can.p, status.p,
                                                               complete ? aut.p : nullptr, coffs.p,
                                                               next.p + n_next * m,
                                                               complete ? aut_out.p + 2 * n_next : nullptr,
                                                               ticket.p + 1);
                e = cudaGetLastError();
            }
            uint64_t n_can = 0;
            unsigned timeout = 0;
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(&timeout, ticket.p + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess)
                e = read_u64(coffs.p + ns, &n_can, s);
            if (e != cudaSuccess)
                return done(CANON_ECUDA, "check", e);
            float gen_ms = 0.f, chk_ms = 0.f;
            cudaEventElapsedTime(&gen_ms, e0, e1);
            cudaEventElapsedTime(&chk_ms, e1, e2);
            st.gen_seconds += gen_ms * 1e-3;
            st.kernel_ms += chk_ms;
            st.level_kernel_ms[m - 1] += chk_ms;
            c->last_ms = chk_ms;
            c->launches += 6;
            ++st.batches;
            if (timeout)
                return done(CANON_ETIMEOUT, "a search hit the trial budget (canon_cfg.max_trials)", cudaSuccess);
            n_next += n_can;
            p0 = p1;
        }
        st.checks += n_cand;
        st.level_checks[m - 1] += n_cand;
        ++st.levels;
        lev.swap(next);
        n_par = n_next;
        n = m;
    }
    if (n == v && n_par) {
        std::vector<uint64_t> rows((size_t)n_par * v), auts((size_t)n_par * 2);
        e = cudaMemcpyAsync(rows.data(), lev.p, rows.size() * sizeof(uint64_t), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(auts.data(), aut_out.p, auts.size() * sizeof(uint64_t), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(s);
        if (e != cudaSuccess)
            return done(CANON_ECUDA, "designs", e);
        st.designs = n_par;
        if (cb)
            for (uint64_t i = 0; i < n_par; ++i)
                cb(user, (const uint8_t *)(rows.data() + i * v), v, b, auts[2 * i], auts[2 * i + 1]);
    }
    st.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (stats)
        *stats = st;
    return done(CANON_OK, "", cudaSuccess);
}
