// canon_levels.cu -- BIBD enumeration, level by level, checks and compaction on the GPU.
//
// The reference enumerates depth-first and checks one partial matrix at a time
// (CEnumerator::Enumerate, Source/Enumerator.cpp:540-1024; checks at :446-447 for
// partial and :364 for complete matrices).  Here a whole level is handled at once:
//   1. the admissible next rows of every canonical parent (canon_rows.cuh) are
//      counted, prefix-summed and written in order -- parents in order, children
//      in the generator's order, so the result does not depend on where or on
//      how many threads they are made: levels of fewer than 128K parents on all
//      host cores into pinned memory, larger levels on the GPU (rows_count_kernel,
//      a scan, rows_emit_kernel), one thread per parent;
//   2. the candidates are checked in slices of at most 16M matrices;
//   3. the check kernel flags the canonical ones: bibd_uniform_kernel (verdict
//      only), or for small slices bibd_split_kernel, the lex-max search split
//      over one thread per (candidate, first row);
//   4. a scan of the flags and compact_kernel pack them into the next level.
// The row generator is a serial depth-first search whose path differs from
// parent to parent; on the GPU the 32 threads of a warp run 32 such paths one
// after another.  A level of BIBD(8,28,14,4,6) (5,328 parents) took 296 ms there
// against under 1 ms on one host core, while the levels of millions of heavy
// searches of BIBD(12,22,11,6,5) took 2.7 s on the GPU against 17 s on 16 host
// cores; hence the split by level size.  Orderly
// generation makes the result independent of the visiting order: every prefix
// of a canonical matrix is canonical, so the canonical complete matrices are
// exactly those the depth-first search finds.

#include <algorithm>
#include <chrono>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/canon_gb300.h"
#include "canon_ctx.h"
#include "canon_internal.h"
#include "canon_hostpool.h"
#include "canon_rows.cuh"
#include "canon_ksys_rounds.cuh"

namespace {

constexpr int SCAN_TPB = 256;
constexpr int SCAN_PER_THREAD = 16;
constexpr int SCAN_TILE = SCAN_TPB * SCAN_PER_THREAD;
// candidates checked per slice: bounds the device memory of one level
constexpr uint64_t SLICE_CAP = 1ull << 24;
constexpr int GEN_TPB = 128;
// levels with at least this many parents generate their children on the GPU
// (enough independent searches to fill it); smaller ones on the host cores.  On
// BIBD(12,22,11,6,5) a level of ~10K parents took 79 ms on 16 host cores against 170 ms
// on the GPU, one of ~60K parents 1.15 s against 0.14 s.
constexpr uint64_t DEVICE_GEN_MIN = 1ull << 14;
// slices up to this size are checked with the search split by first row (one
// thread per matrix and first row): small levels are latency bound
constexpr uint64_t SPLIT_MAX = 1ull << 16;

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
        // at least double, so a growing enumeration reallocates (and synchronises) rarely;
        // if that much does not fit, exactly what is needed (plus a little)
        size_t want = (n > 2 * cap ? n : 2 * cap) + 1024;
        cap = 0;
        cudaError_t e = cudaMalloc(&p, want * sizeof(T));
        if (e == cudaErrorMemoryAllocation && want > n + 1024) {
            (void)cudaGetLastError();   // clear the failed request before the retry
            p = nullptr;
            want = n + 1024;
            e = cudaMalloc(&p, want * sizeof(T));
        }
        if (e == cudaSuccess)
            cap = want;
        else
            p = nullptr;
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
// copies for parents with at most that many children: up to ROW_CACHE_MAX rows a
// parent while the cache stays within ROW_CACHE_BYTES, at least ROW_CACHE_MIN
constexpr uint32_t ROW_CACHE_MIN = 16, ROW_CACHE_MAX = 64;
constexpr uint64_t ROW_CACHE_BYTES = 4ull << 30;
uint32_t row_cache_rows(uint64_t n_par) {
    const uint64_t fit = ROW_CACHE_BYTES / (8 * (n_par ? n_par : 1));
    return fit >= ROW_CACHE_MAX ? ROW_CACHE_MAX : (fit <= ROW_CACHE_MIN ? ROW_CACHE_MIN : (uint32_t)fit);
}

// gens / ngens: automorphisms of every parent that prune its children (none if null)
__global__ void __launch_bounds__(GEN_TPB) rows_count_kernel(canon::rows::Params d, const uint64_t *parents,
                                                             uint32_t n_par, int n, uint32_t *counts,
                                                             uint64_t *cache, uint32_t cache_rows, unsigned *ticket,
                                                             const uint64_t *gens, const uint8_t *ngens) {
    for (;;) {
        const unsigned p = atomicAdd(ticket, 1u);
        if (p >= n_par)
            break;
        counts[p] = canon::rows::children<canon::rows::NEW_ROW>(
            d, parents + (size_t)p * n, n, cache + (size_t)p * cache_rows, cache_rows,
            gens ? gens + (size_t)p * canon::rows::AUT_GENS : nullptr, gens ? ngens[p] : 0);
    }
}

__global__ void __launch_bounds__(GEN_TPB) rows_emit_kernel(canon::rows::Params d, const uint64_t *parents,
                                                            uint32_t p0, uint32_t p1, int n,
                                                            const uint64_t *offsets, const uint32_t *counts,
                                                            const uint64_t *cache, uint32_t cache_rows, uint64_t *out,
                                                            unsigned *ticket, const uint64_t *gens,
                                                            const uint8_t *ngens) {
    const uint64_t base = offsets[p0];
    for (;;) {
        const unsigned p = p0 + atomicAdd(ticket, 1u);
        if (p >= p1)
            break;
        const uint32_t cnt = counts[p];
        const uint64_t *par = parents + (size_t)p * n;
        uint64_t *dst = out + (offsets[p] - base) * (n + 1);
        if (cnt <= cache_rows) {
            for (uint32_t j = 0; j < cnt; ++j) {
                for (int i = 0; i < n; ++i)
                    dst[(size_t)j * (n + 1) + i] = par[i];
                dst[(size_t)j * (n + 1) + n] = cache[(size_t)p * cache_rows + j];
            }
        } else {
            canon::rows::children<canon::rows::CHILD>(d, par, n, dst, cnt,
                                                      gens ? gens + (size_t)p * canon::rows::AUT_GENS : nullptr,
                                                      gens ? ngens[p] : 0);
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
__device__ void scan_sums_body(uint64_t *sums, uint32_t ntiles) {
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

__global__ void __launch_bounds__(SCAN_TPB) scan_sums_kernel(uint64_t *sums, uint32_t ntiles) {
    scan_sums_body(sums, ntiles);
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
        e = cudaMemsetAsync(out, 0, sizeof(uint64_t), s);
        if (e != cudaSuccess)
            return e;
    }
    return cudaGetLastError();
}

// The exclusive scan of `*d_n` inputs (the count in device memory, at most cap):
// out[i] for i < n and out[n] = the total.  Grids are sized by cap; tiles past the
// count do nothing.  sums holds cap / SCAN_TILE + 2 words.
template <typename T>
__global__ void __launch_bounds__(SCAN_TPB) tile_sums_dev_kernel(const T *in, const uint64_t *d_n, uint64_t *sums) {
    const uint64_t n = *d_n;
    if ((uint64_t)blockIdx.x * SCAN_TILE >= n)
        return;
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

__global__ void __launch_bounds__(SCAN_TPB) scan_sums_dev_kernel(uint64_t *sums, const uint64_t *d_n) {
    scan_sums_body(sums, (uint32_t)((*d_n + SCAN_TILE - 1) / SCAN_TILE));
}

template <typename T>
__global__ void __launch_bounds__(SCAN_TPB) tile_scan_dev_kernel(const T *in, const uint64_t *d_n,
                                                                 const uint64_t *sums, uint64_t *out) {
    const uint64_t n = *d_n;
    const uint32_t ntiles = (uint32_t)((n + SCAN_TILE - 1) / SCAN_TILE);
    if (blockIdx.x == 0 && threadIdx.x == 0)
        out[n] = sums[ntiles];
    if (blockIdx.x >= ntiles)
        return;
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
}

template <typename T>
cudaError_t exclusive_scan_dev(const T *in, const uint64_t *d_n, uint64_t cap, uint64_t *out, uint64_t *sums,
                               cudaStream_t s, int *kernels) {
    const uint32_t tiles = (uint32_t)((cap + SCAN_TILE - 1) / SCAN_TILE);
    tile_sums_dev_kernel<T><<<tiles ? tiles : 1, SCAN_TPB, 0, s>>>(in, d_n, sums);
    scan_sums_dev_kernel<<<1, SCAN_TPB, 0, s>>>(sums, d_n);
    tile_scan_dev_kernel<T><<<tiles ? tiles : 1, SCAN_TPB, 0, s>>>(in, d_n, sums, out);
    *kernels += 3;
    return cudaGetLastError();
}

cudaError_t read_u64(const uint64_t *d, uint64_t *h, cudaStream_t s) {
    cudaError_t e = cudaMemcpyAsync(h, d, sizeof(uint64_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    return e;
}

// persistent grid of a generator kernel; a failed occupancy query is returned
cudaError_t gen_grid(const void *kernel, int num_sms, uint64_t work, int *grid) {
    int per_sm = 0;
    const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, GEN_TPB, 0);
    if (e != cudaSuccess)
        return e;
    if (per_sm < 1)
        per_sm = 1;
    uint64_t g = (uint64_t)per_sm * (num_sms > 0 ? num_sms : 1);
    const uint64_t need = (work + GEN_TPB - 1) / GEN_TPB;
    if (g > need)
        g = need;
    *grid = (int)(g ? g : 1);
    return cudaSuccess;
}

// pinned host memory that grows (contents not kept)
struct PinBuf {
    uint64_t *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t n) {
        if (n <= cap)
            return cudaSuccess;
        cudaFreeHost(p);
        p = nullptr;
        // at least double: pinning memory is slow; exactly what is needed if that fails
        size_t want = (n > 2 * cap ? n : 2 * cap) + 1024;
        cap = 0;
        cudaError_t e = cudaHostAlloc((void **)&p, want * sizeof(uint64_t), cudaHostAllocDefault);
        if (e == cudaErrorMemoryAllocation && want > n + 1024) {
            (void)cudaGetLastError();
            p = nullptr;
            want = n + 1024;
            e = cudaHostAlloc((void **)&p, want * sizeof(uint64_t), cudaHostAllocDefault);
        }
        if (e == cudaSuccess)
            cap = want;
        else
            p = nullptr;
        return e;
    }
    PinBuf() = default;
    PinBuf(const PinBuf &) = delete;
    PinBuf &operator=(const PinBuf &) = delete;
    ~PinBuf() { cudaFreeHost(p); }
};

// fn(lo, hi) over [0, n) on the host cores (the persistent pool), in contiguous ranges;
// a level of a few parents stays on the calling thread
template <typename F>
void parallel_ranges(uint64_t n, F fn) {
    if (n < 16) {
        fn((uint64_t)0, n);
        return;
    }
    canon::HostPool::get().ranges(n, fn);
}

// ---- k-system rounds on the device ----------------------------------------
// The walk of a level is split into units: unit u is parent u / np with the second pair's
// partner u % np (ksys_children), so a parent's children are counted and written by np
// threads, in its order.  d_nunits (optional): the unit count in device memory (a captured
// level).
__global__ void ksys_count_kernel(int np, const uint8_t *parents, uint32_t n_units, int d, uint32_t *counts,
                                  const uint64_t *d_nunits = nullptr) {
    if (d_nunits)
        n_units = (uint32_t)*d_nunits;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t u = blockIdx.x * blockDim.x + threadIdx.x; u < n_units; u += stride) {
        const uint32_t p = u / (uint32_t)np, sec = u % (uint32_t)np;
        counts[u] = canon::ksys_children(np, parents + (size_t)p * d * np, d, nullptr, (int)sec);
    }
}

// the children of units [u0, u1) at offsets[u] - offsets[u0], and one work item each
__global__ void ksys_emit_kernel(int np, const uint8_t *parents, uint32_t u0, uint32_t u1, int d,
                                 const uint64_t *offsets, uint8_t *out, canon::Item *items,
                                 const uint64_t *d_nunits = nullptr) {
    if (d_nunits)
        u1 = (uint32_t)*d_nunits;
    const uint64_t base = offsets[u0];
    const uint32_t m = (uint32_t)d + 1;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t u = u0 + blockIdx.x * blockDim.x + threadIdx.x; u < u1; u += stride) {
        const uint32_t p = u / (uint32_t)np, sec = u % (uint32_t)np;
        const uint64_t o = offsets[u] - base;
        const uint32_t cnt =
            canon::ksys_children(np, parents + (size_t)p * d * np, d, out + o * m * np, (int)sec);
        for (uint32_t j = 0; j < cnt; ++j) {
            canon::Item it{};
            it.data_off = (uint32_t)((o + j) * m * np);
            it.kind = canon::KIND_KSYS;
            it.nrows = (uint8_t)m;
            it.ncols = (uint8_t)np;
            it.flags = 0;
            it.out_idx = (uint32_t)(o + j);
            items[o + j] = it;
        }
    }
}

// the canonical children of a slice into the next level, their |Aut| when complete,
// and the relabelings tried (summed per block)
__global__ void ksys_compact_kernel(uint64_t n_cand, uint32_t bytes, const uint8_t *cand, const uint8_t *canonical,
                                    const uint8_t *status, const uint64_t *aut, const uint64_t *trials,
                                    const uint64_t *offs, uint8_t *dst, uint64_t *aut_dst, unsigned *bad,
                                    unsigned long long *trials_sum, const uint64_t *d_ncand = nullptr) {
    if (d_ncand)
        n_cand = *d_ncand;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    unsigned long long tsum = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_cand; i += stride) {
        tsum += trials[i];
        if (status[i] & (canon::ST_TIMEOUT | canon::ST_BADINPUT))
            atomicOr(bad, 1u);
        if (!canonical[i])
            continue;
        const uint64_t o = offs[i];
        for (uint32_t q = 0; q < bytes; ++q)
            dst[o * bytes + q] = cand[i * bytes + q];
        if (aut_dst) {
            aut_dst[2 * o] = aut[2 * i];
            aut_dst[2 * o + 1] = aut[2 * i + 1];
        }
    }
    for (int off = 16; off > 0; off >>= 1)
        tsum += __shfl_down_sync(0xFFFFFFFFu, tsum, off);
    if ((threadIdx.x & 31u) == 0 && tsum)
        atomicAdd(trials_sum, tsum);
}

// ---- the k-system enumeration as one captured CUDA graph -------------------
// Every level's size stays in device memory (KsCtl): the kernels of a level read it
// there, so the whole enumeration -- per level the round generator, the scan, the
// segmented check and the compaction -- is captured once and replayed with one
// launch and one wait.  Level buffers are sized for `cap` parents and candidates; a
// level beyond that raises `overflow`, empties the rest of the run, and the host
// enumerates again level by level with buffers that grow.
struct KsCtl {
    uint64_t n_par;                       // parents of the level in progress
    uint64_t n_units;                     // their walk units (parents x np)
    uint64_t n_cand;                      // its candidates
    uint64_t level_checks[16];
    unsigned long long stamp[16][3];      // globaltimer: level start, candidates written, checked
    unsigned long long trials;            // relabelings tried by all checks
    unsigned levels;                      // levels with parents
    unsigned overflow;
    unsigned bad;                         // a check reported a bad status
    unsigned pad;
};

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// round 0 = (0 1)(2 3)... as the only parent of the first level
__global__ void ksg_start_kernel(KsCtl *ctl, uint8_t *lev, int np) {
    if (threadIdx.x < (unsigned)np)
        lev[threadIdx.x] = (uint8_t)threadIdx.x;
    if (threadIdx.x == 0)
        ctl->n_par = 1;
}

__global__ void ksg_begin_kernel(KsCtl *ctl, int level, int np) {
    ctl->stamp[level][0] = global_ns();
    ctl->n_units = ctl->n_par * (uint64_t)np;
    if (ctl->n_par)
        ++ctl->levels;
}

// the level's candidates: offs[n_units]; beyond the buffers, the run stops here
__global__ void ksg_cand_kernel(KsCtl *ctl, const uint64_t *offs, uint64_t cap, int level) {
    uint64_t n = offs[ctl->n_units];
    if (n > cap) {
        ctl->overflow = 1u;
        n = 0;
        ctl->n_par = 0;
        ctl->n_units = 0;
    }
    ctl->n_cand = n;
    ctl->level_checks[level] = n;
}

__global__ void ksg_stamp_kernel(KsCtl *ctl, int level, int k) { ctl->stamp[level][k] = global_ns(); }

// the next level's parents: the canonical candidates
__global__ void ksg_next_kernel(KsCtl *ctl, const uint64_t *coffs, uint64_t cap) {
    uint64_t n = coffs[ctl->n_cand];
    if (n > cap) {
        ctl->overflow = 1u;
        n = 0;
    }
    ctl->n_par = n;
}

struct KsysGraph {
    uint32_t np = 0, seg = 0;
    uint64_t cap = 0;
    int kernels = 0;
    cudaGraphExec_t exec = nullptr;
    DevBuf<uint8_t> lev[2], cand, can, status, rrow, rtc, wit, len_aut;
    DevBuf<uint64_t> doffs, coffs, sums, aut, aut_out, trials;
    DevBuf<uint32_t> counts;
    DevBuf<int32_t> pidx;
    DevBuf<uint16_t> n_auts;
    DevBuf<canon::Item> items;
    DevBuf<canon::KsysSeg> kseg;
    DevBuf<KsCtl> ctl;
    ~KsysGraph() {
        if (exec)
            cudaGraphExecDestroy(exec);
    }
};

// Allocates the buffers and captures the enumeration of K_np with level buffers of
// `cap` matrices; seg = the segment rule (0 = chosen per level on the device).
cudaError_t ksys_graph_build(canon_ctx *c, KsysGraph &g, uint32_t np, uint64_t cap, uint32_t seg) {
    const uint32_t rounds = np - 1;
    const size_t mbytes = (size_t)rounds * np;     // the largest matrix
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < 2 && e == cudaSuccess; ++i)
        e = g.lev[i].ensure(cap * mbytes);
    if (e == cudaSuccess) e = g.cand.ensure(cap * mbytes);
    if (e == cudaSuccess) e = g.can.ensure(cap);
    if (e == cudaSuccess) e = g.status.ensure(cap);
    if (e == cudaSuccess) e = g.rrow.ensure(cap);
    if (e == cudaSuccess) e = g.rtc.ensure(cap);
    if (e == cudaSuccess) e = g.wit.ensure(cap * 16);
    if (e == cudaSuccess) e = g.len_aut.ensure(cap);
    if (e == cudaSuccess) e = g.doffs.ensure(cap * np + 1);
    if (e == cudaSuccess) e = g.coffs.ensure(cap + 1);
    if (e == cudaSuccess) e = g.sums.ensure(cap * np / SCAN_TILE + 2);
    if (e == cudaSuccess) e = g.aut.ensure(cap * 2);
    if (e == cudaSuccess) e = g.aut_out.ensure(cap * 2);
    if (e == cudaSuccess) e = g.trials.ensure(cap);
    if (e == cudaSuccess) e = g.counts.ensure(cap * np);
    if (e == cudaSuccess) e = g.pidx.ensure(cap);
    if (e == cudaSuccess) e = g.n_auts.ensure(cap);
    if (e == cudaSuccess) e = g.items.ensure(cap);
    if (e == cudaSuccess) e = g.kseg.ensure(cap + 1);
    if (e == cudaSuccess) e = g.ctl.ensure(1);
    if (e != cudaSuccess)
        return e;
    const int sms = c->num_sms > 0 ? c->num_sms : 1;
    int gg = (int)((cap * np + 127) / 128);
    if (gg > 4 * sms)
        gg = 4 * sms;
    int gc = (int)((cap + 255) / 256);
    if (gc > 4 * sms)
        gc = 4 * sms;
    cudaStream_t s = c->stream;
    int kernels = 0;
    e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess)
        return e;
    KsCtl *ctl = g.ctl.p;
    e = cudaMemsetAsync(ctl, 0, sizeof(KsCtl), s);
    if (e == cudaSuccess) {
        ksg_start_kernel<<<1, 32, 0, s>>>(ctl, g.lev[1].p, (int)np);
        ++kernels;
        e = cudaGetLastError();
    }
    // parents with n rounds live in lev[n & 1]
    for (uint32_t n = 1; n < rounds && e == cudaSuccess; ++n) {
        const uint32_t m = n + 1;
        const bool complete = m == rounds;
        const uint8_t *par = g.lev[n & 1].p;
        uint8_t *dst = g.lev[m & 1].p;
        ksg_begin_kernel<<<1, 1, 0, s>>>(ctl, (int)m - 1, (int)np);
        ksys_count_kernel<<<gg, 128, 0, s>>>((int)np, par, 0, (int)n, g.counts.p, &ctl->n_units);
        kernels += 2;
        e = exclusive_scan_dev(g.counts.p, &ctl->n_units, cap * np, g.doffs.p, g.sums.p, s, &kernels);
        if (e != cudaSuccess)
            break;
        ksg_cand_kernel<<<1, 1, 0, s>>>(ctl, g.doffs.p, cap, (int)m - 1);
        ksys_emit_kernel<<<gg, 128, 0, s>>>((int)np, par, 0, 0, (int)n, g.doffs.p, g.cand.p, g.items.p,
                                             &ctl->n_units);
        ksg_stamp_kernel<<<1, 1, 0, s>>>(ctl, (int)m - 1, 1);
        kernels += 3;
        canon::Outputs o{};
        o.canonical = g.can.p;
        o.status = g.status.p;
        o.reject_row = g.rrow.p;
        o.row_to_change = g.rtc.p;
        o.player_index = g.pidx.p;
        o.witness = g.wit.p;
        o.aut = g.aut.p;
        o.trials = g.trials.p;
        o.n_auts = g.n_auts.p;
        o.len_aut = g.len_aut.p;
        e = canon::launch_ksys_check_split(g.items.p, (uint32_t)cap, g.cand.p, o, seg,
                                           canon::ksys_candidates(np, m), g.kseg.p, c->num_sms, s, &ctl->n_cand);
        kernels += 3;
        if (e != cudaSuccess)
            break;
        ksg_stamp_kernel<<<1, 1, 0, s>>>(ctl, (int)m - 1, 2);
        ++kernels;
        e = exclusive_scan_dev(g.can.p, &ctl->n_cand, cap, g.coffs.p, g.sums.p, s, &kernels);
        if (e != cudaSuccess)
            break;
        ksys_compact_kernel<<<gc, 256, 0, s>>>(0, (uint32_t)(m * np), g.cand.p, g.can.p, g.status.p, g.aut.p,
                                               g.trials.p, g.coffs.p, dst, complete ? g.aut_out.p : nullptr,
                                               &ctl->bad, &ctl->trials, &ctl->n_cand);
        ksg_next_kernel<<<1, 1, 0, s>>>(ctl, g.coffs.p, cap);
        kernels += 2;
        e = cudaGetLastError();
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(s, &graph);
    if (e == cudaSuccess)
        e = e2;
    if (e == cudaSuccess)
        e = cudaGraphInstantiate(&g.exec, graph, 0);
    if (graph)
        cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        g.exec = nullptr;
        return e;
    }
    g.np = np;
    g.cap = cap;
    g.seg = seg;
    g.kernels = kernels;
    return cudaSuccess;
}

}  // namespace

namespace canon {
void ksys_graph_release(canon_ctx *c) {
    delete static_cast<KsysGraph *>(c->ksys_graph);
    c->ksys_graph = nullptr;
}
}  // namespace canon

namespace {

// One enumeration of K_np through the captured graph.  Returns CANON_OK with
// *ran = false when a level outgrew the buffers (the caller enumerates level by
// level, and the next graph is built 4x larger).
int ksys_enumerate_graph(canon_ctx *c, uint32_t np, canon_design_cb cb, void *user, canon_enum_stats &st,
                         bool *ran) {
    *ran = false;
    // the segment rule baked into the graph: a fixed size, one segment per matrix, or per level on the device
    const uint32_t seg = c->ksys_seg == CANON_KSYS_WHOLE ? 0xFFFFFFE0u
                                                         : (c->ksys_seg ? ((c->ksys_seg + 31u) & ~31u) : 0u);
    KsysGraph *g = static_cast<KsysGraph *>(c->ksys_graph);
    if (!g || g->np != np || g->cap != c->ksys_graph_cap || g->seg != seg || !g->exec) {
        canon::ksys_graph_release(c);
        g = new KsysGraph();
        c->ksys_graph = g;
        const cudaError_t e = ksys_graph_build(c, *g, np, c->ksys_graph_cap, seg);
        if (e != cudaSuccess) {
            canon::ksys_graph_release(c);
            c->err = std::string("enumerate k-systems: graph capture: ") + cudaGetErrorString(e);
            return e == cudaErrorMemoryAllocation ? CANON_ENOMEM : CANON_ECUDA;
        }
    }
    cudaStream_t s = c->stream;
    KsCtl h{};
    cudaError_t e = cudaGraphLaunch(g->exec, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&h, g->ctl.p, sizeof(KsCtl), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        c->err = std::string("enumerate k-systems: graph: ") + cudaGetErrorString(e);
        return CANON_ECUDA;
    }
    c->launches += g->kernels;
    if (h.overflow) {
        if (c->ksys_graph_cap < (1ull << 24))
            c->ksys_graph_cap *= 4;
        canon::ksys_graph_release(c);
        return CANON_OK;
    }
    *ran = true;
    const uint32_t rounds = np - 1;
    for (uint32_t m = 2; m <= rounds; ++m) {
        const uint64_t nc = h.level_checks[m - 1];
        if (!nc && !h.stamp[m - 1][2])
            continue;
        st.checks += nc;
        st.level_checks[m - 1] = nc;
        const double gen = (double)(h.stamp[m - 1][1] - h.stamp[m - 1][0]) * 1e-9;
        const double chk = (double)(h.stamp[m - 1][2] - h.stamp[m - 1][1]) * 1e-6;
        st.gen_seconds += gen;
        st.level_kernel_ms[m - 1] = chk;
        st.kernel_ms += chk;
    }
    st.levels = h.levels;
    st.batches = h.levels;
    st.trials = h.trials;
    if (h.bad) {
        c->err = "enumerate k-systems: a check reported a bad status";
        return CANON_ETIMEOUT;
    }
    const uint64_t n_final = h.n_par;
    if (n_final) {
        const size_t bytes = (size_t)rounds * np;
        std::vector<uint8_t> mats((size_t)n_final * bytes);
        std::vector<uint64_t> auts((size_t)n_final * 2);
        e = cudaMemcpyAsync(mats.data(), g->lev[rounds & 1].p, mats.size(), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(auts.data(), g->aut_out.p, auts.size() * sizeof(uint64_t), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            c->err = std::string("enumerate k-systems: designs: ") + cudaGetErrorString(e);
            return CANON_ECUDA;
        }
        st.designs = n_final;
        if (cb)
            for (uint64_t i = 0; i < n_final; ++i)
                cb(user, mats.data() + i * bytes, rounds, np, auts[2 * i], auts[2 * i + 1]);
    }
    return CANON_OK;
}

}  // namespace

extern "C" int canon_enumerate_bibd(canon_ctx *c, uint32_t v, uint32_t b, uint32_t r, uint32_t k, uint32_t lambda,
                                    canon_design_cb cb, void *user, canon_enum_stats *stats) {
    if (!c || v < 2 || v > canon::VMAX || b < 1 || b > canon::BMAX || r < 1 || r > b || k < 1 || k > v)
        return CANON_EINVAL;
    const auto t0 = std::chrono::steady_clock::now();
    auto since = [](std::chrono::steady_clock::time_point a) {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - a).count();
    };
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    canon_enum_stats st{};
    const canon::rows::Params prm{(int)v, (int)b, (int)r, (int)k, (int)lambda};
    DevBuf<uint64_t> lev, next, cand, doffs, coffs, sums, aut, aut_out, rcache, gens;
    DevBuf<uint8_t> ngens;
    constexpr uint32_t NG = canon::rows::AUT_GENS;
    std::vector<uint64_t> hgens(NG, 0);     // automorphisms of the host level's parents
    std::vector<uint8_t> hngens(1, 0);
    bool have_gens = false, aut_pruning = (c->cfg.options & CANON_OPT_AUT_PRUNE) != 0;
    DevBuf<uint32_t> dcounts;
    DevBuf<uint8_t> can, status;
    DevBuf<unsigned> ticket, stop;
    DevBuf<canon::SplitPart> parts;
    PinBuf hcand;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    auto done = [&](int rc, const char *what, cudaError_t e) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (rc != CANON_OK)
            c->err = std::string("enumerate: ") + what +
                     (e != cudaSuccess ? std::string(": ") + cudaGetErrorString(e) : std::string());
        return rc;
    };
    cudaError_t e = ticket.ensure(2);      // [0] work-stealing counter, [1] timeout flag
    if (e != cudaSuccess)
        return done(CANON_ENOMEM, "setup", e);
    // level 1: row 0 is forced, r ones first; the parents of a level live on the
    // host (host generation) or in `lev` on the GPU (after a compaction)
    std::vector<uint64_t> level(1, (r >= 64) ? ~0ull : ((1ull << r) - 1ull));
    bool host_valid = true;
    uint64_t n_par = 1;
    uint32_t n = 1;
    while (n < v && n_par) {
        const uint32_t m = n + 1;
        const bool complete = m == v;
        const bool dev = n_par >= DEVICE_GEN_MIN;
        // 1: children per parent and their offsets
        auto tg = std::chrono::steady_clock::now();
        std::vector<uint32_t> counts;
        std::vector<uint64_t> offs;
        uint64_t n_cand = 0;
        if (!dev) {
            if (!host_valid) {
                level.resize((size_t)n_par * n);
                hgens.resize((size_t)n_par * NG);
                hngens.resize(n_par);
                e = cudaMemcpyAsync(level.data(), lev.p, level.size() * sizeof(uint64_t), cudaMemcpyDeviceToHost, s);
                if (e == cudaSuccess && have_gens)
                    e = cudaMemcpyAsync(hgens.data(), gens.p, hgens.size() * sizeof(uint64_t), cudaMemcpyDeviceToHost,
                                        s);
                if (e == cudaSuccess && have_gens)
                    e = cudaMemcpyAsync(hngens.data(), ngens.p, n_par, cudaMemcpyDeviceToHost, s);
                if (e == cudaSuccess)
                    e = cudaStreamSynchronize(s);
                if (e != cudaSuccess)
                    return done(CANON_ECUDA, "level to host", e);
                if (!have_gens)
                    std::fill(hngens.begin(), hngens.end(), (uint8_t)0);
                host_valid = true;
            }
            counts.resize(n_par);
            parallel_ranges(n_par, [&](uint64_t lo, uint64_t hi) {
                for (uint64_t p = lo; p < hi; ++p)
                    counts[p] = canon::rows::children<canon::rows::COUNT>(prm, level.data() + p * n, (int)n,
                                                                         nullptr, 0, hgens.data() + p * NG,
                                                                         hngens[p]);
            });
            offs.assign(n_par + 1, 0);
            for (uint64_t p = 0; p < n_par; ++p)
                offs[p + 1] = offs[p] + counts[p];
            n_cand = offs[n_par];
        } else {
            e = dcounts.ensure(n_par);
            if (e == cudaSuccess)
                e = doffs.ensure(n_par + 1);
            if (e == cudaSuccess)
                e = rcache.ensure((size_t)n_par * row_cache_rows(n_par));
            if (e != cudaSuccess)
                return done(CANON_ENOMEM, "level buffers", e);
            int grid = 0;
            e = cudaMemsetAsync(ticket.p, 0, sizeof(unsigned), s);
            if (e == cudaSuccess)
                e = gen_grid((const void *)rows_count_kernel, c->num_sms, n_par, &grid);
            if (e != cudaSuccess)
                return done(CANON_ECUDA, "count", e);
            rows_count_kernel<<<grid, GEN_TPB, 0, s>>>(prm, lev.p, (uint32_t)n_par, (int)n, dcounts.p, rcache.p,
                                                       row_cache_rows(n_par), ticket.p,
                                                       have_gens ? gens.p : nullptr, ngens.p);
            e = cudaGetLastError();
            if (e == cudaSuccess)
                e = exclusive_scan(dcounts.p, n_par, doffs.p, sums, s);
            if (e == cudaSuccess)
                e = read_u64(doffs.p + n_par, &n_cand, s);
            if (e != cudaSuccess)
                return done(CANON_ECUDA, "count", e);
            c->launches += 4;
        }
        const double g1 = since(tg);
        st.gen_seconds += g1;
        st.level_gen_ms[m - 1] += g1 * 1e3;
        e = next.ensure((size_t)(n_cand ? n_cand : 1) * m);
        if (e == cudaSuccess && complete)
            e = aut_out.ensure((size_t)(n_cand ? n_cand : 1) * 2);
        if (e != cudaSuccess)
            return done(CANON_ENOMEM, "next level", e);
        uint64_t n_next = 0;
        uint64_t p0 = 0;
        while (p0 < n_par) {
            // the largest slice of parents whose children fit SLICE_CAP (at least one)
            uint64_t p1 = p0 + 1, base = 0, end = 0;
            if (!dev) {
                while (p1 < n_par && offs[p1 + 1] - offs[p0] <= SLICE_CAP)
                    ++p1;
                base = offs[p0];
                end = offs[p1];
            } else {
                e = read_u64(doffs.p + p0, &base, s);
                p1 = n_par;
                end = n_cand;
                if (e == cudaSuccess && n_cand - base > SLICE_CAP) {
                    uint64_t lo = p0 + 1, hi = n_par;
                    while (lo < hi) {
                        const uint64_t mid = (lo + hi + 1) / 2;
                        uint64_t at = 0;
                        e = read_u64(doffs.p + mid, &at, s);
                        if (e != cudaSuccess)
                            break;
                        if (at - base <= SLICE_CAP)
                            lo = mid;
                        else
                            hi = mid - 1;
                    }
                    p1 = lo;
                    if (e == cudaSuccess)
                        e = read_u64(doffs.p + p1, &end, s);
                }
                if (e != cudaSuccess)
                    return done(CANON_ECUDA, "slice", e);
            }
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
            if (e == cudaSuccess && !dev)
                e = hcand.ensure((size_t)(ns ? ns : 1) * m);
            if (e != cudaSuccess)
                return done(CANON_ENOMEM, "slice buffers", e);
            // 2: the children of parents [p0, p1), in order
            tg = std::chrono::steady_clock::now();
            if (!dev) {
                parallel_ranges(p1 - p0, [&](uint64_t lo, uint64_t hi) {
                    for (uint64_t p = p0 + lo; p < p0 + hi; ++p)
                        canon::rows::children<canon::rows::CHILD>(prm, level.data() + p * n, (int)n,
                                                                  hcand.p + (offs[p] - base) * m, counts[p],
                                                                  hgens.data() + p * NG, hngens[p]);
                });
                e = cudaMemcpyAsync(cand.p, hcand.p, (size_t)ns * m * sizeof(uint64_t), cudaMemcpyHostToDevice, s);
            } else {
                int grid = 0;
                e = cudaMemsetAsync(ticket.p, 0, sizeof(unsigned), s);
                if (e == cudaSuccess)
                    e = gen_grid((const void *)rows_emit_kernel, c->num_sms, p1 - p0, &grid);
                if (e != cudaSuccess)
                    return done(CANON_ECUDA, "children", e);
                rows_emit_kernel<<<grid, GEN_TPB, 0, s>>>(prm, lev.p, (uint32_t)p0, (uint32_t)p1, (int)n, doffs.p,
                                                          dcounts.p, rcache.p, row_cache_rows(n_par), cand.p,
                                                          ticket.p, have_gens ? gens.p : nullptr, ngens.p);
                e = cudaGetLastError();
                if (e == cudaSuccess)
                    e = cudaStreamSynchronize(s);
                ++c->launches;
            }
            const double g2 = since(tg);
            st.gen_seconds += g2;
            st.level_gen_ms[m - 1] += g2 * 1e3;
            if (e != cudaSuccess)
                return done(CANON_ECUDA, "children", e);
            // 3: the verdicts
            cudaEventRecord(e0, s);
            if (ns <= SPLIT_MAX) {
                e = parts.ensure((size_t)(ns ? ns : 1) * m * (canon::split_levels(ns, m) == 2 ? m : 1));
                if (e == cudaSuccess)
                    e = stop.ensure(ns ? ns : 1);
                if (e == cudaSuccess)
                    e = canon::launch_bibd_check_split((uint32_t)ns, m, b,
                                                       canon::F_VERDICT_ONLY | (complete ? canon::F_COMPLETE : 0u),
                                                       cand.p, can.p, complete ? aut.p : nullptr, status.p, parts.p,
                                                       stop.p, c->cfg.max_trials, c->d_ticket, c->num_sms, s);
            } else {
                // the converged lex-max pass, stopping at the first greater node: 6-8x less
                // check time than the one-pass reference-order check on the large families
                // (BIBD(16,24,9,6,3): 4.2 s against 32.7 s)
                e = canon::launch_bibd_check_uniform((uint32_t)ns, m, b,
                                                     canon::F_VERDICT_ONLY | (complete ? canon::F_COMPLETE : 0u),
                                                     cand.p, can.p, nullptr, complete ? aut.p : nullptr, status.p,
                                                     nullptr, c->cfg.max_trials, c->d_ticket, c->num_sms, s,
                                                     nullptr, canon::VARIANT_CONVERGED);
            }
            cudaEventRecord(e1, s);
            // 4: pack the canonical ones into the next level
            if (e == cudaSuccess)
                e = exclusive_scan(can.p, ns, coffs.p, sums, s);
            if (e == cudaSuccess)
                e = cudaMemsetAsync(ticket.p + 1, 0, sizeof(unsigned), s);
            if (e == cudaSuccess) {
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
            float chk_ms = 0.f;
            cudaEventElapsedTime(&chk_ms, e0, e1);
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
        host_valid = false;
        n_par = n_next;
        n = m;
        // automorphisms of the new parents, which prune their children.  Deeper levels
        // hold fewer symmetric partial matrices; once under 2 % of a level's parents have
        // a nontrivial automorphism the searches for them cost more than they prune, and
        // the deeper levels go without.
        have_gens = false;
        if (aut_pruning && n < v && n_par && n >= 2) {
            e = gens.ensure((size_t)n_par * NG);
            if (e == cudaSuccess)
                e = ngens.ensure(n_par);
            if (e != cudaSuccess)
                return done(CANON_ENOMEM, "automorphism buffers", e);
            cudaEventRecord(e0, s);
            e = canon::launch_bibd_autgen((uint32_t)n_par, n, b, lev.p, gens.p, ngens.p, NG, c->cfg.max_trials,
                                          ticket.p, c->num_sms, s);
            cudaEventRecord(e1, s);
            if (e == cudaSuccess)
                e = cudaEventSynchronize(e1);
            if (e != cudaSuccess)
                return done(CANON_ECUDA, "automorphisms", e);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            st.gen_seconds += ms * 1e-3;
            ++c->launches;
            have_gens = true;
            std::vector<uint8_t> ng(n_par);
            e = cudaMemcpy(ng.data(), ngens.p, n_par, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess)
                return done(CANON_ECUDA, "automorphisms", e);
            uint64_t with = 0;
            for (uint8_t x : ng)
                with += x != 0;
            if (with * 50 < n_par)
                aut_pruning = false;
        }
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
    st.seconds = since(t0);
    if (stats)
        *stats = st;
    return done(CANON_OK, "", cudaSuccess);
}

// All 1-factorizations of K_np up to isomorphism, round by round with every level in
// HBM: the next rounds of all canonical parents are generated on the GPU
// (ksys_count_kernel, a scan, ksys_emit_kernel), checked there (the warp-per-matrix
// cnvCheckNew() kernel), and the canonical ones compacted into the next level.  The
// work of alldata::Run() for group size 2 with the check at every level
// (k-Factorization/TripleSys/Source/TripleSys.cpp:80-775, check at
// checkCurrentResult.cpp:91).
extern "C" int canon_enumerate_ksys(canon_ctx *c, uint32_t np, canon_design_cb cb, void *user,
                                    canon_enum_stats *stats) {
    if (!c || np < 4 || np > (uint32_t)canon::KS_MAXNP || (np & 1u))
        return CANON_EINVAL;
    const auto t0 = std::chrono::steady_clock::now();
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    canon_enum_stats st{};
    if (!(c->cfg.options & CANON_OPT_NO_GRAPH)) {
        bool ran = false;
        const int rc = ksys_enumerate_graph(c, np, cb, user, st, &ran);
        if (rc != CANON_OK || ran) {
            st.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            if (stats)
                *stats = st;
            return rc;
        }
        st = canon_enum_stats{};   // a level outgrew the graph's buffers: level by level below
    }
    DevBuf<uint8_t> lev, next, cand, can, status, rrow, rtc, wit, len_aut;
    DevBuf<uint64_t> doffs, coffs, sums, aut, aut_out, trials;
    DevBuf<uint32_t> dcounts;
    DevBuf<int32_t> pidx;
    DevBuf<uint16_t> n_auts;
    DevBuf<canon::Item> items;
    DevBuf<unsigned> ticket;
    DevBuf<unsigned long long> tsum;
    DevBuf<canon::KsysSeg> kseg;
    cudaEvent_t e0 = nullptr, e1 = nullptr, g0 = nullptr, g1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventCreate(&g0);
    cudaEventCreate(&g1);
    auto done = [&](int rc, const char *what, cudaError_t e) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaEventDestroy(g0);
        cudaEventDestroy(g1);
        if (rc != CANON_OK)
            c->err = std::string("enumerate k-systems: ") + what +
                     (e != cudaSuccess ? std::string(": ") + cudaGetErrorString(e) : std::string());
        return rc;
    };
    cudaError_t e = ticket.ensure(2);      // [0] work-stealing counter, [1] bad-status flag
    if (e == cudaSuccess)
        e = tsum.ensure(1);
    if (e == cudaSuccess)
        e = lev.ensure(np);
    if (e != cudaSuccess)
        return done(CANON_ENOMEM, "setup", e);
    // level 1: round 0 = (0 1)(2 3)...
    {
        uint8_t r0[canon::KS_MAXNP];
        for (uint32_t i = 0; i < np; ++i)
            r0[i] = (uint8_t)i;
        e = cudaMemcpyAsync(lev.p, r0, np, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemsetAsync(ticket.p + 1, 0, sizeof(unsigned), s);
        if (e == cudaSuccess)
            e = cudaMemsetAsync(tsum.p, 0, sizeof(unsigned long long), s);
        if (e != cudaSuccess)
            return done(CANON_ECUDA, "setup", e);
    }
    const uint32_t rounds = np - 1;
    uint64_t n_par = 1;
    uint32_t n = 1;
    const int grid_cap = 4 * (c->num_sms > 0 ? c->num_sms : 1);
    while (n < rounds && n_par) {
        const uint32_t m = n + 1;
        const bool complete = m == rounds;
        // 1: children per walk unit (parent x second-pair partner) and their offsets (on the GPU)
        const uint64_t n_units = n_par * np;
        e = dcounts.ensure(n_units);
        if (e == cudaSuccess)
            e = doffs.ensure(n_units + 1);
        if (e != cudaSuccess)
            return done(CANON_ENOMEM, "level buffers", e);
        int g = (int)((n_units + 127) / 128);
        if (g > grid_cap)
            g = grid_cap;
        cudaEventRecord(g0, s);
        ksys_count_kernel<<<g, 128, 0, s>>>((int)np, lev.p, (uint32_t)n_units, (int)n, dcounts.p);
        e = cudaGetLastError();
        if (e == cudaSuccess)
            e = exclusive_scan(dcounts.p, n_units, doffs.p, sums, s);
        cudaEventRecord(g1, s);
        std::vector<uint64_t> offs(n_units + 1);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(offs.data(), doffs.p, offs.size() * sizeof(uint64_t), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(s);
        if (e != cudaSuccess)
            return done(CANON_ECUDA, "count", e);
        float gms = 0.f;
        cudaEventElapsedTime(&gms, g0, g1);
        st.gen_seconds += gms * 1e-3;
        c->launches += 4;
        const uint64_t n_cand = offs[n_units];
        const size_t bytes = (size_t)m * np;
        e = next.ensure((n_cand ? n_cand : 1) * bytes);
        if (e == cudaSuccess && complete)
            e = aut_out.ensure((size_t)(n_cand ? n_cand : 1) * 2);
        if (e != cudaSuccess)
            return done(CANON_ENOMEM, "next level", e);
        uint64_t n_next = 0, p0 = 0;
        // slices of walk units whose children fit SLICE_CAP
        while (p0 < n_units) {
            uint64_t p1 = p0 + 1;
            while (p1 < n_units && offs[p1 + 1] - offs[p0] <= SLICE_CAP)
                ++p1;
            const uint64_t ns = offs[p1] - offs[p0];
            const size_t cap = ns ? ns : 1;
            e = cand.ensure(cap * bytes);
            if (e == cudaSuccess) e = items.ensure(cap);
            if (e == cudaSuccess) e = can.ensure(cap);
            if (e == cudaSuccess) e = status.ensure(cap);
            if (e == cudaSuccess) e = rrow.ensure(cap);
            if (e == cudaSuccess) e = rtc.ensure(cap);
            if (e == cudaSuccess) e = pidx.ensure(cap);
            if (e == cudaSuccess) e = wit.ensure(cap * 16);
            if (e == cudaSuccess) e = aut.ensure(cap * 2);
            if (e == cudaSuccess) e = trials.ensure(cap);
            if (e == cudaSuccess) e = n_auts.ensure(cap);
            if (e == cudaSuccess) e = len_aut.ensure(cap);
            if (e == cudaSuccess) e = coffs.ensure(cap + 1);
            if (e != cudaSuccess)
                return done(CANON_ENOMEM, "slice buffers", e);
            // 2: the children and their work items
            int ge = (int)((p1 - p0 + 127) / 128);
            if (ge > grid_cap)
                ge = grid_cap;
            cudaEventRecord(g0, s);
            ksys_emit_kernel<<<ge, 128, 0, s>>>((int)np, lev.p, (uint32_t)p0, (uint32_t)p1, (int)n, doffs.p, cand.p,
                                                items.p);
            cudaEventRecord(g1, s);
            e = cudaGetLastError();
            // 3: the verdicts
            canon::Outputs o{};
            o.canonical = can.p;
            o.status = status.p;
            o.reject_row = rrow.p;
            o.row_to_change = rtc.p;
            o.player_index = pidx.p;
            o.witness = wit.p;
            o.aut = aut.p;
            o.trials = trials.p;
            o.n_auts = n_auts.p;
            o.len_aut = len_aut.p;
            o.auts = nullptr;
            o.aut_cap = 0;
            // one warp per matrix, or the candidates of every matrix split over warps
            const uint32_t seg = canon::ksys_segment(c, ns, np, m);
            if (e == cudaSuccess && seg)
                e = kseg.ensure(ns + 1);
            cudaEventRecord(e0, s);
            if (e == cudaSuccess)
                e = seg ? canon::launch_ksys_check_split(items.p, (uint32_t)ns, cand.p, o, seg,
                                                         canon::ksys_candidates(np, m), kseg.p, c->num_sms, s)
                        : canon::launch_ksys_check(items.p, (uint32_t)ns, cand.p, o, ticket.p, c->num_sms, s);
            cudaEventRecord(e1, s);
            // 4: the canonical ones into the next level
            if (e == cudaSuccess)
                e = exclusive_scan(can.p, ns, coffs.p, sums, s);
            if (e == cudaSuccess) {
                const int gc = (int)((ns + 255) / 256 < 4096 ? (ns + 255) / 256 : 4096);
                ksys_compact_kernel<<<gc ? gc : 1, 256, 0, s>>>(ns, (uint32_t)bytes, cand.p, can.p, status.p, aut.p,
                                                                trials.p, coffs.p, next.p + n_next * bytes,
                                                                complete ? aut_out.p + 2 * n_next : nullptr,
                                                                ticket.p + 1, tsum.p);
                e = cudaGetLastError();
            }
            uint64_t n_can = 0;
            if (e == cudaSuccess)
                e = read_u64(coffs.p + ns, &n_can, s);
            if (e != cudaSuccess)
                return done(CANON_ECUDA, "check", e);
            float ms = 0.f, gms2 = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            cudaEventElapsedTime(&gms2, g0, g1);
            st.gen_seconds += gms2 * 1e-3;
            st.kernel_ms += ms;
            st.level_kernel_ms[m - 1] += ms;
            ++st.batches;
            c->launches += 7;
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
    unsigned bad = 0;
    unsigned long long tried = 0;
    e = cudaMemcpyAsync(&bad, ticket.p + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&tried, tsum.p, sizeof(tried), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    if (e != cudaSuccess)
        return done(CANON_ECUDA, "status", e);
    st.trials = tried;
    if (bad) {
        if (stats)
            *stats = st;
        return done(CANON_ETIMEOUT, "a check reported a bad status", cudaSuccess);
    }
    if (n == rounds && n_par) {
        const size_t bytes = (size_t)rounds * np;
        std::vector<uint8_t> mats((size_t)n_par * bytes);
        std::vector<uint64_t> auts((size_t)n_par * 2);
        e = cudaMemcpyAsync(mats.data(), lev.p, mats.size(), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(auts.data(), aut_out.p, auts.size() * sizeof(uint64_t), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(s);
        if (e != cudaSuccess)
            return done(CANON_ECUDA, "designs", e);
        st.designs = n_par;
        if (cb)
            for (uint64_t i = 0; i < n_par; ++i)
                cb(user, mats.data() + i * bytes, rounds, np, auts[2 * i], auts[2 * i + 1]);
    }
    st.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (stats)
        *stats = st;
    return done(CANON_OK, "", cudaSuccess);
}
