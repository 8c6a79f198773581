// canon_ksys.cu -- canonicity test of k-systems on sm_103a: rounds of pairs (group size
// 2, below), and rounds of groups of 3 or 4 (kgen_seg_kernel, with the relabeling step of
// canon_kgen.cuh).
//
// Restates alldata::cnvCheckNew() on its plain path
// (k-Factorization/TripleSys/Source/cnv.cpp:211-351): every relabeling that maps
// one of the filled rounds onto round 0 is applied, the result is brought to the
// reference's sorted form (kmSortMatrixForReorderedPlayers / kmSortRowsBy2ndValue,
// kmSupport.cpp:43-134, 220-274) and compared round by round with the matrix
// (kmProcessMatrix2, kmSupport.cpp:601-700).  The candidates are enumerated in
// the reference's order: Heap's permutations of the groups (cnv.cpp:283-315) x
// in-group orders (cnvCheckTgNew, :186-210) x the round mapped to round 0
// (cnvCheckKm1, :91-163).  The search has no data dependency between
// candidates, so one warp owns one matrix and its 32 lanes take 32 consecutive
// candidates; a ballot finds the first "smaller" candidate, which ends the check
// exactly where the reference stops.  Rounds are kept as nibble-packed partner
// tables, so a round comparison is one XOR and a find-first-set.
#include "canon_bibd_core.cuh"
#include "canon_kgen.cuh"
#include "canon_ksys_core.cuh"

namespace canon {

namespace {

using namespace ksys;

__global__ void __launch_bounds__(KTPB) ksys_kernel(const Item *__restrict__ items, uint32_t n_items,
                                                    const uint8_t *__restrict__ bytes, Outputs out,
                                                    unsigned *ticket) {
    __shared__ uint64_t s_seq[KW][16], s_part[KW][16], s_pair[KW][16];
    const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    for (;;) {
        unsigned it = 0;
        if (lane == 0)
            it = atomicAdd(ticket, 1u);
        it = __shfl_sync(0xFFFFFFFFu, it, 0);
        if (it >= n_items)
            break;
        check_item_warp(items[it], bytes, out, s_seq[warp], s_part[warp], s_pair[warp], lane);
    }
}

// The size of a segmented launch: the items (from device memory when d_n is given,
// as a captured enumeration level holds its size there) and the candidates per
// segment (0 = the automatic choice for that many items).
struct SegSize {
    uint32_t n;
    uint32_t seg;
};
__device__ __forceinline__ SegSize seg_size(uint32_t n_items, const uint64_t *d_n, uint32_t seg_cands,
                                            uint64_t total_max, uint32_t resident_warps) {
    SegSize z;
    z.n = d_n ? (uint32_t)*d_n : n_items;
    z.seg = seg_cands ? seg_cands : ksys_auto_segment(z.n, total_max, resident_warps);
    return z;
}

// Every item's state: no rejection yet (key = all ones), no automorphism, well formed.
__global__ void ksys_seg_init_kernel(KsysSeg *state, uint32_t n_items, const uint64_t *d_n) {
    const uint32_t n = d_n ? (uint32_t)*d_n : n_items;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        state[i] = KsysSeg{~0ull, 0u, 0u};
}

__device__ __forceinline__ unsigned long long volatile_key(const unsigned long long *p) {
    return *reinterpret_cast<const volatile unsigned long long *>(p);
}

// The check of a batch with every matrix's candidates split into segments: the
// unit of work is one (segment, item) pair, taken in segment-major order from a
// 64-bit work counter, so a level of a few hundred matrices whose canonical members
// try all ng! * 2^ng * rounds relabelings still fills the GPU.  Every segment's
// warp publishes a rejection as the key (candidate << 32 | player index) with an
// atomic minimum, and skips chunks that start after the smallest key seen: every
// candidate before the first rejecting one is still evaluated, so the verdict,
// m_playerIndex, the relabelings tried and |Aut| are those of the one-warp check.
__global__ void __launch_bounds__(KTPB) ksys_seg_kernel(const Item *__restrict__ items, uint32_t n_items,
                                                        const uint64_t *d_n, const uint8_t *__restrict__ bytes,
                                                        uint32_t seg_cands, uint64_t total_max,
                                                        uint32_t resident_warps, KsysSeg *state,
                                                        unsigned long long *ticket) {
    __shared__ uint64_t s_seq[KW][16], s_part[KW][16], s_pair[KW][16];
    const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const SegSize z = seg_size(n_items, d_n, seg_cands, total_max, resident_warps);
    const uint64_t n_units = z.n ? ((total_max + z.seg - 1) / z.seg) * z.n : 0;
    for (;;) {
        unsigned long long t = 0;
        if (lane == 0)
            t = atomicAdd(ticket, 1ull);
        t = __shfl_sync(0xFFFFFFFFu, t, 0);
        if (t >= n_units)
            break;
        const uint32_t it = (uint32_t)(t % z.n);
        const uint32_t seg = (uint32_t)(t / z.n);
        const Item item = items[it];
        const unsigned np = item.ncols, nr = item.nrows, ng = np >> 1;
        KsysSeg &st = state[it];
        const uint64_t start = (uint64_t)seg * z.seg;
        // past this item's candidates (a smaller shape than the launch's widest)
        if (seg && np >= 4 && np <= KS_NPMAX && start >= (uint64_t)(c_fact[ng] << ng) * nr)
            continue;
        // rejected before this segment
        if ((volatile_key(&st.key) >> 32) < start)
            continue;
        bool consecutive = false;
        const bool ok = load_item(item, bytes, s_seq[warp], s_part[warp], s_pair[warp], lane, &consecutive);
        if (!ok) {
            if (lane == 0 && seg == 0)
                st.bad = 1u;
            continue;
        }
        const uint64_t total = (uint64_t)(c_fact[ng] << ng) * nr;
        const uint64_t end = start + z.seg < total ? start + z.seg : total;
        const int pidx0 = (int)(nr * np) - 2 - 1;
        unsigned n_aut = 0;
        for (uint64_t base = start; base < end; base += 32u) {
            if ((volatile_key(&st.key) >> 32) < base)
                break;
            const unsigned c = (unsigned)base + lane;
            Cand o;
            o.res = 1;
            if (c < end)
                eval_candidate(c, np, ng, nr, s_seq[warp], s_part[warp], s_pair[warp], consecutive, o);
            const unsigned rej = __ballot_sync(0xFFFFFFFFu, c < end && o.res < 0);
            unsigned aut = __ballot_sync(0xFFFFFFFFu, c < end && o.res == 0);
            if (rej) {
                const unsigned fl = __ffs(rej) - 1u;
                if (lane == fl) {
                    const int pi = player_index_of(o, np, s_seq[warp], pidx0);
                    atomicMin(&st.key, ((unsigned long long)c << 32) | (unsigned)pi);
                }
                break;   // the automorphisms of a rejected matrix are not reported
            }
            n_aut += __popc(aut);
        }
        if (lane == 0 && n_aut)
            atomicAdd(&st.n_aut, n_aut);
    }
}

// The outputs of the segmented check, one thread per item.
__global__ void ksys_seg_finish_kernel(const Item *__restrict__ items, uint32_t n_items, const uint64_t *d_n,
                                       const KsysSeg *state, Outputs out) {
    const uint32_t n = d_n ? (uint32_t)*d_n : n_items;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const Item item = items[i];
        const KsysSeg st = state[i];
        const unsigned np = item.ncols, nr = item.nrows, ng = np >> 1;
        const bool ok = !st.bad && item.kind == KIND_KSYS && np >= 4 && np <= KS_NPMAX && !(np & 1u) && nr >= 1 &&
                        nr < np;
        const bool canonical = ok && st.key == ~0ull;
        const uint64_t total = ok ? (uint64_t)(c_fact[ng] << ng) * nr : 0;
        // candidate 0 (the identity) is not compared
        const uint64_t cands = !ok ? 0 : canonical ? total - 1 : (st.key >> 32);
        const int pidx = canonical || !ok ? (int)(nr * np) - 2 - 1 : (int)(uint32_t)st.key;
        write_item(out, item.out_idx, ok, canonical, false, pidx, st.n_aut, cands, false, np);
    }
}

// ---- k-systems with groups of 3 or 4 ---------------------------------------
// One relabeling is evaluated by kg_eval (canon_kgen.cuh).  Work split, early stop and
// outputs are those of the segmented check of group size 2: one (segment, item) unit per
// warp task, the first rejection kept by an atomic minimum of (candidate << 32 | player
// index), |Aut| reported for canonical matrices.
// Loads one item's rounds into the warp's tables and checks their form (all 32 lanes).
__device__ __noinline__ bool kg_load(const Item &item, unsigned g, const uint8_t *__restrict__ bytes, KgTables &T,
                        unsigned lane) {
    const unsigned np = item.ncols, nr = item.nrows, ng = np / g;
    bool ok = item.kind == KIND_KSYS && kg_shape_ok(np, g, nr);
    if (ok && lane < nr) {
        const uint8_t *row = bytes + item.data_off + lane * np;
        uint64_t sq = 0, ps = 0;
        unsigned seen = 0;
        for (unsigned p = 0; p < np; ++p) {
            const unsigned x = row[p];
            if (x >= np || ((seen >> x) & 1u))
                ok = false;
            seen |= 1u << (x & 15u);
            sq = nib_set(sq, p, x);
            ps = nib_set(ps, x, p);
            // players ascending inside a group, groups by their first player
            if (p % g && x <= row[p - 1])
                ok = false;
            if (p && p % g == 0 && x <= row[p - g])
                ok = false;
            if (lane == 0 && x != p)
                ok = false;   // round 0 = 0 1 2 .. np-1
        }
        T.seq[lane] = sq;
        T.pos[lane] = ps;
        for (unsigned k = 0; k < ng; ++k) {
            uint32_t l[4];
            for (unsigned e = 0; e < 4; ++e)
                l[e] = e < g ? row[k * g + e] & 15u : 0u;
            T.okey[lane][k] = (uint16_t)kg_key(l, g);
        }
    }
    ok = __all_sync(0xFFFFFFFFu, ok);
    __syncwarp();
    // no pair of players in two groups
    if (ok && lane == 0) {
        uint32_t pairs[16] = {};
        for (unsigned r = 0; r < nr && ok; ++r) {
            for (unsigned k = 0; k < ng; ++k)
                for (unsigned e = 0; e < g; ++e)
                    for (unsigned f = e + 1; f < g; ++f) {
                        const unsigned x = nib_get(T.seq[r], k * g + e), y = nib_get(T.seq[r], k * g + f);
                        if ((pairs[x] >> y) & 1u)
                            ok = false;
                        pairs[x] |= 1u << y;
                        pairs[y] |= 1u << x;
                    }
        }
    }
    ok = __shfl_sync(0xFFFFFFFFu, ok, 0);
    return ok;
}

// With CANON_SAVE_AUTS an item's automorphisms are counted one by one in KsysSeg::n_aut,
// whose old value is the arena slot each one is written to (the first aut_cap of them, in
// the order the warps find them; canon_sync sorts the stored set as CGroupInfo keeps it);
// they are reported for canonical matrices, whose every relabeling is tried.
__global__ void __launch_bounds__(KTPB) kgen_seg_kernel(const Item *__restrict__ items, uint32_t n_items,
                                                        const uint8_t *__restrict__ bytes, uint32_t seg_cands,
                                                        uint64_t n_units, KsysSeg *state,
                                                        unsigned long long *ticket, Outputs out) {
    __shared__ KgTables s_t[KW];
    const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    for (;;) {
        unsigned long long t = 0;
        if (lane == 0)
            t = atomicAdd(ticket, 1ull);
        t = __shfl_sync(0xFFFFFFFFu, t, 0);
        if (t >= n_units)
            break;
        const uint32_t it = (uint32_t)(t % n_items);
        const uint32_t seg = (uint32_t)(t / n_items);
        const Item item = items[it];
        const unsigned g = item.pad, np = item.ncols, nr = item.nrows;
        KsysSeg &st = state[it];
        const uint64_t start = (uint64_t)seg * seg_cands;
        if (seg && kg_shape_ok(np, g, nr) && start >= kg_total(np, g, nr))
            continue;
        if ((volatile_key(&st.key) >> 32) < start)
            continue;
        const bool ok = kg_load(item, g, bytes, s_t[warp], lane);
        if (!ok) {
            if (lane == 0 && seg == 0)
                st.bad = 1u;
            continue;
        }
        const uint64_t total = kg_total(np, g, nr);
        const uint64_t end = start + seg_cands < total ? start + seg_cands : total;
        const int pidx0 = (int)(nr * np) - (int)g - 1;
        const uint8_t *heap = ksys::c_heap + ksys::c_heap_off[np / g] * 6u;
        const bool save = (item.flags & F_SAVE_AUTS) && out.auts;
        uint8_t *arena = save ? out.auts + (size_t)item.out_idx * out.aut_cap * 64u : nullptr;
        unsigned n_aut = 0;
        for (uint64_t base = start; base < end; base += 32u) {
            if ((volatile_key(&st.key) >> 32) < base)
                break;
            const unsigned c = (unsigned)base + lane;
            int res = 1, pi = pidx0;
            uint64_t ttr = 0;
            if (c < end)
                res = g == 3 ? kg_eval<3>(c, np, np / 3u, nr, s_t[warp], heap, pidx0, pi, ttr)
                             : kg_eval<4>(c, np, np / 4u, nr, s_t[warp], heap, pidx0, pi, ttr);
            const unsigned rej = __ballot_sync(0xFFFFFFFFu, c < end && res < 0);
            const unsigned aut = __ballot_sync(0xFFFFFFFFu, c < end && res == 0);
            if (rej) {
                const unsigned fl = __ffs(rej) - 1u;
                if (lane == fl)
                    atomicMin(&st.key, ((unsigned long long)c << 32) | (unsigned)pi);
                break;
            }
            if (save) {
                if ((aut >> lane) & 1u) {
                    const unsigned slot = atomicAdd(&st.n_aut, 1u);
                    if (slot < out.aut_cap)
                        for (unsigned x = 0; x < np; ++x)
                            arena[(size_t)slot * 64u + x] = (uint8_t)nib_get(ttr, x);
                }
            } else {
                n_aut += __popc(aut);
            }
        }
        if (lane == 0 && n_aut)
            atomicAdd(&st.n_aut, n_aut);
    }
}

// The outputs of the general check, one thread per item.
__global__ void kgen_finish_kernel(const Item *__restrict__ items, uint32_t n_items, const KsysSeg *state,
                                   Outputs out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_items; i += gridDim.x * blockDim.x) {
        const Item item = items[i];
        const KsysSeg st = state[i];
        const unsigned g = item.pad, np = item.ncols, nr = item.nrows;
        const bool ok = !st.bad && item.kind == KIND_KSYS && kg_shape_ok(np, g, nr);
        const bool canonical = ok && st.key == ~0ull;
        const uint64_t cands = !ok ? 0 : canonical ? kg_total(np, g, nr) - 1 : (st.key >> 32);
        const int pidx = canonical || !ok ? (int)(nr * np) - (int)g - 1 : (int)(uint32_t)st.key;
        const bool save = canonical && (item.flags & F_SAVE_AUTS) && out.auts;
        write_item(out, item.out_idx, ok, canonical, save && st.n_aut > out.aut_cap, pidx, st.n_aut, cands, save,
                   np);
    }
}

// One persistent kernel over a mixed batch (k-systems and incidence matrices of
// any shapes): every warp first takes k-system items from the first work counter,
// one warp per matrix, and then incidence matrices from the second, one thread
// per matrix, so a warp never waits for lanes of the other kind and the long
// incidence checks fill the end of the launch.
constexpr int MTPB = bibd::TPB;     // 64: the per-thread shared-memory layout of the incidence checker
constexpr int MW = MTPB / 32;

// BCAP / VCAP bound the columns / rows of every incidence item of the launch, so the
// per-thread state is sized by the launch's widest shape (v <= 15, b <= 35: 413 B,
// 8 blocks of 64 per SM, against 6 for the general 16 x 63 layout).
template <int BCAP, int VCAP>
__global__ void __launch_bounds__(MTPB) mixed_kernel(const Item *__restrict__ bitems, uint32_t nb,
                                                     const Item *__restrict__ kitems, uint32_t nk,
                                                     const uint64_t *__restrict__ words,
                                                     const uint8_t *__restrict__ bytes, Outputs out,
                                                     uint64_t max_trials, unsigned *ticket) {
    __shared__ uint64_t s_seq[MW][16], s_part[MW][16], s_pair[MW][16];
    __shared__ uint64_t s_rows[VCAP * MTPB];
    __shared__ uint64_t s_lvl[(VCAP + 1) * MTPB];
    __shared__ uint32_t s_vd[VCAP * MTPB];
    __shared__ uint16_t s_cm[BCAP * MTPB];
    __shared__ uint8_t s_pc[BCAP * MTPB];
    const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31u, tid = threadIdx.x;
    for (;;) {
        unsigned it = 0;
        if (lane == 0)
            it = atomicAdd(ticket, 1u);
        it = __shfl_sync(0xFFFFFFFFu, it, 0);
        if (it >= nk)
            break;
        check_item_warp(kitems[it], bytes, out, s_seq[warp], s_part[warp], s_pair[warp], lane);
    }
    bibd::Smem sm{s_rows + tid, s_lvl + tid, s_pc + tid, s_cm + tid, s_vd + tid};
    for (;;) {
        const unsigned it = atomicAdd(ticket + 1, 1u);
        if (it >= nb)
            break;
        const Item item = bitems[it];
        if (item.nrows > VCAP || item.ncols > BCAP) {
            // wider than the launch was sized for (the launcher sizes it by the batch)
            Item bad = item;
            bad.kind = 0xFFu;
            bibd::check_item(sm, bad, words, out, max_trials);
            continue;
        }
        bibd::check_item(sm, item, words, out, max_trials);
    }
}

}  // namespace

cudaError_t launch_mixed_check(const Item *d_bitems, uint32_t nb, const Item *d_kitems, uint32_t nk,
                               const uint64_t *d_words, const uint8_t *d_bytes, Outputs out,
                               uint64_t max_trials, unsigned *tk, int num_sms, cudaStream_t s, uint32_t max_b,
                               uint32_t max_v) {
    if (!nb && !nk)
        return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(tk, 0, 2 * sizeof(unsigned), s);
    if (e != cudaSuccess)
        return e;
    const int shape = (max_v <= 15 && max_b <= 35) ? 0 : (max_b <= 40 ? 1 : 2);
    const void *kfn = shape == 0 ? (const void *)mixed_kernel<35, 15>
                      : shape == 1 ? (const void *)mixed_kernel<40, 16>
                                   : (const void *)mixed_kernel<64, 16>;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, MTPB, 0);
    if (e != cudaSuccess)
        return e;
    if (per_sm < 1)
        per_sm = 1;
    int grid = per_sm * (num_sms > 0 ? num_sms : 1);
    const long need = (long)((nb + MTPB - 1) / MTPB) + (long)((nk + MW - 1) / MW);
    if (grid > need)
        grid = (int)need;
    if (shape == 0)
        mixed_kernel<35, 15><<<grid, MTPB, 0, s>>>(d_bitems, nb, d_kitems, nk, d_words, d_bytes, out, max_trials, tk);
    else if (shape == 1)
        mixed_kernel<40, 16><<<grid, MTPB, 0, s>>>(d_bitems, nb, d_kitems, nk, d_words, d_bytes, out, max_trials, tk);
    else
        mixed_kernel<64, 16><<<grid, MTPB, 0, s>>>(d_bitems, nb, d_kitems, nk, d_words, d_bytes, out, max_trials, tk);
    return cudaGetLastError();
}

cudaError_t ksys_upload_tables() {
    uint8_t heap[ksys::HEAP_TOTAL * 6] = {};
    uint32_t off[7] = {}, fact[7] = {1, 1, 2, 6, 24, 120, 720};
    uint32_t pos = 0;
    for (int ng = 1; ng <= 6; ++ng) {
        off[ng] = pos;
        // Heap's permutations without recursion (Phillip Paul Fuchs), as canonizator() runs them
        uint8_t a[7], p[7];
        for (int i = 0; i < ng; ++i)
            a[i] = p[i] = (uint8_t)i;
        p[ng] = (uint8_t)ng;
        for (int i = 0; i < ng; ++i)
            heap[pos * 6 + i] = a[i];
        ++pos;
        int i = 1;
        while (i < ng) {
            p[i]--;
            const int j = (i % 2) ? p[i] : 0;
            const uint8_t t = a[i];
            a[i] = a[j];
            a[j] = t;
            for (int k = 0; k < ng; ++k)
                heap[pos * 6 + k] = a[k];
            ++pos;
            i = 0;
            while (!p[++i])
                p[i] = (uint8_t)i;
        }
    }
    cudaError_t e = cudaMemcpyToSymbol(ksys::c_heap, heap, sizeof(heap));
    if (e == cudaSuccess)
        e = cudaMemcpyToSymbol(ksys::c_heap_off, off, sizeof(off));
    if (e == cudaSuccess)
        e = cudaMemcpyToSymbol(ksys::c_fact, fact, sizeof(fact));
    return e;
}

cudaError_t launch_ksys_check(const Item *d_items, uint32_t n_items, const uint8_t *d_bytes, Outputs out,
                              unsigned *tk, int num_sms, cudaStream_t s) {
    if (!n_items)
        return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(tk, 0, sizeof(unsigned), s);
    if (e != cudaSuccess)
        return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ksys_kernel, ksys::KTPB, 0);
    if (e != cudaSuccess)
        return e;
    if (per_sm < 1)
        per_sm = 1;
    int grid = per_sm * (num_sms > 0 ? num_sms : 1);
    const int need = (int)((n_items + ksys::KW - 1) / ksys::KW);
    if (grid > need)
        grid = need;
    ksys_kernel<<<grid, ksys::KTPB, 0, s>>>(d_items, n_items, d_bytes, out, tk);
    return cudaGetLastError();
}

// seg_cands: candidates per segment (a multiple of 32, or 0 = chosen on the device
// from the item count); total_max: the most candidates of any item (ng! * 2^ng *
// rounds), which sets the segments per item.  d_n (optional): the item count in
// device memory, at most n_items, which then only sizes the grids; the work counter
// is d_state[n_items].
cudaError_t launch_ksys_check_split(const Item *d_items, uint32_t n_items, const uint8_t *d_bytes, Outputs out,
                                   uint32_t seg_cands, uint64_t total_max, KsysSeg *d_state, int num_sms,
                                   cudaStream_t s, const uint64_t *d_n) {
    if (!n_items)
        return cudaSuccess;
    if (seg_cands & 31u)
        return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(d_state + n_items, 0, sizeof(KsysSeg), s);
    if (e != cudaSuccess)
        return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ksys_seg_kernel, ksys::KTPB, 0);
    if (e != cudaSuccess)
        return e;
    if (per_sm < 1)
        per_sm = 1;
    const int sms = num_sms > 0 ? num_sms : 1;
    uint64_t grid = (uint64_t)per_sm * sms;
    if (!d_n && seg_cands) {
        const uint64_t units = ((total_max + seg_cands - 1) / seg_cands) * n_items;
        const uint64_t need = (units + ksys::KW - 1) / ksys::KW;
        if (grid > need)
            grid = need;
    }
    int gi = (int)((n_items + 255) / 256);
    if (gi > 4 * sms)
        gi = 4 * sms;
    ksys_seg_init_kernel<<<gi, 256, 0, s>>>(d_state, n_items, d_n);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    unsigned long long *ticket = reinterpret_cast<unsigned long long *>(d_state + n_items);
    ksys_seg_kernel<<<(int)grid, ksys::KTPB, 0, s>>>(d_items, n_items, d_n, d_bytes, seg_cands, total_max,
                                                     (uint32_t)(sms * KSYS_RESIDENT_WARPS_PER_SM), d_state, ticket);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    ksys_seg_finish_kernel<<<gi, 256, 0, s>>>(d_items, n_items, d_n, d_state, out);
    return cudaGetLastError();
}
// the check of k-systems with groups of 3 or 4 (Item::pad = the group size): every item's
// relabelings in segments of seg_cands over warps; total_max = the most of any item
cudaError_t launch_kgen_check(const Item *d_items, uint32_t n_items, const uint8_t *d_bytes, Outputs out,
                              uint32_t seg_cands, uint64_t total_max, KsysSeg *d_state, int num_sms,
                              cudaStream_t s) {
    if (!n_items)
        return cudaSuccess;
    if (seg_cands < 32 || (seg_cands & 31u))
        return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(d_state + n_items, 0, sizeof(KsysSeg), s);
    if (e != cudaSuccess)
        return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kgen_seg_kernel, ksys::KTPB, 0);
    if (e != cudaSuccess)
        return e;
    if (per_sm < 1)
        per_sm = 1;
    const int sms = num_sms > 0 ? num_sms : 1;
    const uint64_t units = ((total_max + seg_cands - 1) / seg_cands) * n_items;
    uint64_t grid = (uint64_t)per_sm * sms;
    const uint64_t need = (units + ksys::KW - 1) / ksys::KW;
    if (grid > need)
        grid = need;
    int gi = (int)((n_items + 255) / 256);
    if (gi > 4 * sms)
        gi = 4 * sms;
    ksys_seg_init_kernel<<<gi, 256, 0, s>>>(d_state, n_items, nullptr);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    unsigned long long *ticket = reinterpret_cast<unsigned long long *>(d_state + n_items);
    kgen_seg_kernel<<<(int)grid, ksys::KTPB, 0, s>>>(d_items, n_items, d_bytes, seg_cands, units, d_state, ticket,
                                                     out);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    kgen_finish_kernel<<<gi, 256, 0, s>>>(d_items, n_items, d_state, out);
    return cudaGetLastError();
}

}  // namespace canon
