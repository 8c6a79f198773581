// canon_ksys.cu -- canonicity test of k-systems (rounds of pairs, group size 2) on sm_103a.
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

}  // namespace canon
