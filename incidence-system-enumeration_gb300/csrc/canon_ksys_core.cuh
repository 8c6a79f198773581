// canon_ksys_core.cuh -- device search of the k-system checker (group size 2).
// Included by canon_ksys.cu (the k-system kernel and the mixed persistent kernel).
#pragma once
#include "canon_internal.h"
#include "canon_nibble.cuh"

namespace canon {
namespace ksys {
// internal linkage: the header is compiled into more than one translation unit
namespace {

constexpr int KW = 4;          // warps per block
constexpr int KTPB = 32 * KW;
constexpr int HEAP_TOTAL = 1 + 2 + 6 + 24 + 120 + 720;

__constant__ uint8_t c_heap[HEAP_TOTAL * 6];   // group order of every Heap permutation, ng = 1..6
__constant__ uint32_t c_heap_off[7];
__constant__ uint32_t c_fact[7];

struct Cand {
    int res;          // 0 automorphism, -1 smaller (reject), > 0 greater
    unsigned row;     // output round of the first difference
    unsigned src;     // input round that gave it
    unsigned daymax;  // max input round of the equal output rounds before it
    uint64_t ttr;     // relabeling (player -> new label)
    uint64_t inv;     // inverse relabeling
    uint64_t q;       // relabelled partner table of the differing round
};

__device__ __forceinline__ void eval_candidate(unsigned c, unsigned np, unsigned ng, unsigned nr,
                                               const uint64_t *seq, const uint64_t *part,
                                               const uint64_t *pair, bool consecutive, Cand &o) {
    const unsigned d = c % nr;
    const unsigned qd = c / nr;
    const unsigned t = qd & ((1u << ng) - 1u);
    const unsigned h = qd >> ng;
    const uint8_t *a = c_heap + (c_heap_off[ng] + h) * 6u;
    // the relabeling (player -> label) and its inverse, pair by pair of round d: the
    // players of its i-th pair get label 2a[i] + t_i and the other label of that group,
    // in the order the in-group bit says (cnvCheckKm, cnv.cpp:168-185)
    const uint64_t sd = seq[d];
    uint64_t ttr = 0, inv = 0;
    for (unsigned i = 0; i < ng; ++i) {
        const unsigned lab = 2u * a[i] + ((t >> (ng - 1u - i)) & 1u);
        const unsigned p0 = nib_get(sd, 2u * i), p1 = nib_get(sd, 2u * i + 1u);
        ttr |= ((uint64_t)lab << (4u * p0)) | ((uint64_t)(lab ^ 1u) << (4u * p1));
        inv |= ((uint64_t)p0 << (4u * lab)) | ((uint64_t)p1 << (4u * (lab ^ 1u)));
    }
    o.ttr = ttr;
    o.res = 0;
    if (c == 0)
        return;   // the identity is registered without a comparison (cnv.cpp:85-89)
    o.inv = inv;
    const unsigned u = nib_get(inv, 0);
    // second entries (partner of label 0) of the relabelled rounds; the sorted
    // form lists the rounds in increasing order of it (kmSortRowsBy2ndValue)
    unsigned second = 0;
    if (!consecutive)
        for (unsigned r = 0; r < nr; ++r)
            second |= 1u << nib_get(ttr, nib_get(part[r], u));
    unsigned daymax = d;
    for (unsigned i = consecutive ? 1u : 0u; i < nr; ++i) {
        unsigned w;
        if (consecutive) {
            // rounds 0..i-1 matched second entries 1..i; equality needs i+1 next
            w = nib_get(inv, i + 1u);
            if (!nib_get(pair[u], w)) {
                o.res = 2;
                return;
            }
        } else {
            const unsigned tv = __ffs(second) - 1u;
            second &= second - 1u;
            w = nib_get(inv, tv);
        }
        const unsigned r = nib_get(pair[u], w) - 1u;
        const uint64_t pr = part[r];
        const uint64_t orig = part[i];
        // the relabelled round r against round i, label by label (q[y] = the label of the
        // partner of the player labelled y): rounds in canonical pair order compare like
        // their partner tables, so the first label whose partner differs decides, and
        // most relabelings differ within the first labels
        int cmp = 0;
        for (unsigned y = 0; y < np; ++y) {
            const unsigned qy = nib_get(ttr, nib_get(pr, nib_get(inv, y)));
            const unsigned oy = nib_get(orig, y);
            if (qy != oy) {
                cmp = qy < oy ? -1 : 1;
                break;
            }
        }
        if (!cmp) {
            if (daymax < r)
                daymax = r;
            continue;
        }
        if (cmp < 0) {
            // the whole relabelled round, for the player index of the rejection
            uint64_t q = 0;
            for (unsigned x = 0; x < np; ++x)
                q = nib_set(q, nib_get(ttr, x), nib_get(ttr, nib_get(pr, x)));
            o.res = -1;
            o.row = i;
            o.src = r;
            o.daymax = daymax;
            o.q = q;
        } else {
            o.res = 1;
        }
        return;
    }
}

// setPlayerIndex() / setPlayerIndexByPos(), kmSupport.cpp:314-356
__device__ int player_index_of(const Cand &o, unsigned np, const uint64_t *seq, int current) {
    if (o.daymax > o.src)
        return current;
    // the differing round of the relabelled matrix in the reference's byte order
    uint64_t co = 0, taken = 0;
    unsigned pos = 0;
    for (unsigned x = 0; x < np; ++x) {
        if ((taken >> x) & 1u)
            continue;
        const unsigned y = nib_get(o.q, x);
        co = nib_set(co, pos, x);
        co = nib_set(co, pos + 1u, y);
        taken |= (1ull << x) | (1ull << y);
        pos += 2u;
    }
    const uint64_t ci = seq[o.row];
    const unsigned imax = np - 3u;
    unsigned ip = 0;
    for (; ip < imax; ++ip)
        if (nib_get(co, ip) < nib_get(ci, ip))
            break;
    uint64_t tpr = 0;
    const uint64_t from = seq[o.src];
    for (unsigned p = 0; p < np; ++p)
        tpr = nib_set(tpr, nib_get(from, p), p);
    unsigned j = 0;
    for (unsigned p = 0; p <= ip; ++p) {
        const unsigned k = nib_get(o.inv, nib_get(co, p));
        const unsigned v = nib_get(tpr, k);
        if (j < v)
            j = v;
    }
    const int pi = (int)(o.src * np + j);
    return pi < current ? pi : current;
}

// Loads one item's rounds into the warp's tables (all 32 lanes call it together):
// seq = position -> player, part = player -> partner per round, pair = for every
// player the round (+1) in which it meets each partner.  Returns whether the rounds
// are well formed; *consecutive = round i pairs player 0 with i+1 (every canonical
// matrix does), which allows the fast comparison path.
__device__ bool load_item(const Item &item, const uint8_t *__restrict__ bytes, uint64_t *seq, uint64_t *part,
                          uint64_t *pair, unsigned lane, bool *consecutive) {
    const unsigned np = item.ncols, nr = item.nrows;
    bool ok = item.kind == KIND_KSYS && np >= 4 && np <= KS_NPMAX && !(np & 1u) && nr >= 1 && nr < np;
    if (ok && lane < nr) {
        const uint8_t *row = bytes + item.data_off + lane * np;
        uint64_t sq = 0, pt = 0, seen = 0;
        int prev_first = -1;
        for (unsigned p = 0; p < np; p += 2) {
            const unsigned x = row[p], y = row[p + 1];
            if (x >= np || y >= np || x >= y || (int)x <= prev_first || ((seen >> x) & 1u) ||
                ((seen >> y) & 1u))
                ok = false;
            prev_first = (int)x;
            seen |= (1ull << (x & 63u)) | (1ull << (y & 63u));
            sq = nib_set(sq, p, x);
            sq = nib_set(sq, p + 1, y);
            pt = nib_set(pt, x, y);
            pt = nib_set(pt, y, x);
        }
        // round 0 = 0 1 2 .. np-1 (the first round is fixed)
        if (lane == 0)
            for (unsigned p = 0; p < np; ++p)
                if (row[p] != p)
                    ok = false;
        seq[lane] = sq;
        part[lane] = pt;
    }
    ok = __all_sync(0xFFFFFFFFu, ok);
    *consecutive = __all_sync(0xFFFFFFFFu, !(ok && lane < nr) || nib_get(part[lane], 0) == lane + 1u);
    __syncwarp();
    if (ok && lane < np) {
        uint64_t pr = 0;
        for (unsigned r = 0; r < nr; ++r) {
            const unsigned w = nib_get(part[r], lane);
            if (nib_get(pr, w))
                ok = false;   // a pair used twice
            pr = nib_set(pr, w, r + 1u);
        }
        pair[lane] = pr;
    }
    ok = __all_sync(0xFFFFFFFFu, ok);
    __syncwarp();
    return ok;
}

// The outputs of one k-system item (one thread writes them).
__device__ __forceinline__ void write_item(const Outputs &out, unsigned oi, bool ok, bool canonical, bool overflow,
                                           int pidx, uint64_t n_aut, uint64_t cands, bool save, unsigned np) {
    out.canonical[oi] = canonical ? 1 : 0;
    out.status[oi] = ok ? (overflow ? ST_PERM_OVF : 0) : ST_BADINPUT;
    out.reject_row[oi] = 0xFF;
    out.row_to_change[oi] = 0xFF;
    out.player_index[oi] = pidx;
    uint4 *w = reinterpret_cast<uint4 *>(out.witness + (size_t)oi * 16u);
    *w = make_uint4(~0u, ~0u, ~0u, ~0u);
    out.aut[2 * (size_t)oi] = canonical ? n_aut : 0;
    out.aut[2 * (size_t)oi + 1] = 0;
    out.trials[oi] = cands;
    out.n_auts[oi] = (uint16_t)(save ? (n_aut < out.aut_cap ? n_aut : out.aut_cap) : 0);
    out.len_aut[oi] = (uint8_t)np;
}

// cnvCheckNew() of one item by one warp (all 32 lanes call it together).
__device__ void check_item_warp(const Item &item, const uint8_t *__restrict__ bytes, Outputs out,
                                uint64_t *seq, uint64_t *part, uint64_t *pair, unsigned lane) {
    const unsigned np = item.ncols, nr = item.nrows, ng = np >> 1;
    const unsigned oi = item.out_idx;
    bool consecutive = false;
    bool ok = load_item(item, bytes, seq, part, pair, lane, &consecutive);

    int pidx = (int)(nr * np) - 2 - 1;      // cnvCheckNew(): nrows*numPlayers - groupSize - 1
    uint64_t n_aut = 0, cands = 0;
    bool canonical = ok;
    bool overflow = false;
    const bool save = ok && (item.flags & F_SAVE_AUTS) && out.auts;
    uint8_t *adst = save ? out.auts + (size_t)oi * out.aut_cap * 64u : nullptr;
    if (ok) {
        const unsigned total = (c_fact[ng] << ng) * nr;
        for (unsigned base = 0; base < total; base += 32u) {
            const unsigned c = base + lane;
            Cand o;
            o.res = 1;
            if (c < total)
                eval_candidate(c, np, ng, nr, seq, part, pair, consecutive, o);
            const unsigned rej = __ballot_sync(0xFFFFFFFFu, c < total && o.res < 0);
            unsigned aut = __ballot_sync(0xFFFFFFFFu, c < total && o.res == 0);
            unsigned upto = (total - base < 32u) ? (total - base) : 32u;
            if (rej) {
                const unsigned fl = __ffs(rej) - 1u;
                aut &= (1u << fl) - 1u;
                upto = fl + 1u;
                int pi = 0;
                if (lane == fl)
                    pi = player_index_of(o, np, seq, pidx);
                pidx = __shfl_sync(0xFFFFFFFFu, pi, fl);
                canonical = false;
            }
            if (save && ((aut >> lane) & 1u)) {
                const unsigned slot = (unsigned)n_aut + __popc(aut & ((1u << lane) - 1u));
                if (slot < out.aut_cap) {
                    uint8_t *dst = adst + slot * 64u;
                    for (unsigned x = 0; x < np; ++x)
                        dst[x] = (uint8_t)nib_get(o.ttr, x);
                }
            }
            n_aut += __popc(aut);
            cands += upto - (base == 0 ? 1u : 0u);   // candidate 0 is not compared
            if (rej)
                break;
        }
        if (save && n_aut > out.aut_cap)
            overflow = true;
    }
    if (lane == 0)
        write_item(out, oi, ok, canonical, overflow, pidx, n_aut, cands, save, np);
}

}  // namespace
}  // namespace ksys
}  // namespace canon
