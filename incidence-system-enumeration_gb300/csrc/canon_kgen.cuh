// canon_kgen.cuh -- one relabeling of the k-system check with groups of 3 or 4,
// host and device code (the GPU kernel uses it; a host build tests it).
//
// cnvCheckNew() on the general path of the reference (kmProcessMatrix,
// k-Factorization/TripleSys/Source/kmSupport.cpp:220-313): a relabeling is (Heap
// permutation of the groups) x (an order inside every group: the g! orders of cnvInit(),
// cnv.cpp:45-64, as odometer digits, the first group most significant) x (the round mapped
// to round 0), in that nesting.  The relabelled rounds are brought to sorted form --
// players ascending inside every group, groups by their first player, rounds by their
// second entry -- and compared with the matrix round by round.  A group becomes a 16-bit
// key of its players ascending, the first in the top nibble: groups have equal size and
// distinct first players, so comparing the sorted keys of two rounds compares their
// sorted byte rows.
#pragma once
#include <cstdint>

#include "canon_nibble.cuh"

namespace canon {

constexpr int KG_NGMAX = 5;   // groups per round (np <= 16: 5 of 3 or 4 of 4)

struct KgTables {
    uint64_t seq[16];                 // round r: position -> player
    uint64_t pos[16];                 // round r: player -> position
    uint16_t okey[16][KG_NGMAX];      // round r's groups as keys, in order
};

__host__ __device__ __forceinline__ unsigned kg_ctz(unsigned x) {
#ifdef __CUDA_ARCH__
    return __ffs(x) - 1u;
#else
    return (unsigned)__builtin_ctz(x);
#endif
}

// the players l[0..g) ascending, the first in the top nibble (g = 3: the low nibble 0)
__host__ __device__ __forceinline__ uint32_t kg_key(const uint32_t *l, unsigned g) {
    uint32_t a = l[0], b = l[1], c = l[2], d = g == 4 ? l[3] : 15u;
    uint32_t t;
    if (a > b) { t = a; a = b; b = t; }
    if (c > d) { t = c; c = d; d = t; }
    if (a > c) { t = a; a = c; c = t; }
    if (b > d) { t = b; b = d; d = t; }
    if (b > c) { t = b; b = c; c = t; }
    return g == 4 ? (a << 12) | (b << 8) | (c << 4) | d : (a << 12) | (b << 8) | (c << 4);
}

// player p of a sorted round given as keys (the key picked by compares, so that the
// keys stay in registers)
template <unsigned g>
__host__ __device__ __forceinline__ unsigned kg_key_player(const uint32_t *key, unsigned p) {
    const unsigned k = p / g;
    uint32_t v = key[0];
#pragma unroll
    for (unsigned j = 1; j < (unsigned)KG_NGMAX; ++j)
        v = k == j ? key[j] : v;
    return (v >> (4u * (3u - p % g))) & 15u;
}

// In-group order t (0 .. G!-1) of cnvInit(): the G! orders of 0 .. G-1 in lexicographic
// order, entry j of order t taken from t's factorial digits (the j-th digit picks one of
// the entries not yet used), so no table is read.  Returned nibble-packed, entry j at 4j.
template <unsigned G>
__host__ __device__ __forceinline__ unsigned kg_group_order(unsigned t) {
    unsigned left = G == 3 ? 0x210u : 0x3210u;   // the entries not yet used, ascending
    unsigned out = 0, radix = G == 3 ? 2u : 6u;   // (G - 1 - j)!
#pragma unroll
    for (unsigned j = 0; j + 1 < G; ++j) {
        const unsigned k = t / radix;
        t -= k * radix;
        const unsigned sh = 4u * k;
        out |= ((left >> sh) & 15u) << (4u * j);
        left = (left & ((1u << sh) - 1u)) | ((left >> (sh + 4u)) << sh);
        radix = j + 2 < G ? radix / (G - 1u - j) : 1u;
    }
    out |= (left & 15u) << (4u * (G - 1u));
    return out;
}

// Relabeling c of the matrix in T (np players in ng groups of G, nr rounds).
// heap = the Heap permutations of ng groups (6 bytes each, group indices).  Returns 0 for
// an automorphism (the identity, c = 0, without a comparison, cnv.cpp:85-89), > 0 when
// the relabelled matrix is greater and -1 when it is smaller; then pi_out = min(pidx0,
// the m_playerIndex candidate of setPlayerIndex() / setPlayerIndexByPos(),
// kmSupport.cpp:314-356).  ttr_out = the relabeling (player -> label, nibble-packed), the
// permutation an automorphism is stored as.  G is a compile-time constant so that every
// division by the group size or by G! is a multiplication.
template <unsigned G>
__host__ __device__ __forceinline__ int kg_eval(unsigned c, unsigned np, unsigned ng, unsigned nr,
                                                const KgTables &T, const uint8_t *heap, int pidx0, int &pi_out,
                                                uint64_t &ttr_out) {
    constexpr unsigned g = G, gf = G == 3 ? 6u : 24u;
    unsigned gfn = 1;
    for (unsigned i = 0; i < ng; ++i)
        gfn *= gf;
    const unsigned d = c % nr;
    const unsigned q = c / nr;
    unsigned tgi = q % gfn;
    const unsigned h = q / gfn;
    const uint8_t *a = heap + h * 6u;
    // the in-group order of every group, the first group most significant
    unsigned tg[KG_NGMAX];
#pragma unroll
    for (int i = KG_NGMAX - 1; i >= 0; --i) {
        tg[i] = 0;
        if ((unsigned)i < ng) {
            tg[i] = tgi % gf;
            tgi /= gf;
        }
    }
    // the labels of round d's positions (cnvCheckKm, cnv.cpp:168-185): ttr = player ->
    // label, inv = label -> player
    uint64_t ttr = 0, inv = 0;
    const uint64_t sd = T.seq[d];
#pragma unroll
    for (unsigned i = 0; i < (unsigned)KG_NGMAX; ++i) {
        if (i < ng) {
            const unsigned ord = kg_group_order<G>(tg[i]);
            const unsigned base = (unsigned)a[i] * g;
#pragma unroll
            for (unsigned j = 0; j < g; ++j) {
                const unsigned lab = base + ((ord >> (4u * j)) & 15u);
                const unsigned pl = nib_get(sd, i * g + j);
                ttr |= (uint64_t)lab << (4u * pl);
                inv |= (uint64_t)pl << (4u * lab);
            }
        }
    }
    ttr_out = ttr;
    if (c == 0)
        return 0;
    // the second entry of every relabelled round: the least label among the group-mates
    // of the player labelled 0; the output rounds in increasing order of it.  Round d
    // becomes 0 1 .. np-1 (its groups take the label blocks whole), round 0 of the matrix:
    // it is the first output round (second entry 1; every other round has a larger one, as
    // the player labelled 1 meets the player labelled 0 in round d only), and it is equal,
    // so the comparison starts at output round 1 with day_max = d.
    const unsigned u = nib_get(inv, 0);
    unsigned mask2 = 0;
    uint64_t srcof = 0;
    for (unsigned r = 0; r < nr; ++r) {
        if (r == d)
            continue;
        const unsigned gi = nib_get(T.pos[r], u) / g;
        unsigned m = 15;
        for (unsigned e = 0; e < g; ++e) {
            const unsigned pl = nib_get(T.seq[r], gi * g + e);
            if (pl != u) {
                const unsigned lb = nib_get(ttr, pl);
                m = lb < m ? lb : m;
            }
        }
        mask2 |= 1u << m;
        srcof = nib_set(srcof, m, r);
    }
    unsigned day_max = d;
    for (unsigned i = 1; mask2; ++i) {
        const unsigned m = kg_ctz(mask2);
        mask2 &= mask2 - 1u;
        const unsigned r = nib_get(srcof, m);
        // the relabelled round r as sorted keys.  The group holding label 0 sorts first, and
        // its key alone usually decides (a relabelled round is mostly greater or smaller from
        // its second entry on), so it is compared before the other groups are built
        uint32_t key[KG_NGMAX] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu};
        const unsigned g0 = nib_get(T.pos[r], u) / g;
        {
            uint32_t l[4];
#pragma unroll
            for (unsigned e = 0; e < 4; ++e)
                l[e] = e < g ? (uint32_t)nib_get(ttr, nib_get(T.seq[r], g0 * g + e)) : 0u;
            key[0] = kg_key(l, g);
        }
        int cmp = 0;
        unsigned kd = 0;
        if (key[0] != T.okey[i][0]) {
            cmp = key[0] < T.okey[i][0] ? -1 : 1;
        } else {
#pragma unroll
            for (unsigned k = 1; k < (unsigned)KG_NGMAX; ++k) {
                if (k < ng) {
                    const unsigned grp = k - 1u + (k - 1u >= g0 ? 1u : 0u);   // the groups other than g0
                    uint32_t l[4];
#pragma unroll
                    for (unsigned e = 0; e < 4; ++e)
                        l[e] = e < g ? (uint32_t)nib_get(ttr, nib_get(T.seq[r], grp * g + e)) : 0u;
                    key[k] = kg_key(l, g);
                }
            }
#pragma unroll
            for (unsigned x = 2; x < (unsigned)KG_NGMAX; ++x)
#pragma unroll
                for (unsigned y = x; y > 1; --y)
                    if (key[y] < key[y - 1]) {
                        const uint32_t t = key[y];
                        key[y] = key[y - 1];
                        key[y - 1] = t;
                    }
#pragma unroll
            for (unsigned k = 1; k < (unsigned)KG_NGMAX; ++k) {
                if (!cmp && k < ng) {
                    const uint32_t ok = T.okey[i][k];
                    if (key[k] != ok) {
                        cmp = key[k] < ok ? -1 : 1;
                        kd = k;
                    }
                }
            }
        }
        if (!cmp) {
            if (day_max < r)
                day_max = r;
            continue;
        }
        if (cmp > 0)
            return 1;
        // the first position (below np - g - 1) where the relabelled round is below round
        // i, then the latest position in source round r of the players up to it
        int pi = pidx0;
        if (day_max <= r) {
            const unsigned imax = np - g - 1;
            unsigned ip = imax;
            for (unsigned p = kd * g; p < imax; ++p)
                if (kg_key_player<g>(key, p) < nib_get(T.seq[i], p)) {
                    ip = p;
                    break;
                }
            unsigned j = 0;
            for (unsigned p = 0; p <= ip; ++p) {
                const unsigned tp = nib_get(T.pos[r], nib_get(inv, kg_key_player<g>(key, p)));
                j = tp > j ? tp : j;
            }
            const int cand = (int)(r * np + j);
            pi = cand < pi ? cand : pi;
        }
        pi_out = pi;
        return -1;
    }
    return 0;
}

// relabelings of one check: (np/g)! * (g!)^(np/g) * rounds
__host__ __device__ __forceinline__ uint64_t kg_total(unsigned np, unsigned g, unsigned nr) {
    const unsigned ng = np / g, gf = g == 3 ? 6u : 24u;
    uint64_t t = 1;
    for (unsigned i = 2; i <= ng; ++i)
        t *= i;
    for (unsigned i = 0; i < ng; ++i)
        t *= gf;
    return t * nr;
}

// the shape checks of a matrix with groups of g
__host__ __device__ __forceinline__ bool kg_shape_ok(unsigned np, unsigned g, unsigned nr) {
    return (g == 3 || g == 4) && np <= 16 && np % g == 0 && np / g >= 2 && np / g <= (unsigned)KG_NGMAX &&
           nr >= 1 && nr < np;
}

}  // namespace canon
