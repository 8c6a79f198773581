// canon_ksys_rounds.cuh -- the next rounds of a partial 1-factorization (group size 2),
// host and device code (the device enumerator uses it; a host build tests it).
#pragma once
#include <cstddef>
#include <cstdint>

#ifndef __CUDACC__
#define __host__
#define __device__
#endif

namespace canon {

// The next round of a partial 1-factorization of K_np (group size 2): every perfect
// matching of the players whose pairs were not used in an earlier round, written as
// result() holds a round (pairs ascending, ordered by first player), with player 0
// meeting player d+1 in round d as in every canonical matrix.  This is the round
// construction of alldata::processOneDay() / getNextPlayer()
// (k-Factorization/TripleSys/Source/TripleSys.cpp:487-775) restricted to the matchings
// an orderly enumeration keeps; the children of a parent come in the order of the
// depth-first walk (partners in increasing order).  dst == nullptr: count only.
// second >= 0: only the rounds whose second pair (the lowest player after 0 and d+1)
// takes partner `second` -- the walk of one parent split into independent parts by that
// partner, which in increasing order give the parent's children in its order.
constexpr int KS_MAXNP = 12;

__host__ __device__ inline uint32_t ksys_children(int np, const uint8_t *parent, int d, uint8_t *dst,
                                                  int second = -1) {
    uint16_t used[KS_MAXNP];
    for (int a = 0; a < np; ++a)
        used[a] = 0;
    for (int r = 0; r < d; ++r)
        for (int i = 0; i < np; i += 2) {
            const int x = parent[r * np + i], y = parent[r * np + i + 1];
            used[x] |= (uint16_t)(1u << y);
            used[y] |= (uint16_t)(1u << x);
        }
    const int rl = d * np;          // bytes of the parent
    uint8_t row[KS_MAXNP];
    int next_c[KS_MAXNP / 2];       // per pair: the next partner to try
    unsigned taken = 0;
    int depth = 0;                  // pairs placed
    uint32_t count = 0;
    const int pairs = np / 2;
    next_c[0] = -1;
    for (;;) {
        // the lowest player not yet paired
        int a = 0;
        while ((taken >> a) & 1u)
            ++a;
        int c = next_c[depth] < 0 ? a + 1 : next_c[depth];
        for (; c < np; ++c) {
            if ((taken >> c) & 1u || ((used[a] >> c) & 1u))
                continue;
            if (a == 0 && c != d + 1)
                continue;
            if (depth == 1 && second >= 0 && c != second)
                continue;
            break;
        }
        if (c >= np) {
            // no partner left: back up one pair
            if (depth == 0)
                break;
            --depth;
            taken &= ~((1u << row[2 * depth]) | (1u << row[2 * depth + 1]));
            next_c[depth] = row[2 * depth + 1] + 1;
            continue;
        }
        row[2 * depth] = (uint8_t)a;
        row[2 * depth + 1] = (uint8_t)c;
        taken |= (1u << a) | (1u << c);
        if (depth + 1 == pairs) {
            if (dst) {
                uint8_t *o = dst + (size_t)count * (rl + np);
                for (int q = 0; q < rl; ++q)
                    o[q] = parent[q];
                for (int q = 0; q < np; ++q)
                    o[rl + q] = row[q];
            }
            ++count;
            taken &= ~((1u << a) | (1u << c));
            next_c[depth] = c + 1;
            continue;
        }
        ++depth;
        next_c[depth] = -1;
    }
    return count;
}

}  // namespace canon
