// canon_sts.cuh -- a random Steiner triple system STS(v) by Stinson's hill-climbing
// (D. R. Stinson, "Hill-climbing algorithms for the construction of combinatorial
// designs", Annals of Discrete Mathematics 26, 1985), then a uniform row permutation
// and a uniform column permutation (Fisher-Yates).  Host and device code: the device
// generator of seeded check batches and the host generator of partial designs use it.
#pragma once
#include <cstdint>

#include "canon_nibble.cuh"

namespace canon {

constexpr int STS_VMAX = 16;

// rows[r] = row r of the incidence matrix (bit c = column c); v = 1 or 3 (mod 6),
// v <= 15.  Row r of the output is point prow[r], column c is block pcol[c].
__host__ __device__ inline void sts_random_rows(uint32_t v, uint64_t &s, uint64_t *rows) {
    const uint32_t b = v * (v - 1) / 6;
    int8_t cov[STS_VMAX][STS_VMAX];
    uint8_t blk[64][3];
    for (int i = 0; i < STS_VMAX; ++i)
        for (int j = 0; j < STS_VMAX; ++j)
            cov[i][j] = -1;
    uint32_t nb = 0;
    // bounded: a hill-climb on STS(15) takes a few hundred steps
    for (uint32_t step = 0; nb < b && step < (1u << 20); ++step) {
        int x, nc;
        int cand[STS_VMAX];
        for (;;) {
            x = (int)rand_below(s, v);
            nc = 0;
            for (int y = 0; y < (int)v; ++y)
                if (y != x && cov[x][y] < 0)
                    cand[nc++] = y;
            if (nc >= 2)
                break;
        }
        const int iy = (int)rand_below(s, (uint32_t)nc);
        int iz = (int)rand_below(s, (uint32_t)(nc - 1));
        if (iz >= iy)
            ++iz;
        const int y = cand[iy], z = cand[iz];
        int slot = cov[y][z];
        if (slot < 0) {
            slot = (int)nb++;
        } else {
            for (int a = 0; a < 3; ++a)
                for (int c = 0; c < 3; ++c)
                    if (a != c)
                        cov[blk[slot][a]][blk[slot][c]] = -1;
        }
        blk[slot][0] = (uint8_t)x;
        blk[slot][1] = (uint8_t)y;
        blk[slot][2] = (uint8_t)z;
        for (int a = 0; a < 3; ++a)
            for (int c = 0; c < 3; ++c)
                if (a != c)
                    cov[blk[slot][a]][blk[slot][c]] = (int8_t)slot;
    }
    uint8_t prow[STS_VMAX], pcol[64];
    for (uint32_t i = 0; i < v; ++i)
        prow[i] = (uint8_t)i;
    for (uint32_t i = 0; i < b; ++i)
        pcol[i] = (uint8_t)i;
    for (uint32_t k = v - 1; k >= 1; --k) {
        const uint32_t j = rand_below(s, k + 1);
        const uint8_t t = prow[k];
        prow[k] = prow[j];
        prow[j] = t;
    }
    for (uint32_t k = b - 1; k >= 1; --k) {
        const uint32_t j = rand_below(s, k + 1);
        const uint8_t t = pcol[k];
        pcol[k] = pcol[j];
        pcol[j] = t;
    }
    // point -> output row
    uint8_t rowof[STS_VMAX];
    for (uint32_t r = 0; r < v; ++r)
        rowof[prow[r]] = (uint8_t)r;
    for (uint32_t r = 0; r < v; ++r)
        rows[r] = 0;
    for (uint32_t c = 0; c < b; ++c) {
        const uint8_t *B = blk[pcol[c]];
        for (int a = 0; a < 3; ++a)
            rows[rowof[B[a]]] |= 1ull << c;
    }
}

}  // namespace canon
