// canon_gen.cu -- seeded synthetic STS(v) batches on the device.
//
// Item i draws from its own splitmix64 stream: a random Steiner triple system by
// Stinson's hill-climbing (D. R. Stinson, "Hill-climbing algorithms for the
// construction of combinatorial designs", Annals of Discrete Mathematics 26,
// 1985), then a uniform row permutation and a uniform column permutation
// (Fisher-Yates).  Row r of the output is point prow[r], column c is block
// pcol[c].  One thread builds one matrix in local memory.
#include "canon_internal.h"
#include "canon_nibble.cuh"

namespace canon {

namespace {

constexpr int GTPB = 128;
constexpr int GVMAX = 16;

__global__ void __launch_bounds__(GTPB) sts_generate_kernel(uint32_t n, uint32_t v, uint64_t seed,
                                                            uint64_t *__restrict__ rows) {
    const uint32_t b = v * (v - 1) / 6;
    for (uint32_t it = blockIdx.x * GTPB + threadIdx.x; it < n; it += gridDim.x * GTPB) {
        uint64_t s = item_stream(seed, it);
        int8_t cov[GVMAX][GVMAX];
        uint8_t blk[64][3];
        for (int i = 0; i < GVMAX; ++i)
            for (int j = 0; j < GVMAX; ++j)
                cov[i][j] = -1;
        uint32_t nb = 0;
        // bounded: a hill-climb on STS(15) takes a few hundred steps
        for (uint32_t step = 0; nb < b && step < (1u << 20); ++step) {
            int x, nc;
            int cand[GVMAX];
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
        uint8_t prow[GVMAX], pcol[64];
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
        uint8_t rowof[GVMAX];
        for (uint32_t r = 0; r < v; ++r)
            rowof[prow[r]] = (uint8_t)r;
        uint64_t out[GVMAX];
        for (uint32_t r = 0; r < v; ++r)
            out[r] = 0;
        for (uint32_t c = 0; c < b; ++c) {
            const uint8_t *B = blk[pcol[c]];
            for (int a = 0; a < 3; ++a)
                out[rowof[B[a]]] |= 1ull << c;
        }
        for (uint32_t r = 0; r < v; ++r)
            rows[(size_t)it * v + r] = out[r];
    }
}

}  // namespace

cudaError_t launch_sts_generate(uint32_t n, uint32_t v, uint64_t seed, uint64_t *d_rows, int num_sms,
                                cudaStream_t s) {
    if (!n)
        return cudaSuccess;
    int grid = 4 * (num_sms > 0 ? num_sms : 1);
    const int need = (int)((n + GTPB - 1) / GTPB);
    if (grid > need)
        grid = need;
    sts_generate_kernel<<<grid, GTPB, 0, s>>>(n, v, seed, d_rows);
    return cudaGetLastError();
}

}  // namespace canon
