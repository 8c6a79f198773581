// canon_gen.cu -- seeded synthetic STS(v) batches on the device.
//
// Item i draws from its own splitmix64 stream: a random Steiner triple system by
// Stinson's hill-climbing (D. R. Stinson, "Hill-climbing algorithms for the
// construction of combinatorial designs", Annals of Discrete Mathematics 26,
// 1985), then a uniform row permutation and a uniform column permutation
// (Fisher-Yates).  Row r of the output is point prow[r], column c is block
// pcol[c].  One thread builds one matrix in local memory.
#include "canon_internal.h"
#include "canon_sts.cuh"

namespace canon {

namespace {

constexpr int GTPB = 128;

__global__ void __launch_bounds__(GTPB) sts_generate_kernel(uint32_t n, uint32_t v, uint64_t seed,
                                                            uint64_t *__restrict__ rows) {
    for (uint32_t it = blockIdx.x * GTPB + threadIdx.x; it < n; it += gridDim.x * GTPB) {
        uint64_t s = item_stream(seed, it);
        uint64_t out[STS_VMAX];
        sts_random_rows(v, s, out);
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
