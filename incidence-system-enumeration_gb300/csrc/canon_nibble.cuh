// canon_nibble.cuh -- nibble-packed small permutations (up to 16 entries in one uint64).
#pragma once
#include <cstdint>

#ifndef __CUDACC__
// host-only translation units (g++) include the host-and-device helpers too
#define __host__
#define __device__
#define __forceinline__ inline
#endif

namespace canon {

constexpr uint64_t NIB_ID16 = 0xFEDCBA9876543210ull;   // identity permutation of 0..15
constexpr uint64_t NIB_ONES = 0x1111111111111111ull;

__host__ __device__ __forceinline__ unsigned nib_get(uint64_t p, unsigned i) {
    return (unsigned)(p >> ((i & 15u) << 2)) & 15u;
}
__host__ __device__ __forceinline__ uint64_t nib_set(uint64_t p, unsigned i, unsigned x) {
    const unsigned sh = (i & 15u) << 2;
    return (p & ~(15ull << sh)) | ((uint64_t)(x & 15u) << sh);
}

// splitmix64 stream (same constants as the host generator)
__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
// uniform integer in [0, n) by multiply-shift of the high 32 bits
__host__ __device__ __forceinline__ uint32_t rand_below(uint64_t &s, uint32_t n) {
    return (uint32_t)(((splitmix64(s) >> 32) * (uint64_t)n) >> 32);
}
// per-item stream of a seeded batch
__host__ __device__ __forceinline__ uint64_t item_stream(uint64_t seed, uint64_t index) {
    return seed ^ (index * 0xD1B54A32D192ED03ull);
}

}  // namespace canon
