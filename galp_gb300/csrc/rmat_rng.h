// rmat_rng.h -- counter-based R-MAT edge sampler shared by the CPU and GPU generators.
//
// Edge e of a graph with seed s descends `scale` levels of the recursive adjacency
// matrix; level l draws 32 random bits from a SplitMix64 finaliser applied to
// (s, e, l) and picks quadrant a/b/c/d by comparing them with cumulative thresholds
// scaled to 2^32.  Being a pure function of (s, e, l), every edge can be generated
// independently and identically on the host and on the device.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define GALP_RNG_HD __host__ __device__ __forceinline__
#else
#define GALP_RNG_HD inline
#endif

namespace galp {

GALP_RNG_HD uint64_t splitmix64_mix(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// (u << 32) | v of edge e before symmetrisation
GALP_RNG_HD uint64_t rmat_edge_key(uint64_t seed, uint64_t e, int scale, uint32_t ta, uint32_t tb, uint32_t tc)
{
    uint64_t u = 0, v = 0;
    const uint64_t base = splitmix64_mix(seed ^ 0x52D4A7F1C3B9E605ull) ^ (e * 0x9E3779B97F4A7C15ull);
    for (int l = 0; l < scale; ++l) {
        const uint32_t r = (uint32_t)(splitmix64_mix(base + (uint64_t)l * 0xD1B54A32D192ED03ull) >> 32);
        const uint64_t ub = r >= tb;               // quadrants c, d
        const uint64_t vb = (r >= ta && r < tb) || r >= tc;  // quadrants b, d
        u = (u << 1) | ub;
        v = (v << 1) | vb;
    }
    return (u << 32) | v;
}

}  // namespace galp
