// lp_device.cuh -- device-side building blocks of the exact label-propagation update.
//
// Semantics reproduced (reference: label_propagation/src/dpp/dpp.cuh:104-138 and
// src/common/segmented_reduce.cuh:26-626): vertex v's neighbour labels, sorted
// ascending and run-length encoded, form runs [a, a+d) of a scope-wide run array
// (a = sum of the distinct-label counts of all earlier vertices in the scope).
// The new label is the label of the heaviest run, ties broken by the run's
// global position through the reference's segmented arg-max, whose closed form
// is resolve_rank() below.  Only the positions of the maximum-count runs
// ("candidates") matter: a lighter run never wins a comparison, and between
// candidates every comparison is decided by position alone.
#pragma once

#include <cstdint>
#include <climits>

#include "lp_resolve.h"

namespace galp {

constexpr uint32_t kEmpty = 0xFFFFFFFFu;  // hash-table empty key (labels are < 2^31)

__device__ __forceinline__ uint32_t mix32(uint32_t x)
{
    // murmur3 finaliser
    x ^= x >> 16;
    x *= 0x85EBCA6Bu;
    x ^= x >> 13;
    x *= 0xC2B2AE35u;
    x ^= x >> 16;
    return x;
}

// slot in [0, cap) for key x
__device__ __forceinline__ uint32_t hslot(uint32_t x, uint32_t cap)
{
    return __umulhi(mix32(x), cap);
}

// Neighbour IDs are read once per iteration: the streaming hint (evict first in L1 and
// L2) keeps them from pushing the label array, read at random, out of L2.
__device__ __forceinline__ int32_t ld_nbr(const int32_t *p) { return __ldcs(p); }

// Label gathers: the L2 evict-last policy keeps the label array (read at random, and
// again in the next iteration) resident ahead of streamed and written data.
__device__ __forceinline__ int32_t ld_label(const int32_t *p)
{
    int32_t v;
    asm("{\n\t.reg .b64 pol;\n\tcreatepolicy.fractional.L2::evict_last.b64 pol, 1.0;\n\t"
        "ld.global.nc.L2::cache_hint.b32 %0, [%1], pol;\n\t}" : "=r"(v) : "l"(p));
    return v;
}

// ----- relaxed 64-bit global accesses for the look-back status words -----
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
// Four consecutive 64-bit slots (one 32-byte sector, p 32-byte aligned), two 16-byte
// relaxed loads in flight together.
__device__ __forceinline__ void ld_relaxed_group4(const unsigned long long *p, unsigned long long x[4])
{
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(x[0]), "=l"(x[1]) : "l"(p) : "memory");
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(x[2]), "=l"(x[3]) : "l"(p + 2) : "memory");
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long *p, unsigned long long v)
{
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Status word of one tile in the decoupled look-back scan:
//   [63:62] state (1 = aggregate, 2 = inclusive prefix), [61:40] epoch, [39:0] value
constexpr int kStateShift = 62;
constexpr int kEpochShift = 40;
constexpr unsigned long long kValueMask = (1ull << 40) - 1;
constexpr unsigned long long kEpochMask = (1ull << 22) - 1;

__device__ __forceinline__ unsigned long long pack_status(unsigned state, unsigned epoch, unsigned long long value)
{
    return ((unsigned long long)state << kStateShift) | ((unsigned long long)(epoch & kEpochMask) << kEpochShift) |
           (value & kValueMask);
}

}  // namespace galp
