// galp_tools.cu -- device-side R-MAT edge sampling for building large benchmark graphs.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "../../include/galp_tools.h"
#include "rmat_rng.h"

namespace {

__global__ void rmat_keys_kernel(uint64_t seed, int scale, int64_t ne, uint32_t ta, uint32_t tb, uint32_t tc,
                                 uint64_t *out)
{
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x)
        out[e] = galp::rmat_edge_key(seed, (uint64_t)e, scale, ta, tb, tc);
}

}  // namespace

extern "C" int galp_gen_rmat_keys_device(uint64_t seed, int32_t scale, int64_t nedges, double a, double b, double c,
                                         void *d_out, void *stream)
{
    if (scale <= 0 || scale > 31 || nedges < 0 || (!d_out && nedges > 0)) return GALP_EINVAL;
    if (nedges == 0) return GALP_OK;
    const uint32_t ta = (uint32_t)std::llround(a * 4294967296.0);
    const uint32_t tb = (uint32_t)std::llround((a + b) * 4294967296.0);
    const uint32_t tc = (uint32_t)std::llround((a + b + c) * 4294967296.0);
    rmat_keys_kernel<<<4096, 256, 0, (cudaStream_t)stream>>>(seed, scale, nedges, ta, tb, tc, (uint64_t *)d_out);
    return cudaGetLastError() == cudaSuccess ? GALP_OK : GALP_ECUDA;
}
