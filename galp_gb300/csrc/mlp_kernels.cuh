// mlp_kernels.cuh -- batched FP32 training kernels of the dispatcher's MLP (forward,
// masked MSE gradient, backward, AdamW), used by galp_mlp.cu only.
#pragma once

#include <cstdint>

#include "mlp_layout.h"

namespace galp {

// ---------------------------------------------------------------------------
// batched MLP training kernels (FP32)
// ---------------------------------------------------------------------------

// Y[b][o] = act(bias[o] + sum_i X[b][i] W[i][o]); one thread per output.
__global__ void mlp_linear_fwd(const float *X, const float *W, const float *bias, float *Y, int B, int I, int O,
                               int relu)
{
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)B * O) return;
    const int b = (int)(idx / O), o = (int)(idx % O);
    float s = bias[o];
    for (int i = 0; i < I; ++i) s += X[(int64_t)b * I + i] * W[(int64_t)i * O + o];
    Y[idx] = relu ? fmaxf(s, 0.f) : s;
}

// Masked mean squared error: dP = 2 mask (P - T) / count; loss accumulated in *loss.
__global__ void mlp_mse_grad(const float *P, const float *T, const float *M, float *dP, int64_t total, float inv_count,
                             float *loss)
{
    float acc = 0.f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const float d = (P[i] - T[i]) * M[i];
        dP[i] = 2.f * d * inv_count;
        acc += d * d * inv_count;
    }
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xFFFFFFFFu, acc, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc);
}

// dZ = dY * (Y > 0) in place when relu (Y is the layer's activated output).
__global__ void mlp_relu_bwd(float *dY, const float *Y, int64_t total)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
        if (Y[i] <= 0.f) dY[i] = 0.f;
}

// dW[i][o] = sum_b X[b][i] dZ[b][o]; db[o] = sum_b dZ[b][o] (thread per (i, o), plus I..I
// rows for the bias).
__global__ void mlp_linear_wgrad(const float *X, const float *dZ, float *dW, float *db, int B, int I, int O)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (I + 1) * O) return;
    const int i = idx / O, o = idx % O;
    float s = 0.f;
    if (i < I) {
        for (int b = 0; b < B; ++b) s += X[(int64_t)b * I + i] * dZ[(int64_t)b * O + o];
        dW[(int64_t)i * O + o] = s;
    } else {
        for (int b = 0; b < B; ++b) s += dZ[(int64_t)b * O + o];
        db[o] = s;
    }
}

// dX[b][i] = sum_o dZ[b][o] W[i][o].
__global__ void mlp_linear_xgrad(const float *dZ, const float *W, float *dX, int B, int I, int O)
{
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)B * I) return;
    const int b = (int)(idx / I), i = (int)(idx % I);
    float s = 0.f;
    for (int o = 0; o < O; ++o) s += dZ[(int64_t)b * O + o] * W[(int64_t)i * O + o];
    dX[idx] = s;
}

// Adam with decoupled weight decay (AdamW), bias-corrected.
__global__ void mlp_adam(float *w, const float *g, float *m1, float *m2, int64_t count, float lr, float b1, float b2,
                         float eps, float wd, float c1, float c2)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float a = m1[i] = b1 * m1[i] + (1.f - b1) * gi;
        const float v = m2[i] = b2 * m2[i] + (1.f - b2) * gi * gi;
        w[i] -= lr * ((a / c1) / (sqrtf(v / c2) + eps) + wd * w[i]);
    }
}

}  // namespace galp
