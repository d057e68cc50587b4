// lp_dispatch.cuh -- per-iteration kernel-variant dispatch (MLP inference on the device).
//
// Every iteration of the in-core update reads a DispatchState from device memory: how
// mid-list vertices are split between the warp kernel and the two CTA kernels (degree
// thresholds, as positions in the degree-sorted mid list), whether CTA-table inserts are
// warp-aggregated, and whether the frontier is used.  Every variant computes the same
// labels; they differ only in speed.  dispatch_kernel fills the state on the device
// before each iteration, so no host round trip is needed:
//   * fixed rule: CTA thresholds 256 / 2048, plain inserts, frontier when at most
//     frontier_frac of the labels changed in the previous iteration;
//   * learned: a 3-layer MLP (kFeat -> kHid -> kHid -> kVar, ReLU, FP32) predicts the
//     log slowdown of every variant from the iteration's features; the argmin wins when
//     it is predicted to beat the fixed rule's row by more than a margin (the fixed rule
//     is the fallback and the reference point);
//   * forced: one variant for every iteration (timing sweeps that train the MLP).
// The features of every iteration are logged for those sweeps.
#pragma once

#include <cstdint>

#include "lp_kernels.cuh"
#include "mlp_layout.h"

namespace galp {

constexpr int kFeat = 24;  // features per iteration
constexpr int kHid = 64;   // hidden width
constexpr int kVar = 16;   // variants
constexpr int kDegBins = 16;
constexpr int kMaxLogIters = 64;


struct DispatchState {
    int32_t agg_mode;  // CTA-table inserts: 0 auto, 1 warp-aggregated, 2 plain
    int32_t frontier;  // 1 = skip clean vertices this iteration (frontier mode only)
    // cuts of the degree-sorted mid list: [0, pos1) one warp each; [pos1, pos_a) 128-thread
    // CTAs (degree <= 1024); [pos_a, pos2) 256-thread CTAs; [pos2, pos_b) 512-thread CTAs
    // (degree <= 6144); [pos_b, end) 1024-thread CTAs
    int32_t pos1, pos2, pos_a, pos_b;
    int32_t variant;   // row of the variant table
    int32_t pad;
};

struct DispatchArgs {
    const Ctl *ctl;
    const DispatchState *table;  // kVar rows for this graph
    const float *weights;        // MLP parameters (learned mode)
    const float *static_feat;    // features [0, kDegBins + 3) of the graph
    DispatchState *out;
    float *feat_log;             // [kMaxLogIters][kFeat] or null
    int32_t *var_log;            // [kMaxLogIters] or null
    int64_t n, m;
    int32_t it;                  // iteration about to run (0-based)
    int32_t mode;                // 0 fixed rule, 1 learned, 2 forced
    int32_t forced;              // forced variant
    int32_t frontier_mode;       // the engine keeps frontier state
    float frontier_frac;         // fixed rule: frontier when changed <= frac * n
    int32_t fixed_variant_dense; // fixed rule rows (dense / frontier)
    int32_t fixed_variant_front;
    int32_t fixed_agg;           // fixed rule: CTA-table insert mode
    float margin;                // learned: predicted log gain needed to leave the fixed rule's row
};

// Feature vector of an iteration: edge-weighted log2-degree histogram (kDegBins), log2 m
// / 40, log2 n / 40, log2 mean degree / 16, fraction of labels changed in the previous
// iteration, distinct labels per CSR entry in the previous iteration (runs / m),
// iteration / 16, frontier mode, constant 1, padding.
__device__ __forceinline__ void dispatch_features(const DispatchArgs &a, float *f)
{
    for (int i = 0; i < kDegBins + 3; ++i) f[i] = a.static_feat[i];
    float chg = 1.f, dist = 1.f;
    if (a.it > 0) {
        chg = (float)((double)a.ctl->counts[a.it - 1] / (double)(a.n > 0 ? a.n : 1));
        dist = (float)((double)a.ctl->N / (double)(a.m > 0 ? a.m : 1));
    }
    f[kDegBins + 3] = chg;
    f[kDegBins + 4] = dist;
    f[kDegBins + 5] = (float)a.it / 16.f;
    f[kDegBins + 6] = a.frontier_mode ? 1.f : 0.f;
    f[kDegBins + 7] = 1.f;
    for (int i = kDegBins + 8; i < kFeat; ++i) f[i] = 0.f;
}

// One block of kHid threads.
__global__ void __launch_bounds__(kHid) dispatch_kernel(DispatchArgs a)
{
    __shared__ float x[kFeat], h1[kHid], h2[kHid], y[kVar];
    __shared__ int pick;
    const int t = threadIdx.x;
    if (t == 0) {
        dispatch_features(a, x);
        int v;
        if (a.mode == 2) {
            v = a.forced;
        } else {
            const bool front = a.frontier_mode && x[kDegBins + 3] <= a.frontier_frac;
            v = front ? a.fixed_variant_front : a.fixed_variant_dense;
        }
        pick = v;
    }
    __syncthreads();
    if (a.mode == 1) {
        const float *W1 = a.weights, *b1 = W1 + kFeat * kHid, *W2 = b1 + kHid, *b2 = W2 + kHid * kHid;
        const float *W3 = b2 + kHid, *b3 = W3 + kHid * kVar;
        float s = b1[t];
        for (int i = 0; i < kFeat; ++i) s += x[i] * W1[i * kHid + t];
        h1[t] = fmaxf(s, 0.f);
        __syncthreads();
        s = b2[t];
        for (int i = 0; i < kHid; ++i) s += h1[i] * W2[i * kHid + t];
        h2[t] = fmaxf(s, 0.f);
        __syncthreads();
        if (t < kVar) {
            s = b3[t];
            for (int i = 0; i < kHid; ++i) s += h2[i] * W3[i * kVar + t];
            y[t] = s;
        }
        __syncthreads();
        if (t == 0) {
            // the fixed rule's row stays unless the network predicts a clear gain
            int best = 0;
            for (int k = 1; k < kVar; ++k)
                if (y[k] < y[best]) best = k;
            if (y[pick] - y[best] > a.margin) pick = best;
        }
        __syncthreads();
    }
    if (t == 0) {
        DispatchState d = a.table[pick];
        if (a.mode == 0) d.agg_mode = a.fixed_agg;
        if (!a.frontier_mode) d.frontier = 0;
        *a.out = d;
        if (a.it < kMaxLogIters) {
            if (a.feat_log)
                for (int i = 0; i < kFeat; ++i) a.feat_log[a.it * kFeat + i] = x[i];
            if (a.var_log) a.var_log[a.it] = pick;
        }
    }
}

}  // namespace galp
