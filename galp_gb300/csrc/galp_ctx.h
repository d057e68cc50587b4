// galp_ctx.h -- context and per-graph state behind the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "../../include/galp.h"
#include "lp_kernels.cuh"

namespace galp {

int cuda_status(cudaError_t e);

// Owning device allocation.
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    cudaError_t alloc(size_t b)
    {
        release();
        cudaError_t e = cudaMalloc(&p, b);
        if (e != cudaSuccess) {
            p = nullptr;
            return e;
        }
        bytes = b;
        return cudaSuccess;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
};

struct Schedule {
    std::vector<uint16_t> vpos;
    std::vector<int32_t> tile_v0;
    std::vector<int32_t> tile_big;
    std::vector<uint16_t> tile_used;
    std::vector<int32_t> big_v;
    std::vector<int64_t> big_toff;
    std::vector<uint32_t> big_tcap;
    std::vector<int32_t> chunk_big;
    std::vector<int64_t> chunk_e0, chunk_e1;
    std::vector<int32_t> schunk_big;
    std::vector<int64_t> schunk_s0, schunk_s1;
    int64_t table_slots = 0;
    int32_t last_v = -1;
};

void build_schedule(Schedule &S, int64_t n, const int64_t *off);

// CUDA events around kernel groups (enabled by galp_profile).
struct Profiler {
    bool on = false;
    std::vector<cudaEvent_t> pool;
    size_t used = 0;
    std::vector<std::pair<int, int>> spans[3];  // 0 = tile kernel, 1 = big pre, 2 = big post
    int mark(cudaStream_t st)
    {
        if (used == pool.size()) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return -1;
            pool.push_back(e);
        }
        cudaEventRecord(pool[used], st);
        return (int)used++;
    }
    ~Profiler()
    {
        for (auto e : pool) cudaEventDestroy(e);
    }
};

// Device state of one resident scope (the whole graph for policy 0).
struct InCore {
    int64_t n = 0, m = 0;
    Schedule sched;
    DevBuf b_nbr, b_off, b_vpos, b_tile_v0, b_tile_big, b_tile_used, b_big_v, b_big_toff, b_big_tcap;
    DevBuf b_chunk_big, b_chunk_e0, b_chunk_e1, b_schunk_big, b_schunk_s0, b_schunk_s1;
    DevBuf b_lab0, b_lab1, b_status, b_ctl, b_bstat, b_big_a, b_gkey, b_gcnt, b_bad;
    uint16_t *d_vpos = nullptr;
    int32_t *d_tile_v0 = nullptr, *d_tile_big = nullptr;
    uint16_t *d_tile_used = nullptr;
    int32_t *d_big_v = nullptr;
    int64_t *d_big_toff = nullptr;
    uint32_t *d_big_tcap = nullptr;
    int32_t *d_chunk_big = nullptr;
    int64_t *d_chunk_e0 = nullptr, *d_chunk_e1 = nullptr;
    int32_t *d_schunk_big = nullptr;
    int64_t *d_schunk_s0 = nullptr, *d_schunk_s1 = nullptr;
    unsigned epoch = 0;
    int tile_grid = 1;
    int64_t m_big = 0;
    Profiler prof;

    int setup(const galp_csr &g, cudaStream_t st, int64_t &h2d);
    IterArgs args() const;
    int enqueue_iteration(cudaStream_t st, const int32_t *lab_in, int32_t *lab_out);
    int enqueue_run(cudaStream_t st, int niter, long long thr);
};

}  // namespace galp

struct galp_ctx {
    galp_opts opts{};
    int64_t n = 0, m = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    galp::InCore incore;
    double t_pre = 0;
    int64_t h2d_setup = 0;
    bool pending = false;
    bool have_labels = false;
    int iters = 0;
    int err = 0;
    int64_t runs_last = 0;
    float device_ms = 0;
    int64_t counts[GALP_MAX_ITERS] = {};
    std::vector<int32_t> labels;
};
