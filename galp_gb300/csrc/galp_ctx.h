// galp_ctx.h -- context and per-graph state behind the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/galp.h"
#include "../../include/galp_tools.h"
#include "lp_pipeline.cuh"

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

// One scope of run positions: the whole graph (policy 0) or one out-of-core batch
// (policies 1/2; batch j = vertices [v0, v1) per OutOfCore::compute_batch_boundaries,
// label_propagation/src/common/outofcore.cuh:38-60).
struct Scope {
    int64_t v0 = 0, v1 = 0;    // vertices
    int64_t e0 = 0, e1 = 0;    // CSR entries
    int32_t p0 = 0, np = 0;    // packs of small vertices
    int32_t m0 = 0, nms = 0, nml = 0, nmx = 0;  // mid (33..256), large (..2048), xl (..12288)
    int32_t b0 = 0, nb = 0;    // big vertices
    int32_t c0 = 0, nc = 0;    // big insert chunks
    int32_t s0 = 0, ns = 0;    // big stats chunks
    int32_t sv0 = 0, nsv = 0;  // vertices of degree <= 32 (small_v), in vertex order
    int32_t nnarrow = 0;       // mid-list entries of at most kNarrowMax neighbours
    int32_t last_v = -1;       // last vertex of the scope that owns runs
    int32_t q0 = 0, nq = 0;    // hash partitions of the scope's big vertices
    int64_t pair_slots = 0;    // pair area of those partitions
    int64_t occ_slots = 0;     // distinct-list capacity of the scope's big vertices
};

// Static schedule of a graph (host side, built once): degree buckets per scope.
struct Schedule {
    std::vector<int32_t> pack_v0;    // first vertex of each pack (<= 32 vertices, <= 32 edges)
    std::vector<uint8_t> pack_nv;    // vertices in each pack
    std::vector<int32_t> small_v;    // per scope: the pack vertices one by one, in vertex order
    std::vector<int32_t> mid_v;      // per scope: mid, large and xl vertices in ascending degree
    std::vector<int32_t> mid_deg;    // degree of each mid_v entry
    std::vector<int32_t> big_v;      // vertex of each big entry
    std::vector<int64_t> big_deg;    // its degree
    std::vector<int64_t> big_ooff;   // distinct-list offset, relative to its scope
    std::vector<int32_t> chunk_big;
    std::vector<int64_t> chunk_e0, chunk_e1;
    std::vector<int32_t> schunk_big;
    std::vector<int64_t> schunk_s0, schunk_s1;
    // hash partitions of the big vertices' (label, count) pairs (plan_hub_parts)
    std::vector<int32_t> hub_p0;     // first partition of each big vertex, then the total
    std::vector<int64_t> hub_pbase;  // pair-area offset of its partitions, relative to its scope
    std::vector<int32_t> hub_pcap;   // pair capacity of each of its partitions
    std::vector<int32_t> part_big;   // big vertex of each partition
    int hub_shift = 0;               // partitions per hub: degree * 2^hub_shift / kHubPartPairs
    std::vector<Scope> scopes;
    int64_t max_pair_slots = 0, max_occ_slots = 0, max_scope_edges = 0, m_big = 0;
    int64_t max_scope_small = 0, max_scope_mid = 0, max_scope_vertices = 0;
    double deg_hist[kDegBins] = {};  // CSR entries by log2 degree (dispatch features)
};

// Build the schedule; scope_starts = first vertex of every scope, then n.  False when
// the offsets decrease somewhere.
bool build_schedule(Schedule &S, int64_t n, const int64_t *off, const std::vector<int64_t> &scope_starts);

// (Re)plan the hash partitions of every big vertex: degree * 2^shift / kHubPartPairs
// partitions (at least one), each holding 1.5x its share of the degree, plus 256 pairs,
// plus one pair per insert chunk of the vertex (at most the degree).
void plan_hub_parts(Schedule &S, int shift);

// Batch boundaries of OutOfCore::compute_batch_boundaries (outofcore.cuh:38-60) for
// 2^buffer_pow edges; returns GALP_EBATCH where the reference would loop forever.
int batch_boundaries(int64_t n, const int64_t *off, int buffer_pow, std::vector<int64_t> &bbs);

// CUDA events around kernel groups (level 1) and around every kernel (level 2), enabled
// by galp_profile.  Intervals are folded into per-group and per-kernel-name totals.
struct Profiler {
    bool on = false;  // level >= 1
    int level = 0;
    std::vector<cudaEvent_t> pool;
    size_t used = 0;
    // 0 = count/scan/resolve, 1 = big pre, 2 = big post, 3 = first-iteration shortcut
    std::vector<std::pair<int, int>> spans[4];
    int last = -1;                              // level 2: mark that the next interval starts at
    std::vector<std::pair<const char *, std::pair<int, int>>> kspans;
    double group_ms[4] = {0, 0, 0, 0};
    int group_n[4] = {0, 0, 0, 0};
    std::vector<std::pair<const char *, std::pair<double, int64_t>>> kstats;  // name -> (ms, launches)
    std::vector<std::pair<int, int>> it_spans;  // in-core iterations
    std::vector<float> it_ms;
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
    void kstart(cudaStream_t st)
    {
        if (level >= 2) last = mark(st);
    }
    // level 2: close the interval since the previous mark under `name`
    void kmark(const char *name, cudaStream_t st)
    {
        if (level < 2) return;
        const int e = mark(st);
        if (last >= 0 && e >= 0) kspans.push_back({name, {last, e}});
        last = e;
    }
    // wait for the recorded events and fold their intervals into the totals
    void fold()
    {
        for (int g = 0; g < 4; ++g) {
            for (auto &sp : spans[g]) {
                float t = 0.f;
                if (sp.first >= 0 && sp.second >= 0 &&
                    cudaEventSynchronize(pool[sp.second]) == cudaSuccess &&
                    cudaEventElapsedTime(&t, pool[sp.first], pool[sp.second]) == cudaSuccess)
                    group_ms[g] += t;
                ++group_n[g];
            }
            spans[g].clear();
        }
        for (auto &ks : kspans) {
            float t = 0.f;
            if (cudaEventSynchronize(pool[ks.second.second]) != cudaSuccess ||
                cudaEventElapsedTime(&t, pool[ks.second.first], pool[ks.second.second]) != cudaSuccess)
                t = 0.f;
            size_t i = 0;
            while (i < kstats.size() && std::strcmp(kstats[i].first, ks.first) != 0) ++i;
            if (i == kstats.size()) kstats.push_back({ks.first, {0.0, 0}});
            kstats[i].second.first += t;
            kstats[i].second.second += 1;
        }
        kspans.clear();
        for (auto &sp : it_spans) {
            float t = 0.f;
            if (sp.first < 0 || sp.second < 0 || cudaEventSynchronize(pool[sp.second]) != cudaSuccess ||
                cudaEventElapsedTime(&t, pool[sp.first], pool[sp.second]) != cudaSuccess)
                t = -1.f;
            it_ms.push_back(t);
        }
        it_spans.clear();
        used = 0;
        last = -1;
    }
    ~Profiler()
    {
        for (auto e : pool) cudaEventDestroy(e);
    }
};

// Device state of a graph: resident CSR (policy 0) or streamed neighbours (policies 1/2).
struct Engine {
    int64_t n = 0, m = 0;
    int policy = 0;
    const int32_t *h_nbr = nullptr;  // caller's host neighbours (streamed for policies 1/2)
    bool registered = false;         // the library pinned h_nbr
    Schedule sched;
    DevBuf b_nbr[2], b_off, b_pack_v0, b_pack_nv, b_small_v, b_mid_v, b_big_v;
    DevBuf b_chunk_big, b_chunk_e0, b_chunk_e1, b_schunk_big, b_schunk_s0, b_schunk_s1, b_big_ooff;
    DevBuf b_hub_p0, b_hub_pbase, b_hub_pcap, b_part_big, b_pfill, b_psum, b_pairs, b_big_list;
    DevBuf b_lab0, b_lab1, b_ctl, b_bstat, b_big_a, b_bad;
    DevBuf b_dcnt, b_runbase, b_c0, b_c1, b_kw, b_r, b_run_lab, b_run_cnt, b_tsmall, b_tmid, b_bsum;
    DevBuf b_dirty, b_changed, b_chk;  // frontier mode; setup adjacency checks
    DevBuf b_static_feat, b_vtab, b_disp, b_feat_log, b_var_log, b_weights;  // dispatch
    float static_feat[kDegBins + 3] = {};
    std::vector<DispatchState> vtab;   // variant table of the in-core scope
    int disp_mode = 0;                 // 0 fixed rule, 1 learned MLP, 2 forced variant
    int disp_forced = 0;
    bool have_weights = false;
    bool frontier = false;             // requested, policy 0, and the graph is symmetric
    int32_t *d_pack_v0 = nullptr;
    uint8_t *d_pack_nv = nullptr;
    int32_t *d_small_v = nullptr;
    int32_t *d_mid_v = nullptr;
    int32_t *d_big_v = nullptr;
    int64_t *d_big_ooff = nullptr;
    int32_t *d_chunk_big = nullptr;
    int64_t *d_chunk_e0 = nullptr, *d_chunk_e1 = nullptr;
    int32_t *d_schunk_big = nullptr;
    int64_t *d_schunk_s0 = nullptr, *d_schunk_s1 = nullptr;
    int32_t *d_hub_p0 = nullptr, *d_hub_pcap = nullptr, *d_part_big = nullptr;
    int64_t *d_hub_pbase = nullptr;
    int sms = 1;
    bool adj_sorted = false;  // every adjacency list strictly increasing (first-iteration shortcut)
    bool symmetric = false;   // edge multiset symmetric (frontier marking along out-edges)
    Profiler prof;
    galp_variant variant{0, 0.05f, 0.03f, 2, 1, 0, 1, 0};  // kernel variant knobs (galp_set_variant)
    // out-of-core streaming
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_copied[2] = {nullptr, nullptr}, ev_consumed[2] = {nullptr, nullptr};
    uint64_t batch_seq = 0;   // running batch counter (buffer parity)
    int64_t h2d_run = 0;      // bytes streamed by the last run
    int64_t launches = 0;     // kernels launched by runs so far (setup excluded)
    int hub_count_blocks = 0; // resident blocks of hub_count_kernel (grid = one wave)
    int hub_count_blocks_half = 0, hub_count_blocks_quarter = 0;  // the same for its smaller shapes
    double setup_ms[5] = {};  // host schedule, CSR upload, state upload, dispatch prep, device checks
    // batched mode: graph g = vertices [g_v0[g], g_v0[g+1]) of the concatenated CSR
    bool batched = false;
    int32_t G = 0;
    int early_exit = 1;
    int batch_max_iter = 0;   // row length of b_g_counts
    std::vector<int64_t> g_v0_h;
    std::vector<int32_t> g_last_h;
    DevBuf b_g_v0, b_g_base, b_g_last, b_g_active, b_g_iters, b_g_counts, b_gid;
    int64_t max_label = 0;    // labels stay below this (n, or the largest graph of a batch)
    // launch shapes (blocks per SM), chosen by galp_batch_tune
    int small_bps = 16, mid_bps = 6, resolve_bps = 4;
    // resident blocks per SM of the mid-vertex counting and the resolve kernels (occupancy
    // API): their grid-stride loops run as one full wave, since a partial second wave
    // would start its blocks' whole shares late
    int occ_mid = 0, occ_mid_sort = 0, occ_resolve = 0, occ_resolve_mid = 0;
    int occ_cta64 = 0, occ_cta128 = 0, occ_cta256 = 0;  // resident CTA-kernel blocks per SM
    int launch_limits();
    // hub partitions at 2^shift times the default count: plan, upload, size the pair area
    int setup_hub_parts(int shift, cudaStream_t st, int64_t &h2d);
    int setup_batch(const galp_csr &g, const int64_t *graph_v0, int32_t count, const galp_opts &o, cudaStream_t st,
                    int64_t &h2d);
    void launched(const char *name, cudaStream_t st)
    {
        ++launches;
        prof.kmark(name, st);
    }

    ~Engine();
    int setup(const galp_csr &g, const galp_opts &o, cudaStream_t st, int64_t &h2d);
    IterArgs big_args(const Scope &sc) const;
    PipeArgs pipe_args(const Scope &sc) const;
    void build_variant_table();
    std::vector<DispatchState> static_dispatch() const;
    DispatchArgs dispatch_args(int it) const;
    int enqueue_scope(cudaStream_t st, const Scope &sc, const int32_t *nbr, const int32_t *lab_in,
                      int32_t *lab_out, const uint8_t *dirty = nullptr, int32_t *changed = nullptr);
    int enqueue_run_incore(cudaStream_t st, int niter, long long thr);
    int run_outofcore(cudaStream_t st, int niter, long long thr);
    int enqueue_init(cudaStream_t st, int niter, long long thr);
    const int32_t *final_labels(int iters) const;
};

}  // namespace galp

struct galp_ctx {
    galp_opts opts{};
    // batched mode: the whole run captured once per iteration count as a CUDA graph
    cudaGraphExec_t graph_exec = nullptr;
    int graph_iters = -1;
    int last_niter = 0;      // iterations of the last enqueued run (redone after a hub overflow)
    int64_t n = 0, m = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    galp::Engine eng;
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
