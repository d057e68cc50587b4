// galp_capi.cu -- host side of the C ABI (include/galp.h): context, schedule, launches.
//
// In-core (policy 0) keeps the whole CSR resident in HBM: neighbours int32[m],
// offsets int64[n+1] (no int32 truncation, unlike src/common/incore.cuh:63-69), two
// label buffers, per-vertex count/scan state, a spill area for tied vertices' runs,
// and a static degree-bucketed schedule built once per graph (packs of small
// vertices, mid/large vertex lists, big vertices with open-addressed global tables).
// Out-of-core (policies 1/2) keeps everything but the neighbours resident and streams
// the neighbours of one batch at a time.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <thread>
#include <vector>

#include "../../include/galp.h"
#include "lp_kernels.cuh"
#include "galp_ctx.h"
#include "dispatch_weights.inc"
#include "../../include/galp_tools.h"

using namespace galp;

namespace {

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

namespace galp {

int cuda_status(cudaError_t e)
{
    if (e == cudaSuccess) return GALP_OK;
    if (e == cudaErrorMemoryAllocation) return GALP_ENOMEM;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return GALP_ENODEV;
    return GALP_ECUDA;
}

#define GALP_CUDA(call)                                    \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return cuda_status(e_);     \
    } while (0)

namespace {

// One thread's share of a scope: packs, mid-list vertices (unsorted), big vertices.
struct ChunkPlan {
    std::vector<int32_t> pack_v0;
    std::vector<uint8_t> pack_nv;
    std::vector<int32_t> mid;
    std::vector<int32_t> mid_deg;    // degree of each mid entry
    std::vector<int64_t> mid_count;  // mid entries by degree (up to the largest), then positions
    std::vector<int32_t> big;
    int64_t nsmall = 0;
    int32_t last_v = -1;
    bool bad = false;       // offsets decrease somewhere
    double hist[kDegBins] = {};
};

void plan_chunk(const int64_t *off, int64_t v0, int64_t v1, ChunkPlan &P)
{
    int pv = 0, pe = 0;  // vertices / edges in the open pack
    int64_t pstart = -1;
    auto close = [&]() {
        if (pv) {
            P.pack_v0.push_back((int32_t)pstart);
            P.pack_nv.push_back((uint8_t)pv);
        }
        pv = pe = 0;
    };
    for (int64_t v = v0; v < v1; ++v) {
        const int64_t deg = off[v + 1] - off[v];
        if (deg < 0) {
            P.bad = true;
            return;
        }
        if (deg > 0) {
            P.last_v = (int32_t)v;
            P.hist[std::min(kDegBins - 1, 63 - __builtin_clzll((unsigned long long)deg))] += (double)deg;
        }
        if (deg <= kSmallMax) {
            if (pv == 32 || pe + deg > 32) close();
            if (!pv) pstart = v;
            pv++;
            pe += (int)deg;
            P.nsmall++;
            continue;
        }
        close();
        if (deg <= kXlMax) {
            P.mid.push_back((int32_t)v);
            P.mid_deg.push_back((int32_t)deg);
            if ((size_t)deg >= P.mid_count.size()) P.mid_count.resize((size_t)deg + 1, 0);
            ++P.mid_count[(size_t)deg];
        } else {
            P.big.push_back((int32_t)v);
        }
    }
    close();
}

}  // namespace

constexpr int kMaxHubShift = 6;  // at most 64x the default hub partitions

// Hash partitions of the big vertices: a hub of degree D gets ceil(D * 2^shift / 8192)
// partitions (its chunks emit at most D pairs, about 8192 per partition while labels are
// still mostly distinct).  A partition holds 1.5x its share plus 256 pairs, plus one pair
// per insert chunk of the hub: a label that appears in every chunk (late iterations) sends
// all its pairs to one partition.  Partition indices are global; pair areas are relative
// to the scope (out-of-core batches reuse one area).
void plan_hub_parts(Schedule &S, int shift)
{
    const size_t nb = S.big_v.size();
    S.hub_shift = shift;
    S.hub_p0.assign(nb + 1, 0);
    S.hub_pbase.assign(nb, 0);
    S.hub_pcap.assign(nb, 0);
    S.part_big.clear();
    S.max_pair_slots = 0;
    for (Scope &sc : S.scopes) {
        sc.q0 = (int32_t)S.part_big.size();
        int64_t pbase = 0;
        for (int32_t b = sc.b0; b < sc.b0 + sc.nb; ++b) {
            const int64_t deg = S.big_deg[(size_t)b];
            const double scaled = std::ldexp((double)deg, shift) / kHubPartPairs;
            const int64_t np = std::max<int64_t>(
                1, std::min<int64_t>(std::min<int64_t>((int64_t)std::ceil(scaled), deg), kHubMaxParts));
            const int64_t nchunks = (deg + kBigChunk - 1) / kBigChunk;
            const int64_t cap = std::min<int64_t>(deg, (3 * deg + 2 * np - 1) / (2 * np) + 256 + nchunks);
            S.hub_p0[(size_t)b] = (int32_t)S.part_big.size();
            S.hub_pbase[(size_t)b] = pbase;
            S.hub_pcap[(size_t)b] = (int32_t)cap;
            S.part_big.insert(S.part_big.end(), (size_t)np, b);
            pbase += np * cap;
        }
        sc.nq = (int32_t)S.part_big.size() - sc.q0;
        sc.pair_slots = pbase;
        S.max_pair_slots = std::max(S.max_pair_slots, pbase);
    }
    S.hub_p0[nb] = (int32_t)S.part_big.size();
}

// Static per-graph schedule (host), per scope: packs of consecutive vertices of degree
// <= 32 (at most 32 vertices and 32 edges; a pack ends at a vertex of another bucket or
// at a thread's chunk boundary), the mid list (33..12288) in ascending degree, and big
// vertices (> 12288) with global hash tables (offsets relative to the scope, so
// out-of-core batches reuse one table area) and their work chunks.  Vertex ranges are
// planned by several host threads.  Returns false when the offsets decrease.
bool build_schedule(Schedule &S, int64_t n, const int64_t *off, const std::vector<int64_t> &scope_starts)
{
    S = Schedule();
    const int hw = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    for (size_t k = 0; k + 1 < scope_starts.size(); ++k) {
        Scope sc;
        sc.v0 = scope_starts[k];
        sc.v1 = scope_starts[k + 1];
        sc.e0 = off[sc.v0];
        sc.e1 = off[sc.v1];
        sc.p0 = (int32_t)S.pack_v0.size();
        sc.sv0 = (int32_t)S.small_v.size();
        sc.m0 = (int32_t)S.mid_v.size();
        sc.b0 = (int32_t)S.big_v.size();
        sc.c0 = (int32_t)S.chunk_big.size();
        sc.s0 = (int32_t)S.schunk_big.size();
        const int64_t nv = sc.v1 - sc.v0;
        const int T = nv >= (1 << 20) ? hw : 1;
        std::vector<ChunkPlan> plans(T);
        {
            std::vector<std::thread> th;
            for (int t = 0; t < T; ++t) {
                const int64_t a = sc.v0 + nv * t / T, b = sc.v0 + nv * (t + 1) / T;
                if (T == 1) plan_chunk(off, a, b, plans[t]);
                else th.emplace_back(plan_chunk, off, a, b, std::ref(plans[t]));
            }
            for (auto &x : th) x.join();
        }
        int64_t nsmall = 0;
        std::vector<int32_t> big;
        size_t np = 0, nm = 0;
        for (ChunkPlan &P : plans) {
            if (P.bad) return false;
            np += P.pack_v0.size();
            nm += P.mid.size();
            big.insert(big.end(), P.big.begin(), P.big.end());
            nsmall += P.nsmall;
            if (P.last_v >= 0) sc.last_v = P.last_v;
            for (int b = 0; b < kDegBins; ++b) S.deg_hist[b] += P.hist[b];
        }
        // The mid list in ascending degree (counting sort, stable: threads in vertex order,
        // each thread's entries in vertex order), so any degree threshold is a cut position
        // and the kernel split can change per iteration.  Each thread's bins become its
        // write positions; packs are copied to their offsets by the same threads.
        const size_t pb = S.pack_v0.size(), mb = S.mid_v.size();
        {
            size_t D = 0;
            for (const ChunkPlan &P : plans) D = std::max(D, P.mid_count.size());
            int64_t pos = (int64_t)mb, upto_mid = -1, upto_large = -1;
            for (size_t d = 0; d < D; ++d) {
                if (d == (size_t)kMidSMax + 1) upto_mid = pos - (int64_t)mb;
                if (d == (size_t)kLargeMax + 1) upto_large = pos - (int64_t)mb;
                for (ChunkPlan &P : plans) {
                    if (d >= P.mid_count.size()) continue;
                    const int64_t c = P.mid_count[d];
                    P.mid_count[d] = pos;
                    pos += c;
                }
            }
            const int64_t total = pos - (int64_t)mb;
            if (upto_mid < 0) upto_mid = total;
            if (upto_large < 0) upto_large = total;
            sc.nms = (int32_t)upto_mid;
            sc.nml = (int32_t)(upto_large - upto_mid);
            sc.nmx = (int32_t)(total - upto_large);
        }
        const size_t sb = S.small_v.size();
        S.pack_v0.resize(pb + np);
        S.pack_nv.resize(pb + np);
        S.small_v.resize(sb + (size_t)nsmall);
        S.mid_v.resize(mb + nm);
        S.mid_deg.resize(mb + nm);
        {
            auto place = [&](int t, size_t p0, size_t s0) {
                ChunkPlan &P = plans[(size_t)t];
                std::copy(P.pack_v0.begin(), P.pack_v0.end(), S.pack_v0.begin() + (ptrdiff_t)p0);
                std::copy(P.pack_nv.begin(), P.pack_nv.end(), S.pack_nv.begin() + (ptrdiff_t)p0);
                for (size_t k2 = 0; k2 < P.pack_v0.size(); ++k2)
                    for (int u = 0; u < P.pack_nv[k2]; ++u) S.small_v[s0++] = P.pack_v0[k2] + u;
                for (size_t i = 0; i < P.mid.size(); ++i) {
                    const size_t at = (size_t)P.mid_count[(size_t)P.mid_deg[i]]++;
                    S.mid_v[at] = P.mid[i];
                    S.mid_deg[at] = P.mid_deg[i];
                }
            };
            std::vector<std::thread> th;
            size_t p0 = pb, s0 = sb;
            for (int t = 0; t < T; ++t) {
                if (T == 1) place(t, p0, s0);
                else th.emplace_back(place, t, p0, s0);
                p0 += plans[(size_t)t].pack_v0.size();
                s0 += (size_t)plans[(size_t)t].nsmall;
            }
            for (auto &x : th) x.join();
        }
        sc.nnarrow = (int32_t)(std::upper_bound(S.mid_deg.begin() + (ptrdiff_t)mb, S.mid_deg.end(), kNarrowMax) -
                               (S.mid_deg.begin() + (ptrdiff_t)mb));
        int64_t ooff = 0;
        for (int32_t v : big) {
            const int64_t deg = off[v + 1] - off[v];
            const int32_t b = (int32_t)S.big_v.size();
            S.big_v.push_back(v);
            S.big_deg.push_back(deg);
            S.big_ooff.push_back(ooff);
            for (int64_t e = off[v]; e < off[v + 1]; e += kBigChunk) {
                S.chunk_big.push_back(b);
                S.chunk_e0.push_back(e);
                S.chunk_e1.push_back(std::min<int64_t>(e + kBigChunk, off[v + 1]));
            }
            for (int64_t i = 0; i < deg; i += kBigSlotChunk) {  // over the distinct list
                S.schunk_big.push_back(b);
                S.schunk_s0.push_back(i);
                S.schunk_s1.push_back(std::min<int64_t>(i + kBigSlotChunk, deg));
            }
            ooff += deg;
            S.m_big += deg;
        }
        sc.np = (int32_t)S.pack_v0.size() - sc.p0;
        sc.nsv = (int32_t)S.small_v.size() - sc.sv0;
        sc.nb = (int32_t)S.big_v.size() - sc.b0;
        sc.nc = (int32_t)S.chunk_big.size() - sc.c0;
        sc.ns = (int32_t)S.schunk_big.size() - sc.s0;
        sc.occ_slots = ooff;
        S.max_occ_slots = std::max(S.max_occ_slots, ooff);
        S.max_scope_edges = std::max(S.max_scope_edges, sc.e1 - sc.e0);
        S.max_scope_small = std::max(S.max_scope_small, nsmall);
        S.max_scope_mid = std::max<int64_t>(S.max_scope_mid, (int64_t)sc.nms + sc.nml + sc.nmx);
        S.max_scope_vertices = std::max(S.max_scope_vertices, sc.v1 - sc.v0);
        S.scopes.push_back(sc);
    }
    plan_hub_parts(S, 0);
    return true;
}

int batch_boundaries(int64_t n, const int64_t *off, int buffer_pow, std::vector<int64_t> &bbs)
{
    const int64_t B = (int64_t)1 << buffer_pow;
    const int64_t m = off[n];
    bbs.assign(1, 0);
    int64_t batch_offset = B;
    while (batch_offset < m) {
        int64_t left = 0, right = n + 1;
        while (left < right) {
            const int64_t mid = (left + right) / 2;
            if (off[mid] < batch_offset) left = mid + 1; else right = mid;
        }
        if (left - 1 <= bbs.back()) return GALP_EBATCH;  // a vertex of degree >= 2^buffer_pow
        bbs.push_back(left - 1);
        batch_offset = off[left - 1] + B;
    }
    bbs.push_back(n);
    return GALP_OK;
}

template <class T>
int upload(DevBuf &owner, T *&dst, const std::vector<T> &src, cudaStream_t st, int64_t &h2d)
{
    const size_t bytes = sizeof(T) * std::max<size_t>(src.size(), 1);
    GALP_CUDA(owner.alloc(bytes));
    dst = (T *)owner.p;
    if (!src.empty()) {
        GALP_CUDA(cudaMemcpyAsync(dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice, st));
        h2d += (int64_t)(sizeof(T) * src.size());
    }
    return GALP_OK;
}

Engine::~Engine()
{
    if (copy_stream) cudaStreamSynchronize(copy_stream);
    for (int i = 0; i < 2; ++i) {
        if (ev_copied[i]) cudaEventDestroy(ev_copied[i]);
        if (ev_consumed[i]) cudaEventDestroy(ev_consumed[i]);
    }
    if (copy_stream) cudaStreamDestroy(copy_stream);
    if (registered) cudaHostUnregister((void *)h_nbr);
}

int Engine::setup(const galp_csr &g, const galp_opts &o, cudaStream_t st, int64_t &h2d)
{
    double tp = now_s();
    auto phase = [&](int i) {
        const double t = now_s();
        setup_ms[i] += (t - tp) * 1e3;
        tp = t;
    };
    n = g.n;
    m = g.m;
    policy = o.policy;
    {
        int dev = 0;
        GALP_CUDA(cudaGetDevice(&dev));
        GALP_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    }
    h_nbr = g.neighbors;
    frontier = o.frontier != 0 && policy == 0;  // the frontier needs the whole graph resident
    max_label = n;
    if (policy != 0 && (o.buffer_pow < 1 || o.buffer_pow > 40)) return GALP_EINVAL;
    GALP_CUDA(b_off.alloc(sizeof(int64_t) * (n + 1)));
    // 16 bytes of padding: bulk copies of a vertex's neighbours end at a 16-byte boundary
    if (policy == 0) GALP_CUDA(b_nbr[0].alloc(sizeof(int32_t) * std::max<int64_t>(m, 1) + 16));
    // the CSR upload runs while the host builds the schedule (host or device neighbours:
    // batched callers may hand over a device array)
    GALP_CUDA(cudaMemcpyAsync(b_off.p, g.offsets, sizeof(int64_t) * (n + 1), cudaMemcpyDefault, st));
    h2d += sizeof(int64_t) * (n + 1);
    if (policy == 0 && m) {
        GALP_CUDA(cudaMemcpyAsync(b_nbr[0].p, g.neighbors, sizeof(int32_t) * m, cudaMemcpyDefault, st));
        h2d += sizeof(int32_t) * m;
    }
    std::vector<int64_t> starts;
    int brc = GALP_OK;
    if (policy == 0) starts = {0, n};
    else brc = batch_boundaries(n, g.offsets, o.buffer_pow, starts);
    const bool sched_ok = brc == GALP_OK && build_schedule(sched, n, g.offsets, starts);
    if (!sched_ok) {
        GALP_CUDA(cudaStreamSynchronize(st));  // the copies read the caller's buffers
        return brc != GALP_OK ? brc : GALP_EFORMAT;
    }
    phase(0);

    if (policy != 0) {
        const size_t cap = sizeof(int32_t) * std::max<int64_t>(sched.max_scope_edges, 1) + 16;
        GALP_CUDA(b_nbr[0].alloc(cap));
        GALP_CUDA(b_nbr[1].alloc(cap));
        // pin the caller's neighbours for asynchronous copies (graph.h:108-111 pins them too)
        if (m) {
            cudaError_t e = cudaHostRegister((void *)g.neighbors, sizeof(int32_t) * m, cudaHostRegisterPortable);
            if (e == cudaSuccess) registered = true;
            else (void)cudaGetLastError();  // already pinned by the caller, or not pinnable: copy as is
        }
        GALP_CUDA(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking));
        for (int i = 0; i < 2; ++i) {
            GALP_CUDA(cudaEventCreateWithFlags(&ev_copied[i], cudaEventDisableTiming));
            GALP_CUDA(cudaEventCreateWithFlags(&ev_consumed[i], cudaEventDisableTiming));
        }
    }
    GALP_CUDA(cudaStreamSynchronize(st));
    phase(1);
    int rc;
    if ((rc = upload(b_pack_v0, d_pack_v0, sched.pack_v0, st, h2d))) return rc;
    if ((rc = upload(b_pack_nv, d_pack_nv, sched.pack_nv, st, h2d))) return rc;
    if ((rc = upload(b_small_v, d_small_v, sched.small_v, st, h2d))) return rc;
    if ((rc = upload(b_mid_v, d_mid_v, sched.mid_v, st, h2d))) return rc;
    if ((rc = upload(b_big_v, d_big_v, sched.big_v, st, h2d))) return rc;
    if ((rc = upload(b_big_ooff, d_big_ooff, sched.big_ooff, st, h2d))) return rc;
    if ((rc = upload(b_chunk_big, d_chunk_big, sched.chunk_big, st, h2d))) return rc;
    if ((rc = upload(b_chunk_e0, d_chunk_e0, sched.chunk_e0, st, h2d))) return rc;
    if ((rc = upload(b_chunk_e1, d_chunk_e1, sched.chunk_e1, st, h2d))) return rc;
    if ((rc = upload(b_schunk_big, d_schunk_big, sched.schunk_big, st, h2d))) return rc;
    if ((rc = upload(b_schunk_s0, d_schunk_s0, sched.schunk_s0, st, h2d))) return rc;
    if ((rc = upload(b_schunk_s1, d_schunk_s1, sched.schunk_s1, st, h2d))) return rc;
    if ((rc = setup_hub_parts(variant.hub_part_shift, st, h2d))) return rc;
    // per-vertex state, spill and tied lists
    const size_t nn = (size_t)std::max<int64_t>(n, 1);
    GALP_CUDA(b_dcnt.alloc(sizeof(int32_t) * nn));
    GALP_CUDA(b_runbase.alloc(sizeof(int64_t) * nn));
    GALP_CUDA(b_c0.alloc(sizeof(int32_t) * nn));
    GALP_CUDA(b_c1.alloc(sizeof(int32_t) * nn));
    GALP_CUDA(b_kw.alloc(sizeof(int32_t) * nn));
    GALP_CUDA(b_r.alloc(sizeof(int32_t) * nn));
    const size_t ms = (size_t)std::max<int64_t>(sched.max_scope_edges, 1);
    GALP_CUDA(b_run_lab.alloc(sizeof(int32_t) * ms));
    GALP_CUDA(b_run_cnt.alloc(sizeof(uint16_t) * ms));
    GALP_CUDA(b_tsmall.alloc(sizeof(int32_t) * (size_t)std::max<int64_t>(sched.max_scope_small, 1)));
    GALP_CUDA(b_tmid.alloc(sizeof(int32_t) * (size_t)std::max<int64_t>(sched.max_scope_mid, 1)));
    GALP_CUDA(b_bsum.alloc(sizeof(int64_t) * (size_t)std::max<int64_t>((sched.max_scope_vertices + kScanBlock - 1) / kScanBlock, 1)));
    GALP_CUDA(cudaStreamSynchronize(st));
    phase(2);
    // dispatch: static features, variant table, per-scope state, logs
    {
        float sf[kDegBins + 3] = {};
        for (int b = 0; b < kDegBins; ++b) sf[b] = m > 0 ? (float)(sched.deg_hist[b] / (double)m) : 0.f;
        sf[kDegBins] = (float)(std::log2((double)std::max<int64_t>(m, 1)) / 40.0);
        sf[kDegBins + 1] = (float)(std::log2((double)std::max<int64_t>(n, 1)) / 40.0);
        sf[kDegBins + 2] = (float)(std::log2(std::max(1.0, (double)m / (double)std::max<int64_t>(n, 1))) / 16.0);
        GALP_CUDA(b_static_feat.alloc(sizeof(sf)));
        GALP_CUDA(cudaMemcpyAsync(b_static_feat.p, sf, sizeof(sf), cudaMemcpyHostToDevice, st));
        std::memcpy(static_feat, sf, sizeof(sf));
        build_variant_table();
        GALP_CUDA(b_vtab.alloc(sizeof(DispatchState) * kVar));
        GALP_CUDA(cudaMemcpyAsync(b_vtab.p, vtab.data(), sizeof(DispatchState) * kVar, cudaMemcpyHostToDevice, st));
        GALP_CUDA(b_disp.alloc(sizeof(DispatchState) * std::max<size_t>(sched.scopes.size(), 1)));
        GALP_CUDA(b_feat_log.alloc(sizeof(float) * kMaxLogIters * kFeat));
        GALP_CUDA(b_var_log.alloc(sizeof(int32_t) * kMaxLogIters));
        GALP_CUDA(b_weights.alloc(sizeof(float) * mlp_param_count(kFeat, kHid, kVar)));
        GALP_CUDA(cudaStreamSynchronize(st));
    }

    GALP_CUDA(b_lab0.alloc(sizeof(int32_t) * std::max<int64_t>(n, 1)));
    GALP_CUDA(b_lab1.alloc(sizeof(int32_t) * std::max<int64_t>(n, 1)));
    GALP_CUDA(b_ctl.alloc(sizeof(Ctl)));
    const size_t nbig = sched.big_v.size();
    GALP_CUDA(b_bstat.alloc(sizeof(BigStat) * std::max<size_t>(nbig, 1)));
    GALP_CUDA(b_big_a.alloc(sizeof(int64_t) * std::max<size_t>(nbig, 1)));
    GALP_CUDA(b_big_list.alloc(sizeof(unsigned long long) * std::max<int64_t>(sched.max_occ_slots, 1)));
    if (nbig) {
        init_bigstat_kernel<<<(unsigned)((nbig + 255) / 256), 256, 0, st>>>((BigStat *)b_bstat.p, (int)nbig);
        GALP_CUDA(cudaGetLastError());
    }
    phase(3);
    if (policy == 0) {
        // validate the resident graph before any iteration touches it; strictly increasing
        // adjacency enables the first-iteration shortcut, a symmetric edge multiset the
        // frontier (checked only when the frontier is wanted)
        GALP_CUDA(b_bad.alloc(sizeof(int)));
        GALP_CUDA(b_chk.alloc(5 * sizeof(unsigned long long)));
        GALP_CUDA(cudaMemsetAsync(b_chk.p, 0, 5 * sizeof(unsigned long long), st));
        unsigned long long *dchk = (unsigned long long *)b_chk.p;
        if (frontier) {  // rows needed for the checksum: one pass that knows each entry's row
            adjacency_check_kernel<<<sms * 8, kTB, 0, st>>>((const int64_t *)b_off.p, (const int32_t *)b_nbr[0].p,
                                                            n, 1, dchk);
        } else {
            csr_scan_kernel<<<sms * 16, kTB, 0, st>>>((const int32_t *)b_nbr[0].p, m, n, dchk);
            row_start_kernel<<<sms * 8, kTB, 0, st>>>((const int64_t *)b_off.p, (const int32_t *)b_nbr[0].p, n, dchk);
        }
        GALP_CUDA(cudaGetLastError());
        unsigned long long chk[5] = {1, 1, 1, 1, 0};
        GALP_CUDA(cudaMemcpyAsync(chk, b_chk.p, sizeof(chk), cudaMemcpyDeviceToHost, st));
        GALP_CUDA(cudaStreamSynchronize(st));
        if (chk[3]) return GALP_EFORMAT;
        adj_sorted = chk[0] == chk[4];
        symmetric = frontier && chk[1] == 0 && chk[2] == 0;
        if (!symmetric) frontier = false;
    }
    if (frontier) {
        GALP_CUDA(b_dirty.alloc(nn));
        GALP_CUDA(b_changed.alloc(sizeof(int32_t) * nn));
    }
    GALP_CUDA(cudaStreamSynchronize(st));

    phase(4);
    GALP_CUDA(cudaFuncSetAttribute(count_cta_kernel<512, 2 * kXlAMax>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)(sizeof(unsigned long long) * 2 * kXlAMax)));
    GALP_CUDA(cudaFuncSetAttribute(count_cta_kernel<kXlThreads, kXlSlots>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)(sizeof(unsigned long long) * kXlSlots)));
    return GALP_OK;
}

// Batched mode: `count` graphs concatenated into one CSR whose neighbour IDs are global;
// graph g owns vertices [graph_v0[g], graph_v0[g+1]) and must not reach outside them.
// Each graph keeps its own labels (local IDs), run positions, last vertex and early exit,
// exactly as a separate in-core run of it.
int Engine::setup_batch(const galp_csr &g, const int64_t *graph_v0, int32_t count, const galp_opts &o,
                        cudaStream_t st, int64_t &h2d)
{
    if (o.policy != 0) return GALP_EUNSUPPORTED;
    if (count < 1 || graph_v0[0] != 0 || graph_v0[count] != g.n) return GALP_EINVAL;
    for (int32_t i = 0; i < count; ++i)
        if (graph_v0[i + 1] < graph_v0[i]) return GALP_EINVAL;
    batched = true;
    G = count;
    early_exit = o.early_exit ? 1 : 0;
    galp_opts o2 = o;
    o2.frontier = 0;
    int rc = setup(g, o2, st, h2d);
    if (rc) return rc;
    if (!sched.big_v.empty()) return GALP_EUNSUPPORTED;  // global tables share one run-position scope
    g_v0_h.assign(graph_v0, graph_v0 + count + 1);
    g_last_h.assign(count, -1);
    for (int32_t i = 0; i < count; ++i)
        for (int64_t v = graph_v0[i + 1] - 1; v >= graph_v0[i]; --v)
            if (g.offsets[v + 1] > g.offsets[v]) {
                g_last_h[i] = (int32_t)v;
                break;
            }
    batch_max_iter = GALP_MAX_ITERS;
    int32_t *dummy = nullptr;
    int64_t *dv0 = nullptr;
    if ((rc = upload(b_g_v0, dv0, g_v0_h, st, h2d))) return rc;
    if ((rc = upload(b_g_last, dummy, g_last_h, st, h2d))) return rc;
    GALP_CUDA(b_g_base.alloc(sizeof(int64_t) * (count + 1)));
    GALP_CUDA(b_gid.alloc(sizeof(int32_t) * (size_t)std::max<int64_t>(g.n, 1)));
    batch_gid_kernel<<<(unsigned)std::min<int64_t>(count, 4096), kTB, 0, st>>>(dv0, count, (int32_t *)b_gid.p);
    max_label = 0;
    for (int32_t i = 0; i < count; ++i) max_label = std::max(max_label, graph_v0[i + 1] - graph_v0[i]);
    GALP_CUDA(b_g_active.alloc(sizeof(int32_t) * count));
    GALP_CUDA(b_g_iters.alloc(sizeof(int32_t) * count));
    GALP_CUDA(b_g_counts.alloc(sizeof(long long) * (size_t)count * batch_max_iter));
    GALP_CUDA(cudaMemsetAsync(b_g_counts.p, 0, sizeof(long long) * (size_t)count * batch_max_iter, st));
    GALP_CUDA(cudaMemsetAsync(b_g_iters.p, 0, sizeof(int32_t) * count, st));
    // every edge stays inside its graph
    GALP_CUDA(cudaMemsetAsync(b_bad.p, 0, sizeof(int), st));
    batch_validate_kernel<<<(unsigned)std::min<int64_t>(count, 4096), kTB, 0, st>>>(
        (const int64_t *)b_off.p, (const int32_t *)b_nbr[0].p, dv0, count, (int *)b_bad.p);
    GALP_CUDA(cudaGetLastError());
    int bad = 0;
    GALP_CUDA(cudaMemcpyAsync(&bad, b_bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    GALP_CUDA(cudaStreamSynchronize(st));
    return bad ? GALP_EFORMAT : GALP_OK;
}

int Engine::setup_hub_parts(int shift, cudaStream_t st, int64_t &h2d)
{
    plan_hub_parts(sched, shift);
    int rc;
    if ((rc = upload(b_hub_p0, d_hub_p0, sched.hub_p0, st, h2d))) return rc;
    if ((rc = upload(b_hub_pbase, d_hub_pbase, sched.hub_pbase, st, h2d))) return rc;
    if ((rc = upload(b_hub_pcap, d_hub_pcap, sched.hub_pcap, st, h2d))) return rc;
    if ((rc = upload(b_part_big, d_part_big, sched.part_big, st, h2d))) return rc;
    const size_t nparts = std::max<size_t>(sched.part_big.size(), 1);
    GALP_CUDA(b_pfill.alloc(sizeof(int) * nparts));
    GALP_CUDA(cudaMemsetAsync(b_pfill.p, 0, sizeof(int) * nparts, st));
    GALP_CUDA(b_psum.alloc(sizeof(int4) * nparts));
    GALP_CUDA(b_pairs.alloc(sizeof(unsigned long long) * (size_t)std::max<int64_t>(sched.max_pair_slots, 1)));
    if (!hub_count_blocks && !sched.part_big.empty()) {
        const int smem = (int)(sizeof(uint32_t) * 2 * kHubTab), smem2 = (int)(sizeof(uint32_t) * kHubTab),
                  smem4 = (int)(sizeof(uint32_t) * kHubTab / 2);
        auto *k1 = hub_count_kernel<kHubCountThreads, kHubTab>;
        auto *k2 = hub_count_kernel<kHubCountThreads / 2, kHubTab / 2>;
        auto *k4 = hub_count_kernel<kHubCountThreads / 4, kHubTab / 4>;
        GALP_CUDA(cudaFuncSetAttribute(k1, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        GALP_CUDA(cudaFuncSetAttribute(k2, cudaFuncAttributeMaxDynamicSharedMemorySize, smem2));
        int occ = 0, occ2 = 0, occ4 = 0;
        GALP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k1, kHubCountThreads, smem));
        GALP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ2, k2, kHubCountThreads / 2, smem2));
        GALP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ4, k4, kHubCountThreads / 4, smem4));
        hub_count_blocks = std::max(occ, 1) * sms;
        hub_count_blocks_half = std::max(occ2, 1) * sms;
        hub_count_blocks_quarter = std::max(occ4, 1) * sms;
    }
    GALP_CUDA(cudaStreamSynchronize(st));
    return GALP_OK;
}

IterArgs Engine::big_args(const Scope &sc) const
{
    IterArgs a{};
    a.off = (const int64_t *)b_off.p;
    a.last_v = sc.last_v;
    a.ctl = (Ctl *)b_ctl.p;
    a.b0 = sc.b0;
    a.nbig = sc.nb;
    a.big_v = d_big_v;
    a.big_ooff = d_big_ooff;
    a.c0 = sc.c0;
    a.chunk_big = d_chunk_big;
    a.chunk_e0 = d_chunk_e0;
    a.chunk_e1 = d_chunk_e1;
    a.nchunks = sc.nc;
    a.s0 = sc.s0;
    a.schunk_big = d_schunk_big;
    a.schunk_s0 = d_schunk_s0;
    a.schunk_s1 = d_schunk_s1;
    a.nschunks = sc.ns;
    a.hub_p0 = d_hub_p0;
    a.hub_pbase = d_hub_pbase;
    a.hub_pcap = d_hub_pcap;
    a.part_big = d_part_big;
    a.q0 = sc.q0;
    a.nparts = sc.nq;
    a.pfill = (int *)b_pfill.p;
    a.psum = (int4 *)b_psum.p;
    a.pairs = (unsigned long long *)b_pairs.p;
    a.big_list = (unsigned long long *)b_big_list.p;
    a.bstat = (BigStat *)b_bstat.p;
    a.big_a = (int64_t *)b_big_a.p;
    a.runbase = (const int64_t *)b_runbase.p;
    a.nbr_shift = (policy == 0) ? 0 : sc.e0;
    return a;
}

// Variant table rows of the in-core scope: k = 8 * aggregated + 4 * (warp/CTA split at
// 128) + 2 * (CTA split at 1024) + frontier.  Row 0 is the fixed heuristic's dense
// iteration and row 1 its frontier iteration.
void Engine::build_variant_table()
{
    vtab.assign(kVar, DispatchState{});
    const Scope &sc = sched.scopes.empty() ? Scope() : sched.scopes[0];
    auto cut = [&](int t) {  // mid-list entries of degree <= t
        const int32_t *b = sched.mid_deg.data() + sc.m0;
        const int cnt = sc.nms + sc.nml + sc.nmx;
        return (int32_t)(std::upper_bound(b, b + cnt, t) - b);
    };
    for (int k = 0; k < kVar; ++k) {
        DispatchState &d = vtab[k];
        d.agg_mode = (k & 8) ? 1 : 2;
        d.pos1 = cut((k & 4) ? 128 : kMidSMax);
        d.pos2 = cut((k & 2) ? 1024 : kLargeMax);
        d.pos_a = std::max(d.pos1, cut(kLargeAMax));
        d.pos_b = std::max(d.pos2, cut(kXlAMax));
        d.frontier = k & 1;
        d.variant = k;
    }
}

// Static per-scope states of the fixed rule (out-of-core scopes).
std::vector<DispatchState> Engine::static_dispatch() const
{
    std::vector<DispatchState> ds(std::max<size_t>(sched.scopes.size(), 1));
    for (size_t j = 0; j < sched.scopes.size(); ++j) {
        const Scope &sc = sched.scopes[j];
        ds[j].agg_mode = variant.agg_mode;
        ds[j].pos1 = sc.nms;
        ds[j].pos2 = sc.nms + sc.nml;
        const int32_t *b = sched.mid_deg.data() + sc.m0;
        const int cnt = sc.nms + sc.nml + sc.nmx;
        ds[j].pos_a = (int32_t)(std::upper_bound(b, b + cnt, kLargeAMax) - b);
        ds[j].pos_b = (int32_t)(std::upper_bound(b, b + cnt, kXlAMax) - b);
    }
    return ds;
}

PipeArgs Engine::pipe_args(const Scope &sc) const
{
    PipeArgs q{};
    q.disp = (const DispatchState *)b_disp.p + (&sc - sched.scopes.data());
    q.lab27 = max_label < (1 << 27) - 1;
    q.small_sort = variant.small_sort;
    if (batched) {
        q.g_v0 = (const int64_t *)b_g_v0.p;
        q.g_base = (const int64_t *)b_g_base.p;
        q.g_last = (const int32_t *)b_g_last.p;
        q.gid = (const int32_t *)b_gid.p;
        q.ngraphs = G;
    }
    q.nbr_shift = (policy == 0) ? 0 : sc.e0;
    q.off = (const int64_t *)b_off.p;
    q.ctl = (Ctl *)b_ctl.p;
    q.pack_v0 = d_pack_v0 + sc.p0;
    q.pack_nv = d_pack_nv + sc.p0;
    q.npacks = sc.np;
    q.small_v = d_small_v + sc.sv0;
    q.nsmall = sc.nsv;
    q.mid_v = d_mid_v + sc.m0;
    q.nmid_s = sc.nms;
    q.nmid_l = sc.nml;
    q.nmid_x = sc.nmx;
    q.dcnt = (int32_t *)b_dcnt.p;
    q.runbase = (int64_t *)b_runbase.p;
    q.sm_c0 = (int32_t *)b_c0.p;
    q.sm_c1 = (int32_t *)b_c1.p;
    q.sm_kw = (int32_t *)b_kw.p;
    q.sm_r = (int32_t *)b_r.p;
    q.run_lab = (int32_t *)b_run_lab.p;
    q.run_cnt = (uint16_t *)b_run_cnt.p;
    q.tied_small = (int32_t *)b_tsmall.p;
    q.tied_mid = (int32_t *)b_tmid.p;
    q.v0 = sc.v0;
    q.v1 = sc.v1;
    q.bsum = (int64_t *)b_bsum.p;
    q.last_v = sc.last_v;
    q.narrow_cut = variant.cta_narrow ? sc.nnarrow : -1;
    return q;
}

// One update of one scope: reads lab_in (all vertices), writes lab_out for the scope.
int Engine::launch_limits()
{
    GALP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_mid, count_mid64_kernel, 32 * kMidWarps, 0));
    GALP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_mid_sort, count_mid_sort_kernel, 32 * kMidWarps, 0));
    occ_mid_sort = std::max(occ_mid_sort, 1);
    GALP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_resolve, resolve_small_kernel, kTB, 0));
    GALP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_resolve_mid, resolve_mid_kernel, kTB, 0));
    // the CTA kernels loop over their vertex range: a grid of exactly the resident blocks
    GALP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_cta64, count_cta_kernel<64, 2 * kNarrowMax>, 64,
                                                            sizeof(unsigned long long) * 2 * kNarrowMax));
    GALP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_cta128, count_cta_kernel<128, 2 * kLargeAMax>, 128,
                                                            sizeof(unsigned long long) * 2 * kLargeAMax));
    GALP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_cta256, count_cta_kernel<kTB, 2 * kLargeMax>, kTB,
                                                            sizeof(unsigned long long) * 2 * kLargeMax));
    occ_cta64 = std::max(occ_cta64, 1);
    occ_cta128 = std::max(occ_cta128, 1);
    occ_cta256 = std::max(occ_cta256, 1);
    occ_mid = std::max(occ_mid, 1);
    occ_resolve = std::max(occ_resolve, 1);
    occ_resolve_mid = std::max(occ_resolve_mid, 1);
    return GALP_OK;
}

int Engine::enqueue_scope(cudaStream_t st, const Scope &sc, const int32_t *nbr, const int32_t *lab_in,
                          int32_t *lab_out, const uint8_t *dirty, int32_t *changed)
{
    if (!occ_mid) {
        int rc = launch_limits();
        if (rc) return rc;
    }
    IterArgs a = big_args(sc);
    a.nbr = nbr;
    a.lab_in = lab_in;
    a.lab_out = lab_out;
    a.changed = changed;
    PipeArgs q = pipe_args(sc);
    q.nbr = nbr;
    q.lab_in = lab_in;
    q.lab_out = lab_out;
    q.dirty = dirty;
    q.changed = changed;
    Ctl *ctl = (Ctl *)b_ctl.p;
    GALP_CUDA(cudaMemsetAsync(&ctl->tied_small, 0, 2 * sizeof(int), st));
    prof.kmark("memset", st);
    int e0 = -1;
    if (a.nbig) {
        if (prof.on) e0 = prof.mark(st);
        big_insert_kernel<<<a.nchunks, kTB, 0, st>>>(a);
        launched("big_insert_kernel", st);
        // smaller partitions (hub_part_shift), smaller tables and more CTAs per SM
        if (sched.hub_shift >= 2)
            hub_count_kernel<kHubCountThreads / 4, kHubTab / 4>
                <<<std::min(a.nparts, hub_count_blocks_quarter), kHubCountThreads / 4,
                   sizeof(uint32_t) * kHubTab / 2, st>>>(a);
        else if (sched.hub_shift == 1)
            hub_count_kernel<kHubCountThreads / 2, kHubTab / 2>
                <<<std::min(a.nparts, hub_count_blocks_half), kHubCountThreads / 2, sizeof(uint32_t) * kHubTab,
                   st>>>(a);
        else
            hub_count_kernel<kHubCountThreads, kHubTab>
                <<<std::min(a.nparts, hub_count_blocks), kHubCountThreads, sizeof(uint32_t) * 2 * kHubTab, st>>>(a);
        launched("hub_count_kernel", st);
        big_combine_kernel<<<(a.nbig + 7) / 8, 256, 0, st>>>(a);
        launched("big_combine_kernel", st);
        big_stats_kernel<<<a.nschunks, kTB, 0, st>>>(a);
        launched("big_stats_kernel", st);
        big_dcnt_kernel<<<(a.nbig + 255) / 256, 256, 0, st>>>(a, q.dcnt);
        launched("big_dcnt_kernel", st);
        if (prof.on) prof.spans[1].push_back({e0, prof.mark(st)});
    }
    if (prof.on) e0 = prof.mark(st);
    if (q.npacks && variant.small_sort == 2) {
        // one thread per small vertex, over the small-vertex list
        const int blocks = (int)std::min<int64_t>(((int64_t)q.nsmall + 127) / 128, (int64_t)sms * kSmallLaneBlocks);
        count_small_lane_kernel<<<blocks, 128, 0, st>>>(q);
        launched("count_small_lane_kernel", st);
    } else if (q.npacks) {
        // several waves: blocks that finish early take up the remaining ones (pack costs vary)
        const int blocks = (int)std::min<int64_t>(((int64_t)q.npacks * 32 + 255) / 256, (int64_t)sms * small_bps);
        count_small_kernel<<<blocks, 256, 0, st>>>(q);
        launched("count_small_kernel", st);
    }
    if (q.nmid_s + q.nmid_l + q.nmid_x) {
        // ranges of the degree-sorted mid list come from the dispatch state
        const int gmid = (int)std::min<int64_t>((sc.nms + kMidWarps - 1) / kMidWarps + 1,
                                                (int64_t)sms * std::min(mid_bps, variant.mid_sort ? occ_mid_sort : occ_mid));
        if (variant.mid_sort) {  // sort + reduce counting of the warp range
            count_mid_sort_kernel<<<gmid, 32 * kMidWarps, 0, st>>>(q);
            launched("count_mid_sort_kernel", st);
        } else {
            count_mid64_kernel<<<gmid, 32 * kMidWarps, 0, st>>>(q);
            launched("count_mid64_kernel", st);
        }
        const int g128 = (int)std::max<int64_t>(1, std::min<int64_t>(sc.nms + sc.nml, (int64_t)sms * occ_cta128));
        const int g256 = (int)std::max<int64_t>(1, std::min<int64_t>(sc.nml, (int64_t)sms * occ_cta256));
        if (q.narrow_cut > 0) {  // the lower part of the 128-thread range, in 64-thread CTAs
            const int g64 = (int)std::min<int64_t>(q.narrow_cut, (int64_t)sms * occ_cta64);
            count_cta_kernel<64, 2 * kNarrowMax><<<g64, 64, sizeof(unsigned long long) * 2 * kNarrowMax, st>>>(q, 4);
            launched("count_cta_kernel<64>", st);
        }
        if (variant.cta_stage) {  // neighbour IDs staged by bulk copies (the stage follows the table)
            count_cta_kernel<128, 2 * kLargeAMax, true>
                <<<g128, 128, sizeof(unsigned long long) * 2 * kLargeAMax + sizeof(int32_t) * (kLargeAMax + 8), st>>>(
                    q, 0);
            launched("count_cta_kernel<128>", st);
            count_cta_kernel<kTB, 2 * kLargeMax, true>
                <<<g256, kTB, sizeof(unsigned long long) * 2 * kLargeMax + sizeof(int32_t) * (kLargeMax + 8), st>>>(
                    q, 1);
            launched("count_cta_kernel<256>", st);
        } else {
            count_cta_kernel<128, 2 * kLargeAMax><<<g128, 128, sizeof(unsigned long long) * 2 * kLargeAMax, st>>>(q, 0);
            launched("count_cta_kernel<128>", st);
            count_cta_kernel<kTB, 2 * kLargeMax><<<g256, kTB, sizeof(unsigned long long) * 2 * kLargeMax, st>>>(q, 1);
            launched("count_cta_kernel<256>", st);
        }
        if (q.nmid_x + q.nmid_l) {
            count_cta_kernel<512, 2 * kXlAMax>
                <<<(int)std::max<int64_t>(1, std::min<int64_t>(q.nmid_x + q.nmid_l, (int64_t)sms * 2)), 512,
                   sizeof(unsigned long long) * 2 * kXlAMax, st>>>(q, 2);
            launched("count_cta_kernel<512>", st);
        }
        if (q.nmid_x) {
            count_cta_kernel<kXlThreads, kXlSlots>
                <<<(int)std::min<int64_t>(q.nmid_x, (int64_t)sms), kXlThreads, sizeof(unsigned long long) * kXlSlots,
                   st>>>(q, 3);
            launched("count_cta_kernel<1024>", st);
        }
    }
    const int64_t nv = sc.v1 - sc.v0;
    if (nv > 0) {
        const int nblk = (int)((nv + kScanBlock - 1) / kScanBlock);
        scan_reduce_kernel<<<nblk, kTB, 0, st>>>(q);
        launched("scan_reduce_kernel", st);
        scan_spine_kernel<<<1, kTB, 0, st>>>(q, nblk);
        launched("scan_spine_kernel", st);
        scan_apply_kernel<<<nblk, kTB, 0, st>>>(q);
        launched("scan_apply_kernel", st);
    }
    if (batched) {
        batch_bases_kernel<<<(G + 1 + 255) / 256, 256, 0, st>>>((const int64_t *)b_g_v0.p, G, q.runbase, n,
                                                                (const Ctl *)b_ctl.p, (int64_t *)b_g_base.p);
        launched("batch_bases_kernel", st);
    }
    resolve_small_kernel<<<sms * std::min(resolve_bps, occ_resolve), kTB, 0, st>>>(q);
    launched("resolve_small_kernel", st);
    if (q.nmid_s + q.nmid_l + q.nmid_x) {
        resolve_mid_kernel<<<sms * occ_resolve_mid, kTB, 0, st>>>(q);
        launched("resolve_mid_kernel", st);
    }
    if (prof.on) prof.spans[0].push_back({e0, prof.mark(st)});
    if (a.nbig) {
        if (prof.on) e0 = prof.mark(st);
        big_resolve_kernel<<<a.nbig, 32, sizeof(uint32_t) * kPickScratch, st>>>(a);
        launched("big_resolve_kernel", st);
        big_reset_kernel<<<(a.nbig + 255) / 256, 256, 0, st>>>(a);
        launched("big_reset_kernel", st);
        if (prof.on) prof.spans[2].push_back({e0, prof.mark(st)});
    }
    GALP_CUDA(cudaGetLastError());
    return GALP_OK;
}

int Engine::enqueue_init(cudaStream_t st, int niter, long long thr)
{
    prof.kstart(st);
    if (batched) {
        batch_init_labels_kernel<<<(unsigned)std::min<int64_t>(G, (int64_t)sms * 8), kTB, 0, st>>>(
            (const int64_t *)b_g_v0.p, G, (int32_t *)b_lab0.p);
        launched("batch_init_labels_kernel", st);
        batch_init_kernel<<<(G + 255) / 256, 256, 0, st>>>((int32_t *)b_g_active.p, (int32_t *)b_g_iters.p, G,
                                                           niter > 0 ? 1 : 0);
        launched("batch_init_kernel", st);
    } else if (n > 0) {
        const unsigned blocks = (unsigned)std::min<int64_t>((n + 255) / 256, 4096);
        init_labels_kernel<<<blocks, 256, 0, st>>>((int32_t *)b_lab0.p, n);
        launched("init_labels_kernel", st);
    }
    init_ctl_kernel<<<1, 1, 0, st>>>((Ctl *)b_ctl.p, thr, niter);
    launched("init_ctl_kernel", st);
    GALP_CUDA(cudaGetLastError());
    return GALP_OK;
}

DispatchArgs Engine::dispatch_args(int it) const
{
    DispatchArgs a{};
    a.ctl = (const Ctl *)b_ctl.p;
    a.table = (const DispatchState *)b_vtab.p;
    a.weights = (const float *)b_weights.p;
    a.static_feat = (const float *)b_static_feat.p;
    a.out = (DispatchState *)b_disp.p;
    a.feat_log = (float *)b_feat_log.p;
    a.var_log = (int32_t *)b_var_log.p;
    a.n = n;
    a.m = m;
    a.it = it;
    a.mode = disp_mode;
    a.forced = disp_forced;
    a.frontier_mode = frontier ? 1 : 0;
    a.frontier_frac = variant.frontier_frac;
    a.fixed_variant_dense = 0;
    a.fixed_variant_front = 1;
    a.fixed_agg = variant.agg_mode;
    a.margin = variant.learned_margin;
    return a;
}

int Engine::enqueue_run_incore(cudaStream_t st, int niter, long long thr)
{
    int32_t *lab[2] = {(int32_t *)b_lab0.p, (int32_t *)b_lab1.p};
    int rc = enqueue_init(st, niter, thr);
    if (rc) return rc;
    GALP_CUDA(cudaMemsetAsync(b_var_log.p, 0xFF, sizeof(int32_t) * kMaxLogIters, st));
    GALP_CUDA(cudaMemsetAsync(b_feat_log.p, 0, sizeof(float) * kMaxLogIters * kFeat, st));
    Ctl *ctl = (Ctl *)b_ctl.p;
    uint8_t *dirty = frontier ? (uint8_t *)b_dirty.p : nullptr;
    int32_t *changed = frontier ? (int32_t *)b_changed.p : nullptr;
    bool full_state = false;  // per-vertex counts and summaries hold the previous iteration
    for (int it = 0; it < niter; ++it) {
        const int it0 = prof.on ? prof.mark(st) : -1;
        const bool shortcut = it == 0 && adj_sorted && n > 0;
        if (!shortcut) {
            // this iteration's kernel variant, decided on the device
            dispatch_kernel<<<1, kHid, 0, st>>>(dispatch_args(it));
            launched("dispatch_kernel", st);
        }
        const uint8_t *dirty_it = nullptr;
        if (frontier) {
            if (full_state) {
                // vertices next to a label that changed in the previous iteration
                GALP_CUDA(cudaMemsetAsync(dirty, 0, (size_t)n, st));
                prof.kmark("memset", st);
                mark_dirty_kernel<<<sms * 8, kTB, 0, st>>>((const int64_t *)b_off.p, (const int32_t *)b_nbr[0].p,
                                                           changed, (const DispatchState *)b_disp.p, ctl, dirty);
                launched("mark_dirty_kernel", st);
                dirty_it = dirty;
            }
            GALP_CUDA(cudaMemsetAsync(&ctl->changed_n, 0, sizeof(int), st));
            prof.kmark("memset", st);
        }
        if (shortcut) {
            PipeArgs q = pipe_args(sched.scopes[0]);
            q.nbr = (const int32_t *)b_nbr[0].p;
            q.lab_in = lab[0];
            q.lab_out = lab[1];
            q.changed = changed;
            int e0 = prof.on ? prof.mark(st) : -1;
            first_iteration_kernel<<<(int)std::min<int64_t>((n + kTB - 1) / kTB, (int64_t)sms * 8), kTB, 0, st>>>(q, n, m);
            launched("first_iteration_kernel", st);
            if (prof.on) prof.spans[3].push_back({e0, prof.mark(st)});
            full_state = false;  // the shortcut leaves no per-vertex counts behind
        } else {
            if ((rc = enqueue_scope(st, sched.scopes[0], (const int32_t *)b_nbr[0].p, lab[it & 1], lab[(it + 1) & 1],
                                    dirty_it, changed)))
                return rc;
            full_state = true;
        }
        if (batched) {  // per-graph change counts, early exits and frozen graphs
            batch_commit_kernel<<<(unsigned)std::min<int64_t>(G, (int64_t)sms * 8), kTB, 0, st>>>(
                ctl, (const int64_t *)b_g_v0.p, G, lab[it & 1], lab[(it + 1) & 1], (int32_t *)b_g_active.p,
                (int32_t *)b_g_iters.p, (long long *)b_g_counts.p, batch_max_iter, it, early_exit);
            launched("batch_commit_kernel", st);
            batch_finalize_kernel<<<1, 1024, 0, st>>>(ctl, (const int32_t *)b_g_active.p, G);
            launched("batch_finalize_kernel", st);
        } else {
            finalize_kernel<<<1, 1, 0, st>>>(ctl);
            launched("finalize_kernel", st);
        }
        if (prof.on) prof.it_spans.push_back({it0, prof.mark(st)});
    }
    GALP_CUDA(cudaGetLastError());
    return GALP_OK;
}

// Policies 1/2 (SyncLP::iterate, sync.cuh:42-59; AsyncLP::iterate, async.cuh:65-89):
// batches in order, each gathering from the current labels (earlier batches of the
// iteration already applied) and committing its own labels when it is done.  Policy 2
// copies batch j+1 on the copy stream while batch j computes; events order buffer
// reuse.  With early exit on, the host waits once per iteration for the decision; with
// it off, the whole run is enqueued without a wait.
int Engine::run_outofcore(cudaStream_t st, int niter, long long thr)
{
    int32_t *cur = (int32_t *)b_lab0.p, *tmp = (int32_t *)b_lab1.p;
    int rc = enqueue_init(st, niter, thr);
    if (rc) return rc;
    const std::vector<DispatchState> ds = static_dispatch();
    GALP_CUDA(cudaMemcpyAsync(b_disp.p, ds.data(), sizeof(DispatchState) * ds.size(), cudaMemcpyHostToDevice, st));
    GALP_CUDA(cudaStreamSynchronize(st));  // ds is a local
    h2d_run = 0;
    const int nb = (int)sched.scopes.size();
    auto copy_batch = [&](int j, int buf, cudaStream_t s) -> int {
        const Scope &sc = sched.scopes[(size_t)j];
        const size_t bytes = sizeof(int32_t) * (size_t)(sc.e1 - sc.e0);
        if (bytes) GALP_CUDA(cudaMemcpyAsync(b_nbr[buf].p, h_nbr + sc.e0, bytes, cudaMemcpyHostToDevice, s));
        h2d_run += (int64_t)bytes;
        return GALP_OK;
    };
    uint64_t q = 0;  // batch sequence number of this run
    if (policy == 2 && nb > 0) {
        if ((rc = copy_batch(0, 0, copy_stream))) return rc;
        GALP_CUDA(cudaEventRecord(ev_copied[0], copy_stream));
    }
    for (int it = 0; it < niter; ++it) {
        for (int j = 0; j < nb; ++j, ++q) {
            const Scope &sc = sched.scopes[(size_t)j];
            const int buf = (int)(q & 1);
            if (policy == 2) {
                const bool more = (j + 1 < nb) || (it + 1 < niter);
                if (more) {
                    if (q >= 1) GALP_CUDA(cudaStreamWaitEvent(copy_stream, ev_consumed[buf ^ 1], 0));
                    if ((rc = copy_batch((j + 1 < nb) ? j + 1 : 0, buf ^ 1, copy_stream))) return rc;
                    GALP_CUDA(cudaEventRecord(ev_copied[buf ^ 1], copy_stream));
                }
                GALP_CUDA(cudaStreamWaitEvent(st, ev_copied[buf], 0));
            } else {
                if ((rc = copy_batch(j, buf, st))) return rc;
            }
            const int32_t *nbr = (const int32_t *)b_nbr[buf].p;
            if (it == 0 && sc.e1 > sc.e0) {
                validate_batch_kernel<<<256, 256, 0, st>>>(nbr, sc.e1 - sc.e0, n, (Ctl *)b_ctl.p);
                launched("validate_batch_kernel", st);
                GALP_CUDA(cudaGetLastError());
            }
            if ((rc = enqueue_scope(st, sc, nbr, cur, tmp))) return rc;
            if (sc.v1 > sc.v0)
                GALP_CUDA(cudaMemcpyAsync(cur + sc.v0, tmp + sc.v0, sizeof(int32_t) * (sc.v1 - sc.v0),
                                          cudaMemcpyDeviceToDevice, st));
            if (policy == 2) GALP_CUDA(cudaEventRecord(ev_consumed[buf], st));
        }
        finalize_kernel<<<1, 1, 0, st>>>((Ctl *)b_ctl.p);
        launched("finalize_kernel", st);
        GALP_CUDA(cudaGetLastError());
        // Without early exit every iteration runs: nothing to wait for, the copy stream
        // keeps streaming the next iteration's batches.  With it, the host reads the
        // device's decision once per iteration (the next iteration's first batch is
        // already being copied meanwhile), so no batch is streamed after the exit.
        if (thr >= 0 && it + 1 < niter) {
            int active = 0;
            GALP_CUDA(cudaMemcpyAsync(&active, &((Ctl *)b_ctl.p)->active, sizeof(int), cudaMemcpyDeviceToHost, st));
            GALP_CUDA(cudaStreamSynchronize(st));
            if (!active) break;
        }
    }
    if (copy_stream) GALP_CUDA(cudaStreamSynchronize(copy_stream));
    return GALP_OK;
}

const int32_t *Engine::final_labels(int iters) const
{
    if (policy != 0) return (const int32_t *)b_lab0.p;
    return (iters & 1) ? (const int32_t *)b_lab1.p : (const int32_t *)b_lab0.p;
}

}  // namespace galp

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

void galp_default_opts(galp_opts *o)
{
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->method = 0;
    o->policy = 0;
    o->lfht_policy = 1;
    o->buffer_pow = 24;
    o->frontier = 0;
    o->dispatch = 0;
    o->device = 0;
    o->early_exit = 1;
}

const char *galp_strerror(int code)
{
    switch (code) {
    case GALP_OK: return "ok";
    case GALP_EINVAL: return "invalid argument";
    case GALP_ENOMEM: return "out of memory";
    case GALP_ECUDA: return "CUDA error";
    case GALP_ETIMEOUT: return "device wait timed out";
    case GALP_EFORMAT: return "malformed graph";
    case GALP_EUNSUPPORTED: return "unsupported method/policy";
    case GALP_ENODEV: return "no CUDA device";
    case GALP_EBATCH: return "vertex degree exceeds the out-of-core batch buffer";
    default: return "unknown error";
    }
}

static int create_impl(const galp_csr *g, const galp_opts *o, galp_ctx **out, const int64_t *batch_v0,
                       int32_t batch_count);

int galp_create(const galp_csr *g, const galp_opts *o, galp_ctx **out)
{
    return create_impl(g, o, out, nullptr, 0);
}

static int create_impl(const galp_csr *g, const galp_opts *o, galp_ctx **out, const int64_t *batch_v0,
                       int32_t batch_count)
{
    if (!g || !out) return GALP_EINVAL;
    *out = nullptr;
    galp_opts opts;
    if (o) opts = *o; else galp_default_opts(&opts);
    if (g->n < 0 || g->m < 0 || g->n >= ((int64_t)1 << 31) || !g->offsets || (g->m > 0 && !g->neighbors))
        return GALP_EINVAL;
    if (g->offsets[0] != 0 || g->offsets[g->n] != g->m) return GALP_EFORMAT;
    if (opts.method < 0 || opts.method > 1) return GALP_EUNSUPPORTED;
    if (opts.policy < 0 || opts.policy > 2) return GALP_EUNSUPPORTED;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return GALP_ENODEV;
    if (opts.device < 0 || opts.device >= ndev) return GALP_EINVAL;
    if (cudaSetDevice(opts.device) != cudaSuccess) return GALP_ECUDA;

    std::unique_ptr<galp_ctx> ctx(new (std::nothrow) galp_ctx());
    if (!ctx) return GALP_ENOMEM;
    ctx->opts = opts;
    ctx->n = g->n;
    ctx->m = g->m;
    const double t0 = now_s();
    GALP_CUDA(cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking));
    ctx->stream = ctx->own_stream;
    int rc = batch_v0 ? ctx->eng.setup_batch(*g, batch_v0, batch_count, opts, ctx->stream, ctx->h2d_setup)
                      : ctx->eng.setup(*g, opts, ctx->stream, ctx->h2d_setup);
    if (rc) return rc;
    if (opts.dispatch == 1) {  // the built-in trained dispatcher
#if GALP_HAVE_TRAINED_DISPATCH
        rc = galp_dispatch_set(ctx.get(), 1, 0, kTrainedDispatch,
                               (int64_t)(sizeof(kTrainedDispatch) / sizeof(kTrainedDispatch[0])));
        if (rc) return rc;
#else
        return GALP_EUNSUPPORTED;
#endif
    } else if (opts.dispatch != 0) {
        return GALP_EINVAL;
    }
    GALP_CUDA(cudaEventCreate(&ctx->ev0));
    GALP_CUDA(cudaEventCreate(&ctx->ev1));
    ctx->t_pre = now_s() - t0;
    *out = ctx.release();
    return GALP_OK;
}

int galp_set_stream(galp_ctx *ctx, void *stream)
{
    if (!ctx) return GALP_EINVAL;
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
    return GALP_OK;
}

static long long exit_threshold(const galp_ctx *ctx)
{
    if (!ctx->opts.early_exit) return -1;  // changes are never negative: never stop early
    return (long long)std::floor((double)ctx->n * 1e-5);
}

int galp_enqueue(galp_ctx *ctx, int32_t niter)
{
    if (!ctx || niter < 0) return GALP_EINVAL;
    GALP_CUDA(cudaSetDevice(ctx->opts.device));
    GALP_CUDA(cudaEventRecord(ctx->ev0, ctx->stream));
    int rc;
    if (ctx->eng.batched && !ctx->eng.prof.on) {
        // the whole run (every iteration of every graph) as one CUDA-graph launch
        if (ctx->graph_iters != niter) {
            if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
            ctx->graph_exec = nullptr;
            ctx->graph_iters = -1;
            cudaGraph_t graph = nullptr;
            GALP_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
            rc = ctx->eng.enqueue_run_incore(ctx->stream, niter, exit_threshold(ctx));
            const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
            if (rc) {
                if (graph) cudaGraphDestroy(graph);
                return rc;
            }
            GALP_CUDA(ce);
            const cudaError_t ie = cudaGraphInstantiate(&ctx->graph_exec, graph, 0);
            cudaGraphDestroy(graph);
            GALP_CUDA(ie);
            ctx->graph_iters = niter;
        }
        GALP_CUDA(cudaGraphLaunch(ctx->graph_exec, ctx->stream));
        rc = GALP_OK;
    } else {
        rc = ctx->eng.policy == 0 ? ctx->eng.enqueue_run_incore(ctx->stream, niter, exit_threshold(ctx))
                                  : ctx->eng.run_outofcore(ctx->stream, niter, exit_threshold(ctx));
    }
    if (rc) return rc;
    GALP_CUDA(cudaEventRecord(ctx->ev1, ctx->stream));
    ctx->pending = true;
    ctx->last_niter = niter;
    return GALP_OK;
}

int galp_sync(galp_ctx *ctx, galp_stats *st)
{
    if (!ctx) return GALP_EINVAL;
    GALP_CUDA(cudaStreamSynchronize(ctx->stream));
    Ctl c;
    GALP_CUDA(cudaMemcpy(&c, ctx->eng.b_ctl.p, sizeof(Ctl), cudaMemcpyDeviceToHost));
    // a hub partition overflowed (its pairs were dropped): redo the run with twice the
    // partitions, up to 64x the default count (the labels of the redone run are exact)
    while ((c.err & kErrHubOverflow) && ctx->eng.sched.hub_shift < kMaxHubShift) {
        int64_t h2d = 0;
        int rc = ctx->eng.setup_hub_parts(ctx->eng.sched.hub_shift + 1, ctx->stream, h2d);
        if (rc) return rc;
        if ((rc = galp_enqueue(ctx, ctx->last_niter))) return rc;
        GALP_CUDA(cudaStreamSynchronize(ctx->stream));
        GALP_CUDA(cudaMemcpy(&c, ctx->eng.b_ctl.p, sizeof(Ctl), cudaMemcpyDeviceToHost));
    }
    ctx->iters = c.iter;
    ctx->err = c.err;
    ctx->runs_last = c.N;
    for (int i = 0; i < GALP_MAX_ITERS; ++i) ctx->counts[i] = (int64_t)c.counts[i];
    float ms = 0.f;
    if (ctx->pending) cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    ctx->pending = false;
    ctx->device_ms = ms;
    if (st) {
        std::memset(st, 0, sizeof(*st));
        st->device_ms = ms;
        st->iters_run = c.iter;
        st->err = c.err;
        st->runs_last = c.N;
        for (int i = 0; i < GALP_MAX_ITERS; ++i) st->updates[i] = (int64_t)c.counts[i];
    }
    if (c.err & kErrFormat) return GALP_EFORMAT;
    if (c.err & kErrHubOverflow) return GALP_ENOMEM;
    return (c.err & (kErrLookback | kErrStage)) ? GALP_ETIMEOUT : GALP_OK;
}

int galp_run(galp_ctx *ctx, int32_t niter, galp_stats *st)
{
    if (!ctx || niter < 0) return GALP_EINVAL;
    const double t0 = now_s();
    int rc = galp_enqueue(ctx, niter);
    if (rc) return rc;
    galp_stats tmp;
    rc = galp_sync(ctx, &tmp);
    if (rc && rc != GALP_ETIMEOUT) return rc;
    // final labels to the host (dpp.cuh:93)
    ctx->labels.resize((size_t)ctx->n);
    const int32_t *src = ctx->eng.final_labels(ctx->iters);
    if (ctx->n) GALP_CUDA(cudaMemcpy(ctx->labels.data(), src, sizeof(int32_t) * ctx->n, cudaMemcpyDeviceToHost));
    ctx->have_labels = true;
    const double f1 = now_s() - t0;
    if (st) {
        *st = tmp;
        st->f1 = f1;
        st->f2 = f1 + ctx->t_pre;
        st->h2d_bytes = ctx->h2d_setup + ctx->eng.h2d_run;
        st->d2h_bytes = (int64_t)sizeof(int32_t) * ctx->n;
    }
    return rc;
}

int galp_get_labels(galp_ctx *ctx, int32_t *out, int64_t n)
{
    if (!ctx || n != ctx->n || (!out && n > 0)) return GALP_EINVAL;
    if (!ctx->have_labels) {
        // labels of the last enqueued run, if any, else the initial labels
        const int32_t *src = ctx->eng.final_labels(ctx->iters);
        GALP_CUDA(cudaStreamSynchronize(ctx->stream));
        if (n) GALP_CUDA(cudaMemcpy(out, src, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
        return GALP_OK;
    }
    if (n) std::memcpy(out, ctx->labels.data(), sizeof(int32_t) * n);
    return GALP_OK;
}

void galp_destroy(galp_ctx *ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->opts.device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
}

int galp_probe_gather(galp_ctx *ctx, int32_t reps, float *ms_per_pass)
{
    if (!ctx || reps < 1 || !ms_per_pass) return GALP_EINVAL;
    const galp::Engine &E = ctx->eng;
    if (E.policy != 0 || E.batched) return GALP_EUNSUPPORTED;
    GALP_CUDA(cudaSetDevice(ctx->opts.device));
    unsigned long long *acc = (unsigned long long *)E.b_chk.p;  // 5 words from setup's checks
    if (!acc || ctx->m == 0) {
        *ms_per_pass = 0.f;
        return GALP_OK;
    }
    const int blocks = E.sms * 8;
    galp::gather_probe_kernel<<<blocks, galp::kTB, 0, ctx->stream>>>((const int32_t *)E.b_nbr[0].p, ctx->m,
                                                                      (const int32_t *)E.b_lab0.p, acc);
    GALP_CUDA(cudaGetLastError());
    cudaEvent_t e0, e1;
    GALP_CUDA(cudaEventCreate(&e0));
    GALP_CUDA(cudaEventCreate(&e1));
    cudaEventRecord(e0, ctx->stream);
    for (int r = 0; r < reps; ++r)
        galp::gather_probe_kernel<<<blocks, galp::kTB, 0, ctx->stream>>>((const int32_t *)E.b_nbr[0].p, ctx->m,
                                                                          (const int32_t *)E.b_lab0.p, acc);
    cudaEventRecord(e1, ctx->stream);
    const cudaError_t le = cudaGetLastError();
    const cudaError_t se = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    GALP_CUDA(le);
    GALP_CUDA(se);
    *ms_per_pass = ms / (float)reps;
    return GALP_OK;
}

int galp_schedule_info(galp_ctx *ctx, galp_sched_info *info)
{
    if (!ctx || !info) return GALP_EINVAL;
    std::memset(info, 0, sizeof(*info));
    const galp::Engine &E = ctx->eng;
    info->n = ctx->n;
    info->m = ctx->m;
    info->m_big = E.sched.m_big;
    info->npacks = (int64_t)E.sched.pack_v0.size();
    int64_t nms = 0, nml = 0;
    for (const galp::Scope &sc : E.sched.scopes) {
        nms += sc.nms;
        nml += sc.nml + sc.nmx;
    }
    info->nmid = nms;
    info->nlarge = nml;
    info->nbig = (int64_t)E.sched.big_v.size();
    info->table_slots = E.sched.max_pair_slots;
    info->launches_per_iter = 14 + (info->nbig ? 7 : 0) + (E.frontier ? 1 : 0) + (E.variant.cta_narrow ? 1 : 0);
    info->flags = (E.adj_sorted ? GALP_SCHED_SORTED : 0) | (E.symmetric ? GALP_SCHED_SYMMETRIC : 0) |
                  (E.frontier ? GALP_SCHED_FRONTIER : 0);
    info->launches = E.launches;
    for (int i = 0; i < 5; ++i) info->setup_ms[i] = E.setup_ms[i];
    return GALP_OK;
}

int galp_set_variant(galp_ctx *ctx, const galp_variant *v)
{
    if (!ctx || !v || v->agg_mode < 0 || v->agg_mode > 2 || !(v->frontier_frac >= 0.f && v->frontier_frac <= 1.f) ||
        !(v->learned_margin >= 0.f && v->learned_margin < 10.f) || v->small_sort < 0 || v->small_sort > 2 ||
        v->cta_stage < 0 || v->cta_stage > 1 || v->cta_narrow < 0 || v->cta_narrow > 1 || v->mid_sort < 0 ||
        v->mid_sort > 1)
        return GALP_EINVAL;
    if (v->hub_part_shift < -16 || v->hub_part_shift > kMaxHubShift) return GALP_EINVAL;
    if (v->hub_part_shift != ctx->eng.sched.hub_shift) {
        int64_t h2d = 0;
        GALP_CUDA(cudaStreamSynchronize(ctx->stream));
        const int rc = ctx->eng.setup_hub_parts(v->hub_part_shift, ctx->stream, h2d);
        if (rc) return rc;
    }
    ctx->eng.variant = *v;
    // a batched run is a captured CUDA graph: capture again with the new kernels
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    ctx->graph_exec = nullptr;
    ctx->graph_iters = -1;
    return GALP_OK;
}

int galp_get_variant(galp_ctx *ctx, galp_variant *v)
{
    if (!ctx || !v) return GALP_EINVAL;
    *v = ctx->eng.variant;
    v->hub_part_shift = ctx->eng.sched.hub_shift;
    return GALP_OK;
}

int galp_dispatch_set(galp_ctx *ctx, int32_t mode, int32_t forced_variant, const float *weights, int64_t count)
{
    if (!ctx || mode < 0 || mode > 2) return GALP_EINVAL;
    galp::Engine &E = ctx->eng;
    if (mode == 2 && (forced_variant < 0 || forced_variant >= galp::kVar)) return GALP_EINVAL;
    if (weights) {
        if (count != galp::mlp_param_count(galp::kFeat, galp::kHid, galp::kVar)) return GALP_EINVAL;
        GALP_CUDA(cudaMemcpyAsync(E.b_weights.p, weights, sizeof(float) * count, cudaMemcpyHostToDevice, ctx->stream));
        GALP_CUDA(cudaStreamSynchronize(ctx->stream));
        E.have_weights = true;
    }
    if (mode == 1 && !E.have_weights) return GALP_EINVAL;
    E.disp_mode = mode;
    E.disp_forced = forced_variant;
    return GALP_OK;
}

int galp_dispatch_log(galp_ctx *ctx, float *features, int32_t *variants, int32_t cap_iters, int32_t *count)
{
    if (!ctx || !count || cap_iters < 0) return GALP_EINVAL;
    galp::Engine &E = ctx->eng;
    GALP_CUDA(cudaStreamSynchronize(ctx->stream));
    const int nlog = std::min(std::min(ctx->iters, (int)galp::kMaxLogIters), (int)cap_iters);
    *count = nlog;
    if (nlog > 0 && features)
        GALP_CUDA(cudaMemcpy(features, E.b_feat_log.p, sizeof(float) * galp::kFeat * nlog, cudaMemcpyDeviceToHost));
    if (nlog > 0 && variants)
        GALP_CUDA(cudaMemcpy(variants, E.b_var_log.p, sizeof(int32_t) * nlog, cudaMemcpyDeviceToHost));
    return GALP_OK;
}

int galp_dispatch_table(galp_ctx *ctx, galp_dispatch_row *rows, int32_t cap, int32_t *count)
{
    if (!ctx || !count || cap < 0 || (cap > 0 && !rows)) return GALP_EINVAL;
    const galp::Engine &E = ctx->eng;
    *count = (int32_t)E.vtab.size();
    for (int32_t k = 0; k < cap && k < *count; ++k) {
        rows[k].agg_mode = E.vtab[k].agg_mode;
        rows[k].frontier = E.vtab[k].frontier;
        rows[k].warp_max_degree = (k & 4) ? 128 : galp::kMidSMax;
        rows[k].cta256_max_degree = (k & 2) ? 1024 : galp::kLargeMax;
        rows[k].pos1 = E.vtab[k].pos1;
        rows[k].pos2 = E.vtab[k].pos2;
    }
    return GALP_OK;
}

int galp_profile_iterations(galp_ctx *ctx, float *ms, int32_t cap, int32_t *count)
{
    if (!ctx || !count || cap < 0 || (cap > 0 && !ms)) return GALP_EINVAL;
    GALP_CUDA(cudaStreamSynchronize(ctx->stream));
    galp::Profiler &P = ctx->eng.prof;
    P.fold();
    *count = (int32_t)P.it_ms.size();
    for (int32_t i = 0; i < cap && i < *count; ++i) ms[i] = P.it_ms[i];
    P.it_ms.clear();
    return GALP_OK;
}

int galp_batch_create(const int64_t *offsets, const int32_t *neighbors, int64_t n, int64_t m,
                      const int64_t *graph_v0, int32_t count, const galp_opts *opts, galp_ctx **out)
{
    if (!offsets || !graph_v0 || !out || n < 0 || m < 0 || count < 1) return GALP_EINVAL;
    // the schedule is built on the host: bring device offsets over
    std::vector<int64_t> host_off;
    const int64_t *off = offsets;
    cudaPointerAttributes pa{};
    if (cudaPointerGetAttributes(&pa, offsets) == cudaSuccess && pa.type == cudaMemoryTypeDevice) {
        host_off.resize((size_t)n + 1);
        GALP_CUDA(cudaMemcpy(host_off.data(), offsets, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost));
        off = host_off.data();
    } else {
        (void)cudaGetLastError();
    }
    galp_csr g{neighbors, off, n, m};
    return create_impl(&g, opts, out, graph_v0, count);
}

int galp_batch_stats(galp_ctx *ctx, int32_t graph, galp_stats *st)
{
    if (!ctx || !st || !ctx->eng.batched || graph < 0 || graph >= ctx->eng.G) return GALP_EINVAL;
    galp::Engine &E = ctx->eng;
    GALP_CUDA(cudaStreamSynchronize(ctx->stream));
    std::memset(st, 0, sizeof(*st));
    int32_t it = 0;
    GALP_CUDA(cudaMemcpy(&it, (const int32_t *)E.b_g_iters.p + graph, sizeof(int32_t), cudaMemcpyDeviceToHost));
    st->iters_run = it;
    std::vector<long long> c(E.batch_max_iter);
    GALP_CUDA(cudaMemcpy(c.data(), (const long long *)E.b_g_counts.p + (size_t)graph * E.batch_max_iter,
                         sizeof(long long) * E.batch_max_iter, cudaMemcpyDeviceToHost));
    for (int i = 0; i < GALP_MAX_ITERS && i < it; ++i) st->updates[i] = (int64_t)c[i];
    st->device_ms = ctx->device_ms;
    return GALP_OK;
}

int galp_batch_labels(galp_ctx *ctx, int32_t graph, int32_t *labels, int64_t n)
{
    if (!ctx || !ctx->eng.batched || graph < 0 || graph >= ctx->eng.G) return GALP_EINVAL;
    galp::Engine &E = ctx->eng;
    const int64_t v0 = E.g_v0_h[graph], v1 = E.g_v0_h[graph + 1];
    if (n != v1 - v0 || (n > 0 && !labels)) return GALP_EINVAL;
    GALP_CUDA(cudaStreamSynchronize(ctx->stream));
    if (n) GALP_CUDA(cudaMemcpy(labels, E.final_labels(ctx->iters) + v0, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
    return GALP_OK;
}

int galp_run_batch(const galp_csr *graphs, int32_t count, const galp_opts *opts, int32_t niter, int32_t *labels_out,
                   galp_stats *stats)
{
    if (!graphs || count < 1 || niter < 0) return GALP_EINVAL;
    std::vector<int64_t> v0(count + 1, 0), off;
    int64_t n = 0, m = 0;
    for (int32_t i = 0; i < count; ++i) {
        const galp_csr &g = graphs[i];
        if (g.n < 0 || g.m < 0 || !g.offsets || (g.m > 0 && !g.neighbors)) return GALP_EINVAL;
        if (g.offsets[0] != 0 || g.offsets[g.n] != g.m) return GALP_EFORMAT;
        n += g.n;
        m += g.m;
        v0[i + 1] = n;
    }
    if (n >= ((int64_t)1 << 31)) return GALP_EINVAL;
    off.resize((size_t)n + 1);
    std::vector<int32_t> nbr((size_t)std::max<int64_t>(m, 1));
    int64_t e = 0;
    for (int32_t i = 0; i < count; ++i) {
        const galp_csr &g = graphs[i];
        for (int64_t v = 0; v < g.n; ++v) off[v0[i] + v] = e + g.offsets[v];
        for (int64_t k = 0; k < g.m; ++k) {
            const int32_t u = g.neighbors[k];
            if (u < 0 || u >= g.n) return GALP_EFORMAT;
            nbr[e + k] = (int32_t)(u + v0[i]);
        }
        e += g.m;
    }
    off[n] = m;
    galp_ctx *ctx = nullptr;
    int rc = galp_batch_create(off.data(), nbr.data(), n, m, v0.data(), count, opts, &ctx);
    if (rc) return rc;
    rc = galp_run(ctx, niter, nullptr);
    for (int32_t i = 0; !rc && i < count; ++i) {
        if (labels_out) rc = galp_batch_labels(ctx, i, labels_out + v0[i], v0[i + 1] - v0[i]);
        if (!rc && stats) rc = galp_batch_stats(ctx, i, &stats[i]);
    }
    galp_destroy(ctx);
    return rc;
}

// Launch-shape autotuner for batched runs: coordinate descent over blocks per SM of the
// small-vertex counting, mid-vertex counting and small-vertex resolve kernels, each
// candidate timed on a probe run of niter iterations.
int galp_batch_tune(galp_ctx *ctx, int32_t niter, galp_tune_result *res)
{
    if (!ctx || niter < 1) return GALP_EINVAL;
    galp::Engine &E = ctx->eng;
    int *knob[3] = {&E.small_bps, &E.mid_bps, &E.resolve_bps};
    const int cand[3][4] = {{8, 16, 24, 32}, {2, 4, 6, 8}, {2, 4, 8, 16}};
    float best_ms = 0.f;
    int trials = 0;
    auto probe = [&](float &ms) -> int {  // best of two runs
        ms = 1e30f;
        for (int rep = 0; rep < 2; ++rep) {
            int rc2 = galp_enqueue(ctx, niter);
            if (rc2) return rc2;
            GALP_CUDA(cudaEventSynchronize(ctx->ev1));
            float t = 0.f;
            GALP_CUDA(cudaEventElapsedTime(&t, ctx->ev0, ctx->ev1));
            ms = std::min(ms, t);
        }
        ++trials;
        return GALP_OK;
    };
    const bool was_on = E.prof.on;
    E.prof.on = true;  // enqueue directly while probing (no graph capture)
    const int level = E.prof.level;
    E.prof.level = 0;
    int rc = probe(best_ms);  // warm-up
    if (!rc) rc = probe(best_ms);
    for (int k = 0; !rc && k < 3; ++k) {
        int keep = *knob[k];
        for (int c = 0; !rc && c < 4; ++c) {
            if (cand[k][c] == keep) continue;
            const int old = *knob[k];
            *knob[k] = cand[k][c];
            float ms = 0.f;
            rc = probe(ms);
            if (!rc && ms < best_ms) {
                best_ms = ms;
                keep = cand[k][c];
            }
            *knob[k] = old;
        }
        *knob[k] = keep;
    }
    // bucket shapes: the degree splits between warp and CTA counting (128 / 256) and
    // between CTA sizes (1024 / 2048) and the insert aggregation, as fixed variant rows
    // (frontier off); a row is kept only when it beats the per-iteration fixed rule by 1 %
    int best_row = -1;
    if (!rc && !E.frontier) {
        const int mode0 = E.disp_mode, forced0 = E.disp_forced;
        for (int row = 0; !rc && row < galp::kVar; row += 2) {
            E.disp_mode = 2;
            E.disp_forced = row;
            float ms = 0.f;
            rc = probe(ms);
            if (!rc && ms < 0.99f * best_ms) {
                best_ms = ms;
                best_row = row;
            }
        }
        E.disp_mode = best_row >= 0 ? 2 : mode0;
        E.disp_forced = best_row >= 0 ? best_row : forced0;
    }
    E.prof.on = was_on;
    E.prof.level = level;
    E.prof.spans[0].clear();
    E.prof.spans[1].clear();
    E.prof.spans[2].clear();
    E.prof.spans[3].clear();
    E.prof.it_spans.clear();
    E.prof.used = 0;
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);  // recapture with the chosen shapes
    ctx->graph_exec = nullptr;
    ctx->graph_iters = -1;
    if (rc) return rc;
    if (res) {
        res->small_blocks_per_sm = E.small_bps;
        res->mid_blocks_per_sm = E.mid_bps;
        res->resolve_blocks_per_sm = E.resolve_bps;
        res->trials = trials;
        res->best_ms = best_ms;
        res->dispatch_row = best_row;
    }
    return GALP_OK;
}

int galp_profile(galp_ctx *ctx, int32_t level)
{
    if (!ctx || level < 0 || level > 2) return GALP_EINVAL;
    ctx->eng.prof.level = level;
    ctx->eng.prof.on = level >= 1;
    return GALP_OK;
}

int galp_profile_read(galp_ctx *ctx, galp_kernel_times *out)
{
    if (!ctx || !out) return GALP_EINVAL;
    std::memset(out, 0, sizeof(*out));
    GALP_CUDA(cudaStreamSynchronize(ctx->stream));
    galp::Profiler &P = ctx->eng.prof;
    P.fold();
    out->pipe_ms = P.group_ms[0];
    out->pipe_groups = P.group_n[0];
    out->big_pre_ms = P.group_ms[1];
    out->big_pre_groups = P.group_n[1];
    out->big_post_ms = P.group_ms[2];
    out->big_post_groups = P.group_n[2];
    out->first_ms = P.group_ms[3];
    out->first_groups = P.group_n[3];
    for (int g = 0; g < 4; ++g) {
        P.group_ms[g] = 0;
        P.group_n[g] = 0;
    }
    return GALP_OK;
}

int galp_profile_kernels(galp_ctx *ctx, galp_kernel_stat *out, int32_t cap, int32_t *count)
{
    if (!ctx || !count || cap < 0 || (cap > 0 && !out)) return GALP_EINVAL;
    GALP_CUDA(cudaStreamSynchronize(ctx->stream));
    galp::Profiler &P = ctx->eng.prof;
    P.fold();
    *count = (int32_t)P.kstats.size();
    for (int32_t i = 0; i < cap && i < *count; ++i) {
        std::memset(&out[i], 0, sizeof(out[i]));
        std::strncpy(out[i].name, P.kstats[i].first, sizeof(out[i].name) - 1);
        out[i].ms = P.kstats[i].second.first;
        out[i].launches = P.kstats[i].second.second;
    }
    P.kstats.clear();
    return GALP_OK;
}

int32_t galp_debug_resolve_rank(int64_t a, int64_t d, int64_t N, int32_t is_last, const int32_t *cand, int32_t k)
{
    struct Q {
        const int32_t *c;
        int32_t k;
        __host__ __device__ int first_ge(int64_t x)
        {
            for (int i = 0; i < k; ++i)
                if (c[i] >= x) return c[i];
            return -1;
        }
        __host__ __device__ int last_lt(int64_t y)
        {
            int r = -1;
            for (int i = 0; i < k; ++i)
                if (c[i] < y) r = c[i];
            return r;
        }
        __host__ __device__ int tile_pick(int64_t lo)
        {
            int r = -1, best = -1;
            for (int i = 0; i < k; ++i)
                if (c[i] >= lo && c[i] < lo + galp::kTile && galp::tile_priority(c[i] - lo) > best) {
                    best = galp::tile_priority(c[i] - lo);
                    r = c[i];
                }
            return r;
        }
    } q{cand, k};
    if (!cand || k <= 0 || d <= 0) return -1;
    return galp::resolve_rank(a, d, N, is_last != 0, q);
}

}  // extern "C"
