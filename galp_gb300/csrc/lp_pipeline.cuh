// lp_pipeline.cuh -- count -> scan -> resolve: the exact label-propagation update
// without inter-block waiting.
//
// One iteration over a scope (whole graph, one out-of-core batch):
//
//   count   vertices are degree-bucketed and counted with no dependence between blocks:
//             small (degree <= 32, and degree 0): one warp per pack of <= 32 label
//               slots, counting in registers (__match_any_sync on (vertex, label));
//             mid (33..256): one warp per vertex, shared-memory hash region;
//             large (257..2048): one CTA per vertex, shared-memory hash region;
//             big (> 2048): global tables (big_insert/big_stats, lp_kernels.cuh).
//           Each vertex gets its distinct-label count d; a vertex with a unique
//           most-frequent label is final and written at once.  A tied vertex leaves a
//           summary (smallest/largest candidate, their ranks, #candidates, max count)
//           and its (label, count) runs in a spill area at its own CSR positions,
//           and joins a list of tied vertices.
//   scan    exclusive scan of d over the scope's vertices: each vertex's run base,
//           the position of its first run in the reference's run array
//           (label_propagation/src/dpp/kernel.cuh:66-82 scatter_indexes).
//   resolve each tied vertex picks its winner by the reference's positional tie rule
//           (resolve_rank, lp_resolve.h) from its summary, or from its spilled runs.
//
// Spill layout (indexed by CSR position relative to the scope's first entry):
//   run_lab[e0 + r] label, run_cnt[e0 + r] count of the vertex's r-th run; small
//   vertices write their runs sorted by label, mid/large vertices their table's
//   occupied entries unsorted (queried by order statistics).
#pragma once

#include "rmat_rng.h"
#include "lp_kernels.cuh"
#include "lp_dispatch.cuh"

namespace galp {

constexpr int kMidSMax = 256;        // mid bucket: 33..256 neighbours, one warp each
constexpr int kMidSCap = 2 * kMidSMax;
constexpr int kMidWarps = 8;         // warps (vertices) per mid CTA
constexpr int kScanBlock = 4096;     // vertices per scan block (256 threads x 16)
constexpr int kLargeMax = 2048;      // large bucket: 257..2048, one 256-thread CTA each
constexpr int kXlMax = 12288;        // xl bucket: 2049..12288, one CTA each (512 or 1024 threads)
constexpr int kXlSlots = 2 * kXlMax; // 192 KB of shared-memory table (64-bit slots)
constexpr int kXlThreads = 1024;
constexpr int kLargeAMax = 1024;     // large vertices up to here: 128-thread CTAs, 16 KB tables
constexpr int kXlAMax = 6144;        // xl vertices up to here: 512-thread CTAs, 96 KB tables
constexpr int kNarrowMax = 512;      // narrow CTA variant: large vertices up to here, 64 threads,
                                     // 8 KB tables

struct PipeArgs {
    const int32_t *nbr;     // neighbour buffer holding CSR entries [nbr_shift, ...)
    int64_t nbr_shift;
    const int64_t *off;
    const int32_t *lab_in;
    int32_t *lab_out;
    Ctl *ctl;
    // static buckets of the scope
    const int32_t *pack_v0;
    const uint8_t *pack_nv;
    int32_t npacks;
    const int32_t *small_v; // the same vertices one by one (thread-per-vertex counting)
    int32_t nsmall;
    const int32_t *mid_v;   // mid (33..256), then large (257..2048), then xl (2049..12288) vertices
    int32_t nmid_s, nmid_l, nmid_x;
    // per-vertex state (global vertex index)
    int32_t *dcnt;          // distinct labels
    int64_t *runbase;       // run base relative to the scope
    int32_t *sm_c0, *sm_c1; // smallest / largest candidate label
    int32_t *sm_kw;         // candidates | max count << 16
    int32_t *sm_r;          // rank of smallest | rank of largest << 16
    // spill, indexed by CSR position - nbr_shift
    int32_t *run_lab;
    uint16_t *run_cnt;
    // tied lists
    int32_t *tied_small;
    int32_t *tied_mid;
    // scan
    int64_t v0, v1;         // scope vertices
    int64_t *bsum;          // per scan block
    int32_t last_v;
    // frontier mode (null = every vertex is recounted and no changes are recorded)
    const uint8_t *dirty;   // 1 = a neighbour's label changed in the previous iteration
    int32_t *changed;       // vertices whose label changes in this iteration
    const DispatchState *disp;  // this iteration's variant (mid-list split, inserts, frontier)
    // batched mode (null g_v0 = one graph): graph g owns vertices [g_v0[g], g_v0[g+1]), its
    // own run positions (g_base[g] = run base of its first vertex), labels and last vertex
    const int64_t *g_v0;
    const int64_t *g_base;
    const int32_t *g_last;
    const int32_t *gid;     // graph of every vertex
    int32_t ngraphs;
    int32_t lab27;          // every label below 2^27 - 1 (32-bit sort keys in packs)
    int32_t small_sort;     // small vertices: 0 match-based packs, 1 sort-based packs (needs lab27),
                            // 2 one thread per vertex
    int32_t narrow_cut;     // -1, or the mid-list position of the first vertex above kNarrowMax
                            // neighbours: the 128-thread CTA range is split there, its lower
                            // part going to 64-thread CTAs
};

// Graph of vertex v in batched mode: the largest g with g_v0[g] <= v.
__device__ __forceinline__ int find_graph(const int64_t *g_v0, int ngraphs, int64_t v)
{
    int lo = 0, hi = ngraphs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&g_v0[mid]) <= v) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Run position scope of a vertex: its run base a, the scope's run count N, and whether it
// is the scope's last run-owning vertex (the whole graph, or its graph in batched mode).
struct RunScope {
    long long a, N;
    bool is_last;
};

__device__ __forceinline__ RunScope run_scope(const PipeArgs &p, int v)
{
    if (!p.g_v0) return RunScope{p.runbase[v], p.ctl->N, v == p.last_v};
    const int g = __ldg(&p.gid[v]);
    const long long base = p.g_base[g];
    return RunScope{p.runbase[v] - base, p.g_base[g + 1] - base, v == p.g_last[g]};
}

__device__ __forceinline__ void count_change(unsigned long long &changes, int32_t nl, int32_t old)
{
    changes += (nl != old);
}

// Frontier mode and this iteration not switched to a full recount.
__device__ __forceinline__ bool frontier_on(const PipeArgs &p)
{
    return p.dirty && !*((volatile int *)&p.ctl->frontier_off);
}

// Record a changed vertex for the next iteration's frontier (single thread).
__device__ __forceinline__ void note_change(const PipeArgs &p, int32_t v, int32_t nl, int32_t old)
{
    if (p.changed && nl != old) p.changed[atomicAdd(&p.ctl->changed_n, 1)] = v;
}

__device__ __forceinline__ void flush_changes(unsigned long long changes, Ctl *ctl)
{
    unsigned long long c = changes;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) c += __shfl_xor_sync(kFull, c, off);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(&ctl->changes, c);
}

// warp-aggregated append of the lanes with `pred` to list[ctr++]
__device__ __forceinline__ void warp_append(bool pred, int32_t value, int32_t *list, int *ctr)
{
    const unsigned m = __ballot_sync(kFull, pred);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == __ffs(m) - 1) base = atomicAdd(ctr, __popc(m));
    base = __shfl_sync(kFull, base, __ffs(m) - 1);
    if (pred) list[base + __popc(m & ((1u << lane) - 1))] = value;
}

// Warp-private shared-memory buffer in front of a shared append-only list (the tied
// lists): a warp appends with one ballot, and the buffer reaches the list with one global
// atomic per kWarpBuf entries instead of one per append.  In the tie-heavy iterations
// nearly every pack and vertex appends, and atomics on the one list counter serialise in L2.
constexpr int kWarpBuf = 64;
constexpr int kCtaBuf = 16;
struct WarpBuf {
    int32_t *buf;  // kWarpBuf entries of this warp's shared memory
    int n = 0;     // warp-uniform fill
    __device__ void flush(int32_t *list, int *ctr)
    {
        if (!n) return;
        const int lane = threadIdx.x & 31;
        int base = 0;
        if (lane == 0) base = atomicAdd(ctr, n);
        base = __shfl_sync(kFull, base, 0);
        for (int i = lane; i < n; i += 32) list[base + i] = buf[i];
        __syncwarp();
        n = 0;
    }
    __device__ void append(bool pred, int32_t value, int32_t *list, int *ctr)
    {
        const unsigned m = __ballot_sync(kFull, pred);
        if (!m) return;
        if (n + __popc(m) > kWarpBuf) flush(list, ctr);
        const int lane = threadIdx.x & 31;
        if (pred) buf[n + __popc(m & ((1u << lane) - 1))] = value;
        n += __popc(m);
        __syncwarp();
    }
};

// warp-level version of note_change (all lanes call it)
__device__ __forceinline__ void warp_note_changes(const PipeArgs &p, bool changed, int32_t v)
{
    if (p.changed) warp_append(changed, v, p.changed, &p.ctl->changed_n);
}

// Per-vertex results of a counted pack: the values live at each vertex's first slot lane
// and move to the vertex lanes, which write the vertex state (all lanes call this).
__device__ __forceinline__ void finish_small_pack(const PipeArgs &p, bool vl, int v, int deg, int pos, int d, int k,
                                                  int W, int cmin, int cmax, int rmin, int rmax,
                                                  unsigned long long &changes, WarpBuf &tb)
{
    const int lane = threadIdx.x & 31;
    // results live at each vertex's first slot lane; bring them to the vertex lanes
    const int src = (vl && deg > 0) ? pos : lane;
    // d, k, W <= 32 and ranks < 32: one word
    const uint32_t packed = (uint32_t)d | ((uint32_t)k << 6) | ((uint32_t)W << 12) | ((uint32_t)rmin << 18) |
                            ((uint32_t)rmax << 23);
    const uint32_t pk_v = __shfl_sync(kFull, packed, src);
    const int d_v = (int)(pk_v & 63), k_v = (int)((pk_v >> 6) & 63), W_v = (int)((pk_v >> 12) & 63);
    const int r0_v = (int)((pk_v >> 18) & 31), r1_v = (int)((pk_v >> 23) & 31);
    const int c0_v = __shfl_sync(kFull, cmin, src);
    const int c1_v = __shfl_sync(kFull, cmax, src);
    const bool tied = vl && deg > 0 && k_v > 1;
    bool chg = false;
    if (vl) {
        p.dcnt[v] = deg > 0 ? d_v : 0;
        const int32_t old = __ldg(&p.lab_in[v]);
        if (deg > 0) p.sm_kw[v] = k_v | (W_v << 16);
        if (!tied) {
            const int32_t nl = deg > 0 ? c0_v : old;
            p.lab_out[v] = nl;
            count_change(changes, nl, old);
            chg = nl != old;
        } else {
            p.sm_c0[v] = c0_v;
            p.sm_c1[v] = c1_v;
            p.sm_r[v] = r0_v | (r1_v << 16);
        }
    }
    tb.append(tied, v, p.tied_small, &p.ctl->tied_small);
    warp_note_changes(p, chg, v);
}

// ---------------------------------------------------------------------------
// small vertices: one warp per pack
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256, 6) count_small_kernel(PipeArgs p)
{
    __shared__ int32_t tbuf[8][kWarpBuf];
    if (!ctl_active(p.ctl)) return;
    const bool fr = frontier_on(p);
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    unsigned long long changes = 0;
    WarpBuf tb{tbuf[threadIdx.x >> 5]};
    for (int pk = gw; pk < p.npacks; pk += nw) {
        const int v0 = p.pack_v0[pk], nv = p.pack_nv[pk];
        // vertex lanes: offsets, degrees, slot positions
        const bool vl = lane < nv;
        const int v = v0 + lane;
        if (fr && !__any_sync(kFull, vl && p.dirty[v])) {
            // no label around this pack changed: counts and summaries carry over; labels
            // of untied vertices stay, tied vertices are resolved again (run bases move)
            bool tied = false;
            if (vl && (__ldg(&p.off[v + 1]) > __ldg(&p.off[v]))) tied = (p.sm_kw[v] & 0xFFFF) > 1;
            if (vl && !tied) p.lab_out[v] = __ldg(&p.lab_in[v]);
            tb.append(tied, v, p.tied_small, &p.ctl->tied_small);
            continue;
        }
        // The pack's CSR entries are contiguous: slot lane i holds entry obase + i.  Vertex
        // lanes read their offsets (an offset minus obase is the vertex's first slot lane);
        // the slot lanes of one vertex form a segment [first, last] found from the mask of
        // segment starts.
        const int64_t ol = __ldg(&p.off[v0 + min(lane, nv)]);
        const int64_t obase = __shfl_sync(kFull, ol, 0);
        const int64_t oend = nv < 32 ? __shfl_sync(kFull, ol, nv) : __ldg(&p.off[v0 + 32]);
        const int64_t onext = __shfl_down_sync(kFull, ol, 1);
        const int deg = vl ? (int)((lane == 31 ? oend : onext) - ol) : 0;
        const int pos = (int)(ol - obase);
        const int total = (int)(oend - obase);
        const bool valid = lane < total;
        const unsigned starts = __reduce_or_sync(kFull, (vl && deg > 0) ? (1u << pos) : 0u);
        const unsigned upto = (2u << lane) - 1u;  // lanes 0..lane
        const int j = valid ? 31 - __clz(starts & upto) : lane;  // segment id = its first lane
        const unsigned later_start = starts & ~upto;
        const int seg_last = valid ? (later_start ? __ffs(later_start) - 2 : total - 1) : lane;
        const int64_t oj = obase + j;  // the owner's first CSR entry
        int lab = 0;
        if (valid) lab = ld_label(&p.lab_in[ld_nbr(&p.nbr[obase + lane - p.nbr_shift])]);
        const unsigned vm = valid ? (((seg_last == 31) ? kFull : ((2u << seg_last) - 1u)) & ~((1u << j) - 1u))
                                  : (1u << lane);
        if (p.small_sort && p.lab27) {
            // Sort-based counting: sort the pack by (vertex lane << 27 | label) in one 32-bit
            // key (padding lanes last; a vertex keeps its slot lanes), then every run of equal
            // keys is one distinct label: heads give d, run lengths give counts, and
            // candidates come out in label order (cmin/cmax and their ranks by bit scans).
            uint32_t sk = valid ? (((uint32_t)j << 27) | (uint32_t)lab) : 0xFFFFFFFFu;
#pragma unroll
            for (int kk = 2; kk <= 32; kk <<= 1) {
#pragma unroll
                for (int jj = kk >> 1; jj > 0; jj >>= 1) {
                    const uint32_t ok = __shfl_xor_sync(kFull, sk, jj);
                    const bool up = (lane & kk) == 0, lower = (lane & jj) == 0;
                    sk = ((lower == up) ? (ok < sk) : (ok > sk)) ? ok : sk;
                }
            }
            const int first = __ffs(vm) - 1, last = 31 - __clz(vm);
            const int slab = (int)(sk & ((1u << 27) - 1));
            const uint32_t prevk = __shfl_up_sync(kFull, sk, 1);
            const bool head = valid && (lane == first || prevk != sk);
            const unsigned hm = __ballot_sync(kFull, head) & vm;
            const unsigned later = hm & ~((2u << lane) - 1u);
            const int cnt = head ? (later ? __ffs(later) - 1 : last + 1) - lane : 0;
            const int W = seg_max(cnt, lane, first, last);
            const unsigned cm = __ballot_sync(kFull, head && cnt == W) & vm;
            const int k = __popc(cm), d = __popc(hm);
            const int lo = cm ? __ffs(cm) - 1 : lane, hi = cm ? 31 - __clz(cm) : lane;
            const int cmin = __shfl_sync(kFull, slab, lo), cmax = __shfl_sync(kFull, slab, hi);
            const int rmin = __popc(hm & ((1u << lo) - 1)), rmax = __popc(hm & ((1u << hi) - 1));
            if (head && k > 2) {
                const int64_t e = oj - p.nbr_shift + __popc(hm & ((1u << lane) - 1));
                p.run_lab[e] = slab;
                p.run_cnt[e] = (uint16_t)cnt;
            }
            finish_small_pack(p, vl, v, deg, pos, d, k, W, cmin, cmax, rmin, rmax, changes, tb);
            continue;
        }
        const unsigned eq = __match_any_sync(kFull, valid ? (uint32_t)lab : (0x80000000u | (uint32_t)lane)) & vm;
        const int cnt = __popc(eq);
        const bool leader = valid && ((__ffs(eq) - 1) == lane);
        const unsigned lm = __ballot_sync(kFull, leader);
        const int first = __ffs(vm) - 1, last = 31 - __clz(vm);
        const int W = seg_max(valid ? cnt : 0, lane, first, last);
        const bool cand = leader && cnt == W;
        const unsigned cm = __ballot_sync(kFull, cand);
        const int k = __popc(cm & vm);
        const int d = __popc(lm & vm);
        int cmin, cmax, rmin = 0, rmax = 0;
        if (__all_sync(kFull, !valid || k == 1)) {
            const unsigned m = cm & vm;
            cmin = cmax = __shfl_sync(kFull, lab, m ? (__ffs(m) - 1) : lane);
        } else {
            cmin = seg_min(cand ? lab : INT_MAX, lane, first, last);
            cmax = seg_max(cand ? lab : -1, lane, first, last);
            rmin = __popc(__ballot_sync(kFull, leader && lab < cmin) & vm);
            rmax = __popc(__ballot_sync(kFull, leader && lab < cmax) & vm);
            if (p.lab27 && __any_sync(kFull, valid && k > 2)) {
                // resolving a vertex with more than two candidates may need its runs in
                // label order: sort the pack by (vertex lane << 27 | label) in one 32-bit
                // key (labels below 2^27 - 1; padding lanes sort last), then spill the
                // runs of those vertices; run lengths come from the run heads
                uint32_t sk = valid ? (((uint32_t)j << 27) | (uint32_t)lab) : 0xFFFFFFFFu;
#pragma unroll
                for (int kk = 2; kk <= 32; kk <<= 1) {
#pragma unroll
                    for (int jj = kk >> 1; jj > 0; jj >>= 1) {
                        const uint32_t ok = __shfl_xor_sync(kFull, sk, jj);
                        const bool up = (lane & kk) == 0, lower = (lane & jj) == 0;
                        sk = ((lower == up) ? (ok < sk) : (ok > sk)) ? ok : sk;
                    }
                }
                const int slab = (int)(sk & ((1u << 27) - 1));
                const uint32_t prevk = __shfl_up_sync(kFull, sk, 1);
                const bool head = valid && (lane == first || prevk != sk);
                const unsigned hm = __ballot_sync(kFull, head) & vm;
                const int rank = __popc(hm & ((1u << lane) - 1));
                const unsigned later = hm & ~((2u << lane) - 1u);
                const int sc = (later ? __ffs(later) - 1 : last + 1) - lane;
                if (head && k > 2) {
                    const int64_t e = oj - p.nbr_shift + rank;
                    p.run_lab[e] = slab;
                    p.run_cnt[e] = (uint16_t)sc;
                }
            } else if (__any_sync(kFull, valid && k > 2)) {
                // labels of 27 bits or more: 64-bit (vertex, label) keys
                unsigned long long sk =
                    valid ? (((unsigned long long)(unsigned)j << 32) | (unsigned)lab) : (0xFFFFFFFF00000000ull | lane);
                int sc = valid ? cnt : 0;
#pragma unroll
                for (int kk = 2; kk <= 32; kk <<= 1) {
#pragma unroll
                    for (int jj = kk >> 1; jj > 0; jj >>= 1) {
                        const unsigned long long ok = __shfl_xor_sync(kFull, sk, jj);
                        const int oc = __shfl_xor_sync(kFull, sc, jj);
                        const bool up = (lane & kk) == 0, lower = (lane & jj) == 0;
                        if ((lower == up) ? (ok < sk) : (ok > sk)) {
                            sk = ok;
                            sc = oc;
                        }
                    }
                }
                const int slab = (int)(unsigned)sk;
                const int prev = __shfl_up_sync(kFull, slab, 1);
                const bool head = valid && (lane == first || prev != slab);
                const unsigned hm = __ballot_sync(kFull, head) & vm;
                const int rank = __popc(hm & ((1u << lane) - 1));
                if (head && k > 2) {
                    const int64_t e = oj - p.nbr_shift + rank;
                    p.run_lab[e] = slab;
                    p.run_cnt[e] = (uint16_t)sc;
                }
            }
        }
        finish_small_pack(p, vl, v, deg, pos, d, k, W, cmin, cmax, rmin, rmax, changes, tb);
    }
    tb.flush(p.tied_small, &p.ctl->tied_small);
    flush_changes(changes, p.ctl);
}

// ---------------------------------------------------------------------------
// mid, large and xl vertices: generation-tagged hash tables in shared memory
// ---------------------------------------------------------------------------
//
// A slot is one 64-bit word: generation (19 bits) | label (31 bits) | count (14 bits).
// Every vertex a table serves gets a new generation, so slots left by earlier vertices
// read as free and the table is never cleared between vertices; an insert either adds
// to the slot holding its label or claims a stale slot with one compare-and-swap.
// Degrees stay below 2^14 on these paths and labels below 2^31.
constexpr int kT64GenShift = 45;
constexpr uint32_t kT64GenMax = (1u << 19) - 1;
constexpr unsigned long long kT64CntMask = (1ull << 14) - 1;

__device__ __forceinline__ unsigned long long t64_tag(uint32_t gen, uint32_t label)
{
    return ((unsigned long long)gen << kT64GenShift) | ((unsigned long long)label << 14);
}

// Adds c occurrences of label.  Returns the label's count right after this insert and
// sets `claimed` when the insert took a new slot (the label's first insert).
__device__ __forceinline__ uint32_t t64_insert(unsigned long long *tab, uint32_t cap, uint32_t gen, uint32_t label,
                                               uint32_t c, bool &claimed)
{
    const unsigned long long tag = t64_tag(gen, label);
    uint32_t h = hslot(label, cap);
    // Plain loads: a slot that holds this vertex's generation never changes its label, and
    // a stale view of a free slot is caught by the compare-and-swap.
    unsigned long long cur = tab[h];
    for (;;) {
        if ((cur & ~kT64CntMask) == tag) {
            // the count is the low 14 bits of the low word (little-endian), and the total
            // stays below 2^14: a 32-bit add never carries into the label
            claimed = false;
            return (atomicAdd((unsigned int *)&tab[h], c) & (uint32_t)kT64CntMask) + c;
        }
        if ((uint32_t)(cur >> kT64GenShift) != gen) {  // stale: claim it
            const unsigned long long prev = atomicCAS(&tab[h], cur, tag | c);
            if (prev == cur) {
                claimed = true;
                return c;
            }
            cur = prev;  // taken meanwhile: look at it again
            continue;
        }
        h = (h + 1 == cap) ? 0 : h + 1;
        cur = tab[h];
    }
}

// Per-vertex summary: distinct labels d, maximum count W, number k of labels with count
// W and the smallest / largest of them.
struct Sum5 {
    int d, W, k, mn, mx;
};

__device__ __forceinline__ Sum5 sum5_empty() { return Sum5{0, 0, 0, INT_MAX, -1}; }

// Fold the count a label has right after one of its inserts (d is left to the caller).
// The counts a label passes through rise strictly and its last insert sees its final
// count, so folding every insert of a vertex gives its maximum count W, the number k
// of labels that reach W (each sees W exactly once) and their smallest and largest
// label, with no pass over the table; d is the number of slot claims.
__device__ __forceinline__ void sum5_observe(Sum5 &s, int lab, int c)
{
    if (c > s.W) {
        s.W = c;
        s.k = 1;
        s.mn = s.mx = lab;
    } else if (c == s.W) {
        s.k++;
        s.mn = min(s.mn, lab);
        s.mx = max(s.mx, lab);
    }
}

__device__ __forceinline__ Sum5 sum5_warp(const Sum5 &s)
{
    Sum5 r;
    r.W = __reduce_max_sync(kFull, s.W);
    const bool top = s.W == r.W;
    r.d = __reduce_add_sync(kFull, s.d);
    r.k = __reduce_add_sync(kFull, top ? s.k : 0);
    r.mn = __reduce_min_sync(kFull, top ? s.mn : INT_MAX);
    r.mx = __reduce_max_sync(kFull, top ? s.mx : -1);
    return r;
}

// Ranks of cmin and cmax among the vertex's distinct labels (partial counts).
__device__ __forceinline__ void t64_ranks(const unsigned long long *tab, int cap, int t0, int stride, uint32_t gen,
                                          int cmin, int cmax, int &a0, int &a1)
{
    a0 = a1 = 0;
    for (int i = t0; i < cap; i += stride) {
        const unsigned long long x = tab[i];
        if ((uint32_t)(x >> kT64GenShift) == gen) {
            const int lab = (int)((x >> 14) & 0x7FFFFFFF);
            a0 += lab < cmin;
            a1 += lab < cmax;
        }
    }
}

// Write the vertex's (label, count) entries, unsorted, to its spill positions; `ctr` is
// a shared counter the group has zeroed.
__device__ __forceinline__ void t64_spill(const unsigned long long *tab, int cap, int t0, int stride, uint32_t gen,
                                          int32_t *rl, uint16_t *rc, int *ctr)
{
    const int lane = threadIdx.x & 31;
    for (int i0 = t0 - lane; i0 < cap; i0 += stride) {  // warp-uniform trip count
        const int i = i0 + lane;
        const unsigned long long x = i < cap ? tab[i] : 0ull;
        const bool occ = i < cap && (uint32_t)(x >> kT64GenShift) == gen;
        const unsigned m = __ballot_sync(kFull, occ);
        if (!m) continue;
        int base = 0;
        if (lane == __ffs(m) - 1) base = atomicAdd(ctr, __popc(m));
        base = __shfl_sync(kFull, base, __ffs(m) - 1);
        if (occ) {
            const int at = base + __popc(m & ((1u << lane) - 1));
            rl[at] = (int32_t)((x >> 14) & 0x7FFFFFFF);
            rc[at] = (uint16_t)(x & kT64CntMask);
        }
    }
}

// Insert one row of gathered labels: lanes holding the same label add once when
// `aggregate` (heavy labels would otherwise serialise on one slot).  Each insert's
// observed count folds into `obs`; obs.d counts the claims.
__device__ __forceinline__ void t64_insert_row(unsigned long long *tab, uint32_t cap, uint32_t gen, uint32_t lb,
                                               bool aggregate, Sum5 &obs)
{
    uint32_t c = 1;
    bool mine = lb != kEmpty;
    if (aggregate) {
        const unsigned same = __match_any_sync(kFull, lb);
        mine = mine && (int)(threadIdx.x & 31) == __ffs(same) - 1;
        c = (uint32_t)__popc(same);
    }
    if (mine) {
        bool claimed;
        const uint32_t now = t64_insert(tab, cap, gen, lb, c, claimed);
        obs.d += claimed;
        sum5_observe(obs, (int)lb, (int)now);
    }
}

// Finish a counted vertex: per-vertex state, and its label unless it is tied.  One
// thread; returns whether the vertex is tied (the caller appends it to the tied list).
__device__ __forceinline__ bool finish_counted(const PipeArgs &p, int v, const Sum5 &s, int rmin, int rmax,
                                               unsigned long long &changes, int32_t old)
{
    p.dcnt[v] = s.d;
    p.sm_kw[v] = s.k | (s.W << 16);
    if (s.k == 1) {
        p.lab_out[v] = s.mn;
        count_change(changes, s.mn, old);
        note_change(p, v, s.mn, old);
        return false;
    }
    p.sm_c0[v] = s.mn;
    p.sm_c1[v] = s.mx;
    p.sm_r[v] = rmin | (rmax << 16);
    return true;
}

__device__ __forceinline__ bool finish_counted(const PipeArgs &p, int v, const Sum5 &s, int rmin, int rmax,
                                               unsigned long long &changes)
{
    return finish_counted(p, v, s, rmin, rmax, changes, __ldg(&p.lab_in[v]));
}

// Frontier: a clean vertex keeps its counts; it is re-resolved if tied, else keeps its
// label.  One thread; returns whether the vertex is tied.
__device__ __forceinline__ bool carry_clean(const PipeArgs &p, int v)
{
    if ((p.sm_kw[v] & 0xFFFF) > 1) return true;
    p.lab_out[v] = __ldg(&p.lab_in[v]);
    return false;
}

// One thread's buffer of tied vertices in shared memory (thread 0 finishes every vertex of
// a CTA counting kernel): one list reservation per kCtaBuf vertices.  Buffer and fill
// live in shared memory, so the CTA's other threads carry no registers for it; 16 entries
// keep two 96 KB-table CTAs inside the 196 KB shared-memory carve-out (more would leave
// the label gathers almost no L1).
__device__ __forceinline__ void tbuf_flush(int32_t *buf, int *n, int32_t *list, int *ctr)
{
    const int c = *n;
    if (!c) return;
    const int base = atomicAdd(ctr, c);
    for (int i = 0; i < c; ++i) list[base + i] = buf[i];
    *n = 0;
}

__device__ __forceinline__ void tbuf_append(int32_t *buf, int *n, int32_t value, int32_t *list, int *ctr)
{
    if (*n == kCtaBuf) tbuf_flush(buf, n, list, ctr);
    buf[(*n)++] = value;
}

// Small vertices (at most 32 neighbours), one thread each (`small_sort` 2): a vertex's
// neighbour labels go to the thread's 32-entry row of shared memory (element j of lane l at
// l * 32 + (j ^ l): the lanes' rows are bank-disjoint), are sorted there by insertion, and
// one pass over the sorted row gives the distinct count, the runs' counts, the maximum, the
// candidates and the ranks of the smallest and largest candidate; vertices with more than
// two candidates spill their runs in label order, as the pack kernel does.  Against the
// warp-per-pack kernel this spends per vertex a few instructions per neighbour instead of
// the per-pack segment masks, matches and segmented shuffles.
constexpr int kSmallLaneBlocks = 8;  // resident 128-thread blocks per SM (16 KB of rows each)
__global__ void __launch_bounds__(128, kSmallLaneBlocks) count_small_lane_kernel(PipeArgs p)
{
    __shared__ int32_t rows[4][32 * 32];
    __shared__ int32_t tbuf[4][kWarpBuf];
    if (!ctl_active(p.ctl)) return;
    const bool fr = frontier_on(p);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int32_t *row = rows[w] + lane * 32;
    WarpBuf tb{tbuf[w]};
    unsigned long long changes = 0;
    const int stride = gridDim.x * 128;
    // warp-uniform trip count: every lane runs the loop the same number of times
    // a lane's next vertex: index, offsets, label and dirty flag load one round ahead
    struct Head {
        int v, deg;
        int64_t o0;
        int32_t old;
        int dirty;
    };
    auto head = [&](int i) {
        Head h{0, 0, 0, 0, 1};
        if (i < p.nsmall) {
            h.v = p.small_v[i];
            h.o0 = __ldg(&p.off[h.v]);
            h.deg = (int)(__ldg(&p.off[h.v + 1]) - h.o0);
            h.old = __ldg(&p.lab_in[h.v]);
            h.dirty = fr ? (int)p.dirty[h.v] : 1;
        }
        return h;
    };
    Head nxt = head(blockIdx.x * 128 + w * 32 + lane);
    for (int base = blockIdx.x * 128 + w * 32; base < p.nsmall; base += stride) {
        const int i = base + lane;
        const bool active = i < p.nsmall;
        const Head h = nxt;
        nxt = head(i + stride);
        const int v = h.v;
        bool tied = false, chg = false;
        if (active) {
            const int64_t o0 = h.o0;
            const int deg = h.deg;
            const int32_t old = h.old;
            if (!h.dirty) {
                // no label around the vertex changed: its counts carry over
                tied = deg > 0 && (p.sm_kw[v] & 0xFFFF) > 1;
                if (!tied) p.lab_out[v] = old;
            } else if (deg == 0) {
                p.dcnt[v] = 0;
                p.lab_out[v] = old;
            } else {
                const int32_t *nb = p.nbr + (o0 - p.nbr_shift);
                // gather: all of the vertex's neighbour IDs, then all its labels, in flight
                int ids[4];
                int j = 0;
                for (; j + 4 <= deg; j += 4) {
#pragma unroll
                    for (int u = 0; u < 4; ++u) ids[u] = __ldg(&nb[j + u]);
#pragma unroll
                    for (int u = 0; u < 4; ++u) row[(j + u) ^ lane] = ld_label(&p.lab_in[ids[u]]);
                }
                for (; j < deg; ++j) row[j ^ lane] = ld_label(&p.lab_in[__ldg(&nb[j])]);
                // insertion sort of the row
                for (int a = 1; a < deg; ++a) {
                    const int32_t x = row[a ^ lane];
                    int b = a - 1;
                    while (b >= 0 && row[b ^ lane] > x) {
                        row[(b + 1) ^ lane] = row[b ^ lane];
                        --b;
                    }
                    row[(b + 1) ^ lane] = x;
                }
                // runs
                int d = 0, W = 0, k = 0, rmin = 0, rmax = 0;
                int32_t cmin = 0, cmax = 0;
                for (int a = 0; a < deg;) {
                    const int32_t lab = row[a ^ lane];
                    int e = a + 1;
                    while (e < deg && row[e ^ lane] == lab) ++e;
                    const int c = e - a;
                    if (c > W) {
                        W = c;
                        k = 1;
                        cmin = cmax = lab;
                        rmin = rmax = d;
                    } else if (c == W) {
                        ++k;
                        cmax = lab;
                        rmax = d;
                    }
                    ++d;
                    a = e;
                }
                if (k > 2) {  // resolving may need the runs: spill them in label order
                    int32_t *rl = p.run_lab + (o0 - p.nbr_shift);
                    uint16_t *rc = p.run_cnt + (o0 - p.nbr_shift);
                    int r = 0;
                    for (int a = 0; a < deg;) {
                        const int32_t lab = row[a ^ lane];
                        int e = a + 1;
                        while (e < deg && row[e ^ lane] == lab) ++e;
                        rl[r] = lab;
                        rc[r] = (uint16_t)(e - a);
                        ++r;
                        a = e;
                    }
                }
                p.dcnt[v] = d;
                p.sm_kw[v] = k | (W << 16);
                if (k == 1) {
                    p.lab_out[v] = cmin;
                    count_change(changes, cmin, old);
                    chg = cmin != old;
                } else {
                    tied = true;
                    p.sm_c0[v] = cmin;
                    p.sm_c1[v] = cmax;
                    p.sm_r[v] = rmin | (rmax << 16);
                }
            }
        }
        tb.append(tied, v, p.tied_small, &p.ctl->tied_small);
        warp_note_changes(p, chg, v);
    }
    tb.flush(p.tied_small, &p.ctl->tied_small);
    flush_changes(changes, p.ctl);
}

// What a warp or CTA needs of a mid-list vertex before counting it: loaded one vertex ahead, so
// these dependent loads (list entry, then offsets and state) are in flight while the
// previous vertex is counted.
struct CtaHead {
    int v;         // vertex, -1 past the end of the range
    int deg;
    int64_t o0;    // first CSR entry
    int dcnt;      // distinct labels in the previous iteration (aggregation rule)
    int32_t old;   // current label
    int dirty;     // 0: frontier mode and no neighbour label changed
};

__device__ __forceinline__ CtaHead cta_head(const PipeArgs &p, int first, int i, int count, bool fr)
{
    CtaHead h{-1, 0, 0, 0, 0, 1};
    if (i < count) {
        h.v = p.mid_v[first + i];
        h.o0 = __ldg(&p.off[h.v]);
        h.deg = (int)(__ldg(&p.off[h.v + 1]) - h.o0);
        h.dcnt = p.dcnt[h.v];
        h.old = __ldg(&p.lab_in[h.v]);
        h.dirty = fr ? (int)p.dirty[h.v] : 1;
    }
    return h;
}

// One warp per mid vertex (33..256 neighbours): a 512-slot table of generation-tagged
// 64-bit slots per warp (as the CTA tables: never cleared between vertices), probed over
// up to 4 slots per neighbour.  Against 32-bit key and count arrays cleared per vertex:
// no clear pass and one shared-memory atomic per insert.  The next vertex's head and its
// neighbour IDs load while the current one is counted (as in the CTA kernels).
__global__ void __launch_bounds__(32 * kMidWarps) count_mid64_kernel(PipeArgs p)
{
    __shared__ unsigned long long stab[kMidWarps][kMidSCap];
    __shared__ int32_t tbuf[kMidWarps][kWarpBuf];
    if (!ctl_active(p.ctl)) return;
    const bool fr = frontier_on(p);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int gw = blockIdx.x * kMidWarps + w;
    const int nw = gridDim.x * kMidWarps;
    unsigned long long changes = 0;
    unsigned long long *tab = stab[w];
    WarpBuf tb{tbuf[w]};
    for (int s = lane; s < kMidSCap; s += 32) tab[s] = 0ull;
    uint32_t gen = 0;
    __syncwarp();
    const int nwarp_v = p.disp->pos1;  // the degree-sorted mid list's prefix of warp vertices
    constexpr int PER = kMidSMax / 32;
    // the next vertex's head and neighbour IDs load while the current one is counted
    auto ids_ahead = [&](int (&nb)[PER], const CtaHead &h) {
#pragma unroll
        for (int u = 0; u < PER; ++u) {
            const int e = lane + u * 32;
            nb[u] = (h.v >= 0 && h.dirty && e < h.deg) ? ld_nbr(&p.nbr[h.o0 + e - p.nbr_shift]) : -1;
        }
    };
    CtaHead nxt = cta_head(p, 0, gw, nwarp_v, fr);
    int nbn[PER];
    ids_ahead(nbn, nxt);
    for (int i = gw; i < nwarp_v; i += nw) {
        const CtaHead h = nxt;
        const int v = h.v;
        int nb[PER];
#pragma unroll
        for (int u = 0; u < PER; ++u) nb[u] = nbn[u];
        nxt = cta_head(p, 0, i + nw, nwarp_v, fr);
        if (!h.dirty) {
            tb.append(lane == 0 && carry_clean(p, v), v, p.tied_mid, &p.ctl->tied_mid);
            ids_ahead(nbn, nxt);
            continue;
        }
        if (++gen > kT64GenMax) {
            for (int s = lane; s < kMidSCap; s += 32) tab[s] = 0ull;
            __syncwarp();
            gen = 1;
        }
        const int64_t o0 = h.o0;
        const int deg = h.deg;
        const uint32_t cap = (uint32_t)min(kMidSCap, 4 * pad32(deg));
        uint32_t lb[PER];
#pragma unroll
        for (int u = 0; u < PER; ++u) lb[u] = (nb[u] >= 0) ? (uint32_t)ld_label(&p.lab_in[nb[u]]) : kEmpty;
        Sum5 part = sum5_empty();  // observed counts (sum5_observe); d = claims
#pragma unroll
        for (int u = 0; u < PER; ++u) {
            if (u * 32 >= deg) break;  // warp-uniform
            // lanes holding the same label add once (heavy labels would serialise)
            t64_insert_row(tab, cap, gen, lb[u], true, part);
        }
        ids_ahead(nbn, nxt);
        __syncwarp();
        const Sum5 sm = sum5_warp(part);
        int rmin = 0, rmax = sm.d - 1;  // when every distinct label is a candidate
        if (sm.k > 1) {
            if (sm.k < sm.d) {
                t64_ranks(tab, (int)cap, lane, 32, gen, sm.mn, sm.mx, rmin, rmax);
                rmin = __reduce_add_sync(kFull, rmin);
                rmax = __reduce_add_sync(kFull, rmax);
            }
            if (sm.k > 2) {  // resolving may need the runs themselves (unsorted)
                int32_t *rl = p.run_lab + (o0 - p.nbr_shift);
                uint16_t *rc = p.run_cnt + (o0 - p.nbr_shift);
                int base = 0;
                for (int s0 = 0; s0 < (int)cap; s0 += 32) {  // cap is a multiple of 128
                    const unsigned long long x = tab[s0 + lane];
                    const bool occ = (uint32_t)(x >> kT64GenShift) == gen;
                    const unsigned m = __ballot_sync(kFull, occ);
                    if (occ) {
                        const int at = base + __popc(m & ((1u << lane) - 1));
                        rl[at] = (int32_t)((x >> 14) & 0x7FFFFFFF);
                        rc[at] = (uint16_t)(x & kT64CntMask);
                    }
                    base += __popc(m);
                }
            }
        }
        const bool tied = lane == 0 && finish_counted(p, v, sm, rmin, rmax, changes, h.old);
        tb.append(tied, v, p.tied_mid, &p.ctl->tied_mid);
        __syncwarp();
    }
    tb.flush(p.tied_mid, &p.ctl->tied_mid);
    flush_changes(changes, p.ctl);
}

// One warp per mid vertex (33..256 neighbours), counted the segmented sort + reduce way
// (the reference's method 0, dpp/segmented_sort.cuh and the boundary/scan/reduce steps of
// dpp/kernel.cuh, within one warp): the vertex's labels are sorted by a 256-key bitonic
// network (8 keys per lane; sorted position i lives in lane i / 8, register i % 8; unused
// keys are 0xFFFFFFFF and sort last), run heads are the positions whose label differs from
// the previous one, and a run's count is the distance to the next head.  The summary and
// the spill (runs in label order, which the unsorted-spill queries accept) are the ones
// the hash kernels produce.  Variant `mid_sort` 1; no table, no shared memory but the tied
// buffer.
__device__ __forceinline__ void warp_bitonic256(uint32_t (&a)[8], int lane)
{
#pragma unroll
    for (int k = 2; k <= 256; k <<= 1) {
#pragma unroll
        for (int jj = k >> 1; jj > 0; jj >>= 1) {
            if (jj >= 8) {  // partner in lane ^ (jj / 8), same register
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int i = lane * 8 + j;
                    const uint32_t o = __shfl_xor_sync(kFull, a[j], jj >> 3);
                    const bool up = (i & k) == 0, lower = (i & jj) == 0;
                    a[j] = (lower == up) ? min(a[j], o) : max(a[j], o);
                }
            } else {  // partner in this lane's registers
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int pj = j ^ jj;
                    if (pj > j) {
                        const bool up = ((lane * 8 + j) & k) == 0;
                        const uint32_t x = a[j], y = a[pj];
                        a[j] = up ? min(x, y) : max(x, y);
                        a[pj] = up ? max(x, y) : min(x, y);
                    }
                }
            }
        }
    }
}

__global__ void __launch_bounds__(32 * kMidWarps) count_mid_sort_kernel(PipeArgs p)
{
    __shared__ int32_t tbuf[kMidWarps][kWarpBuf];
    if (!ctl_active(p.ctl)) return;
    const bool fr = frontier_on(p);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int gw = blockIdx.x * kMidWarps + w;
    const int nw = gridDim.x * kMidWarps;
    unsigned long long changes = 0;
    WarpBuf tb{tbuf[w]};
    const int nwarp_v = p.disp->pos1;  // the degree-sorted mid list's prefix of warp vertices
    for (int i = gw; i < nwarp_v; i += nw) {
        const int v = p.mid_v[i];
        if (fr && !p.dirty[v]) {
            tb.append(lane == 0 && carry_clean(p, v), v, p.tied_mid, &p.ctl->tied_mid);
            continue;
        }
        const int64_t o0 = __ldg(&p.off[v]);
        const int deg = (int)(__ldg(&p.off[v + 1]) - o0);  // 33..256
        uint32_t a[8];
        {
            int nb[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int e = j * 32 + lane;  // coalesced loads; placement does not matter to the sort
                nb[j] = e < deg ? ld_nbr(&p.nbr[o0 + e - p.nbr_shift]) : -1;
            }
#pragma unroll
            for (int j = 0; j < 8; ++j) a[j] = nb[j] >= 0 ? (uint32_t)ld_label(&p.lab_in[nb[j]]) : 0xFFFFFFFFu;
        }
        warp_bitonic256(a, lane);
        // run heads: position i is valid when i < deg and a head when its label differs
        // from position i - 1's (the previous lane's last key for register 0)
        const uint32_t prev_last = __shfl_up_sync(kFull, a[7], 1);
        unsigned hm = 0;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int pos = lane * 8 + j;
            const uint32_t prev = j ? a[j - 1] : prev_last;
            if (pos < deg && (pos == 0 || a[j] != prev)) hm |= 1u << j;
        }
        // the first head at or after the next lane (suffix minimum over lanes), else deg
        int first = hm ? lane * 8 + __ffs(hm) - 1 : deg;
        int after = deg;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int o = __shfl_down_sync(kFull, first, off);
            if (lane + off < 32) first = min(first, o);
        }
        after = __shfl_down_sync(kFull, first, 1);  // minimum over lanes > this one
        if (lane == 31) after = deg;
        // heads before this lane, for the runs' ranks
        const int nh = __popc(hm);
        int before = nh;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int o = __shfl_up_sync(kFull, before, off);
            if (lane >= off) before += o;
        }
        before -= nh;
        // this lane's runs: count = next head position - head position
        Sum5 part = sum5_empty();
        int cnt[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            cnt[j] = 0;
            if (hm & (1u << j)) {
                const unsigned later = hm & ~((2u << j) - 1u);
                const int next = later ? lane * 8 + __ffs(later) - 1 : after;
                cnt[j] = next - (lane * 8 + j);
                part.d += 1;
                sum5_observe(part, (int)a[j], cnt[j]);
            }
        }
        const Sum5 sm = sum5_warp(part);
        // ranks of the smallest and largest candidate: heads before them (labels ascend)
        int rmin = 0, rmax = sm.d - 1;
        if (sm.k > 1) {
            int lo = 0, hi = 0;
#pragma unroll
            for (int j = 0; j < 8; ++j)
                if (hm & (1u << j)) {
                    lo += (int)a[j] < sm.mn;
                    hi += (int)a[j] < sm.mx;
                }
            rmin = __reduce_add_sync(kFull, lo);
            rmax = __reduce_add_sync(kFull, hi);
            if (sm.k > 2) {  // spill the runs in label order
                int32_t *rl = p.run_lab + (o0 - p.nbr_shift);
                uint16_t *rc = p.run_cnt + (o0 - p.nbr_shift);
                int r = before;
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    if (hm & (1u << j)) {
                        rl[r] = (int32_t)a[j];
                        rc[r] = (uint16_t)cnt[j];
                        ++r;
                    }
            }
        }
        const bool tied = lane == 0 && finish_counted(p, v, sm, rmin, rmax, changes);
        tb.append(tied, v, p.tied_mid, &p.ctl->tied_mid);
        __syncwarp();
    }
    tb.flush(p.tied_mid, &p.ctl->tied_mid);
    flush_changes(changes, p.ctl);
}

// Block-wide Sum5 / pair reductions with one barrier each: warps publish partials, then
// every warp folds all of them.  Buffers hold one entry per warp (W = THREADS / 32): buf
// is [5][W], buf2 [2][W].  The kernel's end-of-vertex barrier orders a buffer's reads
// before its next writes.
template <int THREADS>
struct BlockRed5 {
    static constexpr int W = THREADS / 32;
    int *buf;   // [5][W]
    int *buf2;  // [2][W]
    __device__ Sum5 reduce(Sum5 s) const
    {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        s = sum5_warp(s);
        if (lane == 0) {
            buf[0 * W + warp] = s.d;
            buf[1 * W + warp] = s.W;
            buf[2 * W + warp] = s.k;
            buf[3 * W + warp] = s.mn;
            buf[4 * W + warp] = s.mx;
        }
        __syncthreads();
        Sum5 t = sum5_empty();
        if (lane < W) t = Sum5{buf[lane], buf[W + lane], buf[2 * W + lane], buf[3 * W + lane], buf[4 * W + lane]};
        return sum5_warp(t);
    }
    __device__ void reduce2(int &a, int &b) const
    {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        a = __reduce_add_sync(kFull, a);
        b = __reduce_add_sync(kFull, b);
        if (lane == 0) {
            buf2[warp] = a;
            buf2[W + warp] = b;
        }
        __syncthreads();
        const int x = lane < W ? buf2[lane] : 0, y = lane < W ? buf2[W + lane] : 0;
        a = __reduce_add_sync(kFull, x);
        b = __reduce_add_sync(kFull, y);
    }
};

// ----- bulk copies into shared memory (cp.async.bulk) with mbarrier completion -----
__device__ __forceinline__ uint32_t smem_u32(const void *ptr)
{
    return (uint32_t)__cvta_generic_to_shared(ptr);
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// One thread: expect `bytes` on the barrier, then copy them global -> shared (both
// addresses 16-byte aligned, bytes a multiple of 16).
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, unsigned long long *bar)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for the barrier's phase `parity`; false after kStageSpinLimit polls.
constexpr long long kStageSpinLimit = 1ll << 22;
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, uint32_t parity)
{
    for (long long i = 0; i < kStageSpinLimit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// One CTA of THREADS threads per vertex of degree <= SLOTS/2 (table of SLOTS 64-bit
// slots in dynamic shared memory), for a range of the degree-sorted mid list.
//
// Software pipelining across the CTA's vertices: the next vertex's head (CtaHead) and, in
// CTAs of up to 256 threads that do not stage, its first PER * THREADS neighbour IDs are
// loaded into registers while the current vertex's labels are gathered and counted, so a
// vertex starts with its label gathers instead of three dependent global round trips.
//
// STAGE: the next vertex's neighbour IDs are copied into a shared-memory stage by one
// bulk copy (cp.async.bulk, completion on an mbarrier) while the current vertex is
// counted, so the IDs are read from shared memory and no thread waits on their global
// loads.  The copy starts at the 16-byte boundary below the vertex's first entry and
// ends at the one above its last (the neighbour buffers carry 16 bytes of padding).  A
// wait that runs out (it cannot for a valid address) sets kErrStage, waits for that copy
// once more before the CTA exits and counts the remaining vertices from global loads.
// Not in frontier mode (clean vertices need no IDs).
template <int THREADS, int SLOTS, bool STAGE = false>
__global__ void __launch_bounds__(THREADS, THREADS >= 1024 ? 1 : THREADS >= 512 ? 2 : THREADS >= 256 ? 4
                                           : THREADS >= 128 ? 8 : 16)
    count_cta_kernel(PipeArgs p, int which)
{
    extern __shared__ __align__(16) unsigned long long cta_tab[];
    __shared__ int red[5 * (THREADS / 32)], red2[2 * (THREADS / 32)];
    __shared__ int sctr;
    __shared__ __align__(8) unsigned long long stage_bar;
    __shared__ int stage_ok;
    __shared__ int32_t ctbuf[kCtaBuf];  // thread 0's tied vertices
    __shared__ int ctn;
    if (!ctl_active(p.ctl)) return;
    if (threadIdx.x == 0) ctn = 0;  // ordered before thread 0's own uses
    // ranges of the degree-sorted mid list: 0 [pos1, pos_a), 1 [pos_a, pos2), 2 [pos2, pos_b),
    // 3 [pos_b, end); with a narrow cut c, 0 is [max(pos1, c), pos_a) and 4 [pos1, min(pos_a, c))
    const DispatchState &ds = *p.disp;
    int first = which == 0 ? ds.pos1 : which == 1 ? ds.pos_a : which == 2 ? ds.pos2 : which == 3 ? ds.pos_b : ds.pos1;
    int end = which == 0 ? ds.pos_a : which == 1 ? ds.pos2 : which == 2 ? ds.pos_b : which == 3 ? p.nmid_s + p.nmid_l + p.nmid_x
                                                                                            : ds.pos_a;
    if (p.narrow_cut >= 0) {
        if (which == 0) first = max(first, p.narrow_cut);
        if (which == 4) end = min(end, p.narrow_cut);
    }
    const int count = end - first;
    const bool fr = frontier_on(p);
    const int tid = threadIdx.x;
    const BlockRed5<THREADS> br{red, red2};
    unsigned long long changes = 0;
    for (int s = tid; s < SLOTS; s += THREADS) cta_tab[s] = 0ull;
    uint32_t gen = 0;
    // staging: thread 0 copies the neighbour IDs of list entry i into the stage
    const bool staged = STAGE && !fr;
    int32_t *stage = reinterpret_cast<int32_t *>(cta_tab + SLOTS);
    uint32_t parity = 0, lost_parity = 2;
    auto stage_issue = [&](int i) {
        if (i >= count) return;
        const int vn = p.mid_v[first + i];
        const int64_t a = __ldg(&p.off[vn]) - p.nbr_shift;
        const int64_t b = __ldg(&p.off[vn + 1]) - p.nbr_shift;
        const int64_t a4 = a & ~(int64_t)3, b4 = (b + 3) & ~(int64_t)3;
        // the proxy fence orders the threads' reads of the stage before the copy's writes
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        bulk_load(stage, p.nbr + a4, (uint32_t)(4 * (b4 - a4)), &stage_bar);
    };
    if (staged && tid == 0) {
        mbar_init(&stage_bar, 1);
        stage_ok = 1;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        stage_issue(blockIdx.x);
    }
    __syncthreads();
    constexpr int PER = 8;  // a thread's loads in flight together per round
    // The first round of a vertex's neighbour IDs, loaded one vertex ahead (not staged; CTAs
    // of up to 256 threads: in the 512- and 1024-thread CTAs the extra registers cost the
    // gathers more than the early IDs save).
    constexpr bool kAhead = THREADS <= 256;
    const bool ahead = kAhead && !staged;
    auto ids_ahead = [&](int (&nb)[PER], const CtaHead &h) {
#pragma unroll
        for (int u = 0; u < PER; ++u) {
            const int e = tid + u * THREADS;
            nb[u] = (ahead && h.v >= 0 && h.dirty && e < h.deg) ? ld_nbr(&p.nbr[h.o0 + e - p.nbr_shift]) : -1;
        }
    };
    CtaHead nxt = cta_head(p, first, blockIdx.x, count, fr);
    int nbn[PER];
    ids_ahead(nbn, nxt);
    for (int i = blockIdx.x; i < count; i += gridDim.x) {
        const CtaHead h = nxt;
        const int v = h.v;
        int nb0[PER];
#pragma unroll
        for (int u = 0; u < PER; ++u) nb0[u] = nbn[u];
        nxt = cta_head(p, first, i + gridDim.x, count, fr);
        if (!h.dirty) {
            if (tid == 0 && carry_clean(p, v)) tbuf_append(ctbuf, &ctn, v, p.tied_mid, &p.ctl->tied_mid);
            ids_ahead(nbn, nxt);
            continue;
        }
        if (++gen > kT64GenMax) {
            for (int s = tid; s < SLOTS; s += THREADS) cta_tab[s] = 0ull;
            __syncthreads();
            gen = 1;
        }
        const int64_t o0 = h.o0;
        const int deg = h.deg;
        // this vertex's IDs in the stage (the copy was issued one vertex earlier)
        bool from_stage = false;
        if (staged && stage_ok) {
            const bool got = mbar_wait(&stage_bar, parity);
            if (!got) stage_ok = 0;  // any thread that gave up turns staging off for the CTA
            __syncthreads();
            from_stage = stage_ok != 0;
            if (!from_stage) {
                lost_parity = parity;  // the copy still in flight completes this phase
                if (tid == 0) atomicOr(&p.ctl->err, kErrStage);
            }
            parity ^= 1u;
        }
        const int skip = (int)((o0 - p.nbr_shift) & 3);
        // probe range: the whole table up to 4 slots per neighbour (load <= 1/4 where the
        // table allows, at most 1/2): the longest probe of a warp's inserts sets its pace
        const uint32_t cap = (uint32_t)min(SLOTS, 4 * pad32(deg));
        // warp-aggregated inserts when the vertex had at most half as many distinct labels
        // as neighbours in the previous iteration (agg_mode 0); always (1); never (2)
        const int mode = p.disp->agg_mode;
        const bool agg = mode == 1 || (mode == 0 && 2 * h.dcnt <= deg);
        Sum5 obs = sum5_empty();
        // gather in rounds of PER loads per thread in flight together; the first round's IDs
        // are in registers already (or in the stage)
        for (int base = 0; base < deg; base += THREADS * PER) {
            int nb[PER];
#pragma unroll
            for (int u = 0; u < PER; ++u) {
                const int e = base + tid + u * THREADS;
                if (base == 0 && ahead) nb[u] = nb0[u];
                else nb[u] = (e < deg) ? (from_stage ? stage[skip + e] : ld_nbr(&p.nbr[o0 + e - p.nbr_shift])) : -1;
            }
            uint32_t lb[PER];
#pragma unroll
            for (int u = 0; u < PER; ++u) lb[u] = (nb[u] >= 0) ? (uint32_t)ld_label(&p.lab_in[nb[u]]) : kEmpty;
#pragma unroll
            for (int u = 0; u < PER; ++u) {
                if (base + u * THREADS >= deg) break;  // block-uniform
                t64_insert_row(cta_tab, cap, gen, lb[u], agg, obs);
            }
        }
        // the next vertex's first IDs (its head has arrived during the gathers and inserts)
        // load while this vertex is reduced, ranked, spilled and finished
        ids_ahead(nbn, nxt);
        // the reduction's barrier also completes the table for the rank and spill passes,
        // and every thread's reads of the stage: the next vertex's copy may start
        const Sum5 s = br.reduce(obs);
        if (from_stage && tid == 0) stage_issue(i + gridDim.x);
        int rmin = 0, rmax = s.d - 1;  // when every distinct label is a candidate
        if (s.k > 1) {
            if (s.k < s.d) {
                t64_ranks(cta_tab, (int)cap, tid, THREADS, gen, s.mn, s.mx, rmin, rmax);
                br.reduce2(rmin, rmax);
            }
            if (s.k > 2) {
                if (tid == 0) sctr = 0;
                __syncthreads();
                t64_spill(cta_tab, (int)cap, tid, THREADS, gen, p.run_lab + (o0 - p.nbr_shift),
                          p.run_cnt + (o0 - p.nbr_shift), &sctr);
            }
        }
        if (tid == 0 && finish_counted(p, v, s, rmin, rmax, changes, h.old))
            tbuf_append(ctbuf, &ctn, v, p.tied_mid, &p.ctl->tied_mid);
        __syncthreads();
    }
    if (tid == 0) tbuf_flush(ctbuf, &ctn, p.tied_mid, &p.ctl->tied_mid);
    // a copy that a wait gave up on still lands in this CTA's shared memory: wait for it
    // (bounded) before the CTA exits
    if (staged && lost_parity < 2) (void)mbar_wait(&stage_bar, lost_parity);
    flush_changes(changes, p.ctl);
}

// One CTA per hub partition (grid-stride over the scope's partitions): count the
// partition's (label, count) pairs in a shared-memory table sized to them (all pairs of a
// label fall in one partition, so its count is complete here), fold the counts each
// insert observes into the partition's summary, append its distinct labels to the hub's
// distinct list and reset the partition's fill for the next scope.
//
// Three shapes: 1024 threads with 16384-slot tables (one CTA per SM), 512 threads with
// 8192-slot tables (three per SM) for partitions of half the size (hub_part_shift 1), and
// 256 threads with 4096-slot tables (six per SM) for a quarter (hub_part_shift >= 2).
template <int kT, int TAB>
__global__ void __launch_bounds__(kT, kT >= 1024 ? 1 : kT >= 512 ? 3 : 6) hub_count_kernel(IterArgs p)
{
    extern __shared__ __align__(16) uint32_t hub_tab[];  // TAB keys, then TAB counts
    __shared__ int red[5 * (kT / 32)], red2[2 * (kT / 32)];
    __shared__ int sfill, sbase, sctr;
    if (!ctl_active(p.ctl)) return;
    uint32_t *key = hub_tab;
    uint32_t *cnt = hub_tab + TAB;
    const BlockRed5<kT> br{red, red2};
    const int tid = threadIdx.x, lane = tid & 31;
    for (int x = blockIdx.x; x < p.nparts; x += gridDim.x) {
        const int gp = p.q0 + x;
        const int bi = p.part_big[gp];
        const int pcap = p.hub_pcap[bi];
        if (tid == 0) sfill = min(p.pfill[gp], pcap);
        __syncthreads();
        const int fill = sfill;
        uint32_t tcap = 64;  // load <= 1/2 when every pair is a distinct label
        while (tcap < 2u * (uint32_t)fill && tcap < (uint32_t)TAB) tcap <<= 1;
        for (int s2 = tid; s2 < (int)tcap; s2 += kT) {
            key[s2] = kEmpty;
            cnt[s2] = 0;
        }
        __syncthreads();
        const unsigned long long *src = p.pairs + p.hub_pbase[bi] + (int64_t)(gp - p.hub_p0[bi]) * pcap;
        Sum5 obs = sum5_empty();
        constexpr int PER = 8;  // a thread's pair loads in flight together
        for (int j0 = 0; j0 < fill; j0 += kT * PER) {
            unsigned long long xs[PER];
#pragma unroll
            for (int u = 0; u < PER; ++u) {
                const int j = j0 + tid + u * kT;
                xs[u] = j < fill ? src[j] : ~0ull;  // a pair is never all ones (labels < 2^31)
            }
#pragma unroll
            for (int u = 0; u < PER; ++u) {
                if (xs[u] == ~0ull) continue;
                const uint32_t L = (uint32_t)(xs[u] >> 32), c = (uint32_t)xs[u];
                uint32_t h = hslot(L, tcap);
                // a full table (more distinct labels than slots: pairs repeating few labels
                // made it small) ends the probe after one round and flags the run
                for (uint32_t probe = 0;; ++probe) {
                    if (probe == tcap) {
                        atomicOr(&p.ctl->err, kErrHubOverflow);
                        break;
                    }
                    const uint32_t prev = atomicCAS(&key[h], kEmpty, L);
                    if (prev == kEmpty || prev == L) {
                        obs.d += prev == kEmpty;
                        sum5_observe(obs, (int)L, (int)(atomicAdd(&cnt[h], c) + c));
                        break;
                    }
                    h = (h + 1 == tcap) ? 0 : h + 1;
                }
            }
        }
        const Sum5 sm = br.reduce(obs);  // its barrier also completes the table
        if (tid == 0) {
            sbase = sm.d ? atomicAdd(&p.bstat[bi].d, sm.d) : 0;
            sctr = 0;
            p.psum[gp] = make_int4(sm.W, sm.k, sm.mn, sm.mx);
            p.pfill[gp] = 0;
        }
        __syncthreads();
        unsigned long long *list = p.big_list + p.big_ooff[bi] + sbase;
        for (int s0 = 0; s0 < (int)tcap; s0 += kT) {
            const int s2 = s0 + tid;
            const bool used = s2 < (int)tcap && key[s2] != kEmpty;
            const unsigned m = __ballot_sync(kFull, used);
            if (!m) continue;
            int at = 0;
            if (lane == __ffs(m) - 1) at = atomicAdd(&sctr, __popc(m));
            at = __shfl_sync(kFull, at, __ffs(m) - 1) + __popc(m & ((1u << lane) - 1));
            if (used) list[at] = ((unsigned long long)key[s2] << 32) | cnt[s2];
        }
        __syncthreads();
    }
}

// Measurement probe: one pass over the CSR that streams every neighbour ID and gathers its
// label with the loads the counting kernels use (streaming IDs, evict-last label gathers),
// 8 entries per thread in flight, and nothing else; the block XORs the labels into one
// word.  Its time is the floor of any update that gathers every neighbour's label.
__global__ void __launch_bounds__(kTB) gather_probe_kernel(const int32_t *nbr, int64_t m, const int32_t *lab,
                                                           unsigned long long *acc)
{
    constexpr int PER = 8;
    uint32_t x = 0;
    const int64_t stride = (int64_t)gridDim.x * kTB * PER;
    for (int64_t base = (int64_t)blockIdx.x * kTB * PER + threadIdx.x; base < m; base += stride) {
        int nb[PER];
#pragma unroll
        for (int u = 0; u < PER; ++u) {
            const int64_t e = base + (int64_t)u * kTB;
            nb[u] = e < m ? ld_nbr(&nbr[e]) : -1;
        }
#pragma unroll
        for (int u = 0; u < PER; ++u) x ^= nb[u] >= 0 ? (uint32_t)ld_label(&lab[nb[u]]) : 0u;
    }
    x = __reduce_xor_sync(kFull, x);
    if ((threadIdx.x & 31) == 0 && x) atomicXor(acc, (unsigned long long)x);
}

__global__ void big_dcnt_kernel(IterArgs a, int32_t *dcnt)
{
    if (!ctl_active(a.ctl)) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nbig; i += gridDim.x * blockDim.x)
        dcnt[a.big_v[a.b0 + i]] = a.bstat[a.b0 + i].d;
}

// ---------------------------------------------------------------------------
// scan of distinct counts -> run bases (reduce, spine, apply)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kTB) scan_reduce_kernel(PipeArgs p)
{
    __shared__ long long ws[kNW];
    if (!ctl_active(p.ctl)) return;
    const int64_t b0 = p.v0 + (int64_t)blockIdx.x * kScanBlock;
    long long s = 0;
    for (int i = threadIdx.x; i < kScanBlock; i += kTB) {
        const int64_t v = b0 + i;
        if (v < p.v1) s += p.dcnt[v];
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(kFull, s, off);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long t = 0;
        for (int w = 0; w < kNW; ++w) t += ws[w];
        p.bsum[blockIdx.x] = t;
    }
}

// one CTA: exclusive scan of the block sums in place; total -> ctl->N
__global__ void __launch_bounds__(kTB) scan_spine_kernel(PipeArgs p, int nblocks)
{
    __shared__ long long ws[kNW];
    __shared__ long long carry;
    if (!ctl_active(p.ctl)) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nblocks; base += kTB) {
        const int i = base + threadIdx.x;
        const long long x = i < nblocks ? p.bsum[i] : 0;
        long long incl = x;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const long long o = __shfl_up_sync(kFull, incl, off);
            if (lane >= off) incl += o;
        }
        if (lane == 31) ws[warp] = incl;
        __syncthreads();
        long long wb = 0, tot = 0;
        for (int w = 0; w < kNW; ++w) {
            if (w < warp) wb += ws[w];
            tot += ws[w];
        }
        const long long c = carry;
        if (i < nblocks) p.bsum[i] = c + wb + incl - x;
        __syncthreads();
        if (threadIdx.x == 0) carry = c + tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) p.ctl->N = carry;
}

__global__ void __launch_bounds__(kTB) scan_apply_kernel(PipeArgs p)
{
    __shared__ long long ws[kNW];
    if (!ctl_active(p.ctl)) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int PER = kScanBlock / kTB;
    const int64_t b0 = p.v0 + (int64_t)blockIdx.x * kScanBlock + (int64_t)threadIdx.x * PER;
    int x[PER];
    long long s = 0;
#pragma unroll
    for (int u = 0; u < PER; ++u) {
        x[u] = (b0 + u < p.v1) ? p.dcnt[b0 + u] : 0;
        s += x[u];
    }
    long long incl = s;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const long long o = __shfl_up_sync(kFull, incl, off);
        if (lane >= off) incl += o;
    }
    if (lane == 31) ws[warp] = incl;
    __syncthreads();
    long long wb = 0;
    for (int w = 0; w < warp; ++w) wb += ws[w];
    long long run = p.bsum[blockIdx.x] + wb + incl - s;
#pragma unroll
    for (int u = 0; u < PER; ++u) {
        if (b0 + u < p.v1) p.runbase[b0 + u] = run;
        run += x[u];
    }
}

// ---------------------------------------------------------------------------
// resolution of tied vertices
// ---------------------------------------------------------------------------

// Sorted spilled runs of a small vertex, scanned by one thread.
struct SpillRunQuery {
    const int32_t *lab;
    const uint16_t *cnt;
    int d, W;
    __device__ int first_ge(int64_t x) const
    {
        for (int r = (int)(x < 0 ? 0 : x); r < d; ++r)
            if ((int)cnt[r] == W) return r;
        return -1;
    }
    __device__ int last_lt(int64_t y) const
    {
        for (int r = (int)(y < d ? y : d) - 1; r >= 0; --r)
            if ((int)cnt[r] == W) return r;
        return -1;
    }
    __device__ int tile_pick(int64_t) const { return -1; }  // d <= 32 never spans a tile
};

__global__ void __launch_bounds__(kTB) resolve_small_kernel(PipeArgs p)
{
    if (!ctl_active(p.ctl)) return;
    const int nt = *((volatile int *)&p.ctl->tied_small);
    unsigned long long changes = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nt; i += gridDim.x * blockDim.x) {
        const int v = p.tied_small[i];
        const int kw = p.sm_kw[v], rr = p.sm_r[v];
        const int k = kw & 0xFFFF, W = kw >> 16, rmin = rr & 0xFFFF, rmax = rr >> 16;
        const int d = p.dcnt[v];
        const RunScope rs = run_scope(p, v);
        const long long a = rs.a, N = rs.N;
        const bool is_last = rs.is_last;
        SummaryQuery q(k, d, rmin, rmax);
        int r = resolve_rank(a, d, N, is_last, q);
        int32_t nl;
        if (!q.fail && r == rmin) {
            nl = p.sm_c0[v];
        } else if (!q.fail && r == rmax) {
            nl = p.sm_c1[v];
        } else {
            const int64_t e = __ldg(&p.off[v]) - p.nbr_shift;
            SpillRunQuery sq{p.run_lab + e, p.run_cnt + e, d, W};
            if (q.fail) r = resolve_rank(a, d, N, is_last, sq);
            nl = p.run_lab[e + r];
        }
        const int32_t old = __ldg(&p.lab_in[v]);
        p.lab_out[v] = nl;
        count_change(changes, nl, old);
        note_change(p, v, nl, old);
    }
    flush_changes(changes, p.ctl);
}

// Unsorted spilled (label, count) entries of a mid/large vertex, one warp.
struct SpillTableQuery {
    const int32_t *lab;
    const uint16_t *cnt;
    int d, W, rmin, rmax;
    int *hist;
    int lane;
    __device__ uint32_t select(int x)
    {
        uint32_t prefix = 0;
        int remaining = x;
        for (int shift = 24; shift >= 0; shift -= 8) {
            for (int b = lane; b < 256; b += 32) hist[b] = 0;
            __syncwarp();
            const uint32_t hi_mask = (shift == 24) ? 0u : (0xFFFFFFFFu << (shift + 8));
            for (int i = lane; i < d; i += 32) {
                const uint32_t k = (uint32_t)lab[i];
                if ((k & hi_mask) == (prefix & hi_mask)) atomicAdd(&hist[(k >> shift) & 255], 1);
            }
            __syncwarp();
            int c[8];
            int local = 0;
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                c[i] = hist[lane * 8 + i];
                local += c[i];
            }
            int incl = local;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const int o = __shfl_up_sync(kFull, incl, off);
                if (lane >= off) incl += o;
            }
            const int excl = incl - local;
            const unsigned who = __ballot_sync(kFull, remaining >= excl && remaining < incl);
            const int src = who ? (__ffs(who) - 1) : 31;
            int digit = 0, before = 0;
            if (lane == src) {
                int acc = excl, i = 0;
                for (; i < 7; ++i) {
                    if (remaining < acc + c[i]) break;
                    acc += c[i];
                }
                digit = lane * 8 + i;
                before = acc;
            }
            digit = __shfl_sync(kFull, digit, src);
            before = __shfl_sync(kFull, before, src);
            prefix |= (uint32_t)digit << shift;
            remaining -= before;
            __syncwarp();
        }
        return prefix;
    }
    __device__ int rank_of(uint32_t c) const
    {
        int n = 0;
        for (int i = lane; i < d; i += 32) n += (uint32_t)lab[i] < c;
        return __reduce_add_sync(kFull, n);
    }
    __device__ int first_ge(int64_t x)
    {
        if (x >= d) return -1;
        if (x <= rmin) return rmin;
        const uint32_t L = select((int)x);
        uint32_t best = kEmpty;
        for (int i = lane; i < d; i += 32) {
            const uint32_t k = (uint32_t)lab[i];
            if ((int)cnt[i] == W && k >= L && k < best) best = k;
        }
        best = __reduce_min_sync(kFull, best);
        return best == kEmpty ? -1 : rank_of(best);
    }
    __device__ int last_lt(int64_t y)
    {
        if (y > rmax) return rmax;
        if (y <= rmin) return -1;
        const uint32_t L = select((int)y);
        int best = -1;
        for (int i = lane; i < d; i += 32) {
            const uint32_t k = (uint32_t)lab[i];
            if ((int)cnt[i] == W && k < L && (int)k > best) best = (int)k;
        }
        best = __reduce_max_sync(kFull, best);
        return best < 0 ? -1 : rank_of((uint32_t)best);
    }
    // Among candidates of rank in [lo, lo + kTile) (a whole tile), the one of highest
    // tile_priority; ranks by full passes (only vertices of > 4352 distinct labels
    // whose last tile holds no candidate get here).
    __device__ int tile_pick(int64_t lo)
    {
        int best = -1, bestr = -1;
        for (int i0 = 0; i0 < d; i0 += 32) {
            const int i = i0 + lane;
            const bool c = i < d && (int)cnt[i] == W;
            unsigned m = __ballot_sync(kFull, c);
            while (m) {
                const int src = __ffs(m) - 1;
                m &= m - 1;
                const uint32_t lab_c = (uint32_t)__shfl_sync(kFull, i < d ? lab[i] : 0, src);
                const int r = rank_of(lab_c);
                if (r >= lo && r < lo + kTile && tile_priority(r - lo) > best) {
                    best = tile_priority(r - lo);
                    bestr = r;
                }
            }
        }
        return bestr;
    }
};

__global__ void __launch_bounds__(kTB) resolve_mid_kernel(PipeArgs p)
{
    __shared__ int hist[kNW][256];
    if (!ctl_active(p.ctl)) return;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int nt = *((volatile int *)&p.ctl->tied_mid);
    unsigned long long changes = 0;
    for (int i = blockIdx.x * kNW + w; i < nt; i += gridDim.x * kNW) {
        const int v = p.tied_mid[i];
        const int kw = p.sm_kw[v], rr = p.sm_r[v];
        const int k = kw & 0xFFFF, W = kw >> 16, rmin = rr & 0xFFFF, rmax = rr >> 16;
        const int d = p.dcnt[v];
        const RunScope rs = run_scope(p, v);
        const long long a = rs.a, N = rs.N;
        const bool is_last = rs.is_last;
        SummaryQuery q(k, d, rmin, rmax);
        int r = resolve_rank(a, d, N, is_last, q);
        int32_t nl;
        if (!q.fail && r == rmin) {
            nl = p.sm_c0[v];
        } else if (!q.fail && r == rmax) {
            nl = p.sm_c1[v];
        } else {
            const int64_t e = __ldg(&p.off[v]) - p.nbr_shift;
            SpillTableQuery tq{p.run_lab + e, p.run_cnt + e, d, W, rmin, rmax, hist[w], lane};
            if (q.fail) r = resolve_rank(a, d, N, is_last, tq);
            nl = (r == rmin) ? p.sm_c0[v] : (r == rmax) ? p.sm_c1[v] : (int32_t)tq.select(r);
        }
        if (lane == 0) {
            const int32_t old = __ldg(&p.lab_in[v]);
            p.lab_out[v] = nl;
            count_change(changes, nl, old);
            note_change(p, v, nl, old);
        }
    }
    flush_changes(changes, p.ctl);
}

// Frontier: mark the neighbours of every vertex that changed in the previous iteration
// (the graph is symmetric, so they are exactly the vertices whose neighbour labels
// changed).  One warp per changed vertex.  When the dispatcher chose a full recount for
// this iteration (e.g. most labels changed, so marking would touch most of the graph)
// nothing is marked and ctl->frontier_off tells the count kernels.
__global__ void __launch_bounds__(kTB) mark_dirty_kernel(const int64_t *off, const int32_t *nbr,
                                                         const int32_t *changed, const DispatchState *disp, Ctl *ctl,
                                                         uint8_t *dirty)
{
    const int lane = threadIdx.x & 31;
    const int nc = *((volatile int *)&ctl->changed_n);
    const bool dense = !disp->frontier;
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->frontier_off = dense ? 1 : 0;
    if (dense) return;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < nc; i += (gridDim.x * blockDim.x) >> 5) {
        const int u = changed[i];
        const int64_t e0 = off[u], e1 = off[u + 1];
        for (int64_t e = e0 + lane; e < e1; e += 32) dirty[nbr[e]] = 1;
    }
}

// ---------------------------------------------------------------------------
// first iteration on strictly increasing adjacency lists
// ---------------------------------------------------------------------------
//
// With labels = vertex IDs (the reference's initialize_labels, dpp/kernel.cuh:15-22) and
// every adjacency list strictly increasing, each vertex's neighbour labels are distinct
// and already sorted: d = degree, every run has count 1 (all are candidates), the run
// base of v is offsets[v] and the scope holds N = m runs.  The winning run r follows
// from the closed form alone and its label is the neighbour ID at offsets[v] + r.

// Every distinct label is a candidate (k == d).
struct AllCandidates {
    int64_t d;
    __device__ int first_ge(int64_t x) const { return x < d ? (int)(x < 0 ? 0 : x) : -1; }
    __device__ int last_lt(int64_t y) const { return y > 0 ? (int)((y < d ? y : d) - 1) : -1; }
    __device__ int tile_pick(int64_t lo) const { return (int)(lo + kTile - 1); }
};

__global__ void __launch_bounds__(kTB) first_iteration_kernel(PipeArgs p, int64_t n, int64_t m)
{
    if (!ctl_active(p.ctl)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) p.ctl->N = m;  // one run per CSR entry
    unsigned long long changes = 0;
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const int64_t o0 = __ldg(&p.off[v]);
        const int64_t deg = __ldg(&p.off[v + 1]) - o0;
        const int32_t old = __ldg(&p.lab_in[v]);
        int32_t nl = old;
        if (deg > 0) {
            AllCandidates q{deg};
            if (!p.g_v0) {
                const int r = resolve_rank(o0, deg, m, v == p.last_v, q);
                nl = __ldg(&p.nbr[o0 + r]);
            } else {  // graph-local run positions and labels
                const int g = __ldg(&p.gid[v]);
                const int64_t vg = p.g_v0[g], e0 = __ldg(&p.off[vg]), e1 = __ldg(&p.off[p.g_v0[g + 1]]);
                const int r = resolve_rank(o0 - e0, deg, e1 - e0, v == p.g_last[g], q);
                nl = (int32_t)(__ldg(&p.nbr[o0 + r]) - vg);
            }
        }
        p.lab_out[v] = nl;
        p.dcnt[v] = (int32_t)deg;  // every neighbour label distinct (insert-aggregation hint)
        count_change(changes, nl, old);
        note_change(p, (int32_t)v, nl, old);
    }
    flush_changes(changes, p.ctl);
}

// Setup checks without the symmetry checksum, as two streaming passes:
//   csr_scan_kernel:     out[3] += neighbour IDs outside [0, n); out[0] += entries e >= 1
//                        with nbr[e] <= nbr[e-1] (all descents, row boundaries included);
//   row_start_kernel:    out[4] += those descents that sit at a row start (e = offsets[v]
//                        of a vertex with neighbours), which do not count.
// Adjacency lists are strictly increasing when out[0] == out[4].
__global__ void __launch_bounds__(kTB) csr_scan_kernel(const int32_t *nbr, int64_t m, int64_t n,
                                                       unsigned long long *out)
{
    unsigned long long desc = 0, outside = 0;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t u = __ldg(&nbr[e]);
        outside += (u < 0 || u >= n);
        if (e > 0) desc += (u <= __ldg(&nbr[e - 1]));
    }
    desc = __reduce_add_sync(kFull, (unsigned)desc);
    outside = __reduce_add_sync(kFull, (unsigned)outside);
    if ((threadIdx.x & 31) == 0) {
        if (desc) atomicAdd(&out[0], desc);
        if (outside) atomicAdd(&out[3], outside);
    }
}

__global__ void __launch_bounds__(kTB) row_start_kernel(const int64_t *off, const int32_t *nbr, int64_t n,
                                                        unsigned long long *out)
{
    unsigned long long b = 0;
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = off[v];
        if (e > 0 && off[v + 1] > e) b += (__ldg(&nbr[e]) <= __ldg(&nbr[e - 1]));
    }
    b = __reduce_add_sync(kFull, (unsigned)b);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(&out[4], b);
}

// One pass over the resident CSR at setup (warp per 32 consecutive vertices, lanes over
// the warp's edge range, row of each edge by a shuffle binary search over the 33 offsets):
//   out[3] += neighbour IDs outside [0, n) (the graph is rejected);
//   out[0] += adjacent entries of one row that are not strictly increasing
//             (0 enables the first-iteration shortcut);
//   out[1], out[2] += sum over entries (v, u) of g(v)k(u) - g(u)k(v) (mod 2^64) for two
//             hash pairs g, k.  The form is antisymmetric, so every graph whose edge
//             multiset is symmetric sums to 0 in both; an asymmetric one does so only by a
//             hash collision (about 2^-64 per sum).  Both 0 enables the frontier, whose
//             dirty marking pushes along out-edges.  Computed only when want_sym.
__device__ __forceinline__ uint64_t adj_hash(uint64_t x, uint64_t salt)
{
    return splitmix64_mix(x * 0x9E3779B97F4A7C15ull + salt);
}

__global__ void __launch_bounds__(kTB) adjacency_check_kernel(const int64_t *off, const int32_t *nbr, int64_t n,
                                                              int want_sym, unsigned long long *out)
{
    const int lane = threadIdx.x & 31;
    const int64_t nwb = (n + 31) >> 5;
    unsigned long long desc = 0, s1 = 0, s2 = 0, outside = 0;
    for (int64_t wb = (int64_t)(blockIdx.x * blockDim.x + threadIdx.x) >> 5; wb < nwb;
         wb += (int64_t)(gridDim.x * blockDim.x) >> 5) {
        const int64_t vb = wb << 5;
        const int64_t o = off[min(vb + lane, n)];  // lanes past n hold off[n]
        const int64_t oend = off[min(vb + 32, n)];
        const int64_t e_begin = __shfl_sync(kFull, o, 0);
        int32_t carry = 0;  // last entry of the previous chunk
        for (int64_t c = e_begin; c < oend; c += 32) {
            const int64_t e = c + lane;
            int r = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1) {
                const int64_t oc = __shfl_sync(kFull, o, r + step);
                if (oc <= e) r += step;
            }
            const bool valid = e < oend;
            const int32_t u = valid ? __ldg(&nbr[e]) : 0;
            int32_t prev = __shfl_up_sync(kFull, u, 1);
            if (lane == 0) prev = carry;
            carry = __shfl_sync(kFull, u, 31);
            const int64_t row_start = __shfl_sync(kFull, o, r);
            if (valid) {
                if (e != row_start && u <= prev) ++desc;
                outside += (u < 0 || u >= n);
            }
            if (valid && want_sym) {
                const uint64_t v = (uint64_t)(vb + r);
                s1 += adj_hash(v, 0x1234567ull) * adj_hash((uint64_t)u, 0xABCDEF1ull) -
                      adj_hash((uint64_t)u, 0x1234567ull) * adj_hash(v, 0xABCDEF1ull);
                s2 += adj_hash(v, 0x7777777ull) * adj_hash((uint64_t)u, 0x3141592ull) -
                      adj_hash((uint64_t)u, 0x7777777ull) * adj_hash(v, 0x3141592ull);
            }
        }
    }
#pragma unroll
    for (int sh = 16; sh > 0; sh >>= 1) {
        desc += __shfl_xor_sync(kFull, desc, sh);
        s1 += __shfl_xor_sync(kFull, s1, sh);
        s2 += __shfl_xor_sync(kFull, s2, sh);
        outside += __shfl_xor_sync(kFull, outside, sh);
    }
    if (lane == 0) {
        if (desc) atomicAdd(&out[0], desc);
        if (want_sym) {
            atomicAdd(&out[1], s1);
            atomicAdd(&out[2], s2);
        }
        if (outside) atomicAdd(&out[3], outside);
    }
}

// ---------------------------------------------------------------------------
// batched mode: many independent graphs in one concatenated CSR
// ---------------------------------------------------------------------------

// Graph of every vertex (set up once).  One block per graph (grid-stride).
__global__ void __launch_bounds__(kTB) batch_gid_kernel(const int64_t *g_v0, int ngraphs, int32_t *gid)
{
    for (int g = blockIdx.x; g < ngraphs; g += gridDim.x)
        for (int64_t v = g_v0[g] + threadIdx.x; v < g_v0[g + 1]; v += blockDim.x) gid[v] = g;
}

// Initial labels: graph-local vertex IDs.  One block per graph (grid-stride).
// Sets *bad when an edge leaves its graph.  One block per graph (grid-stride).
__global__ void __launch_bounds__(kTB) batch_validate_kernel(const int64_t *off, const int32_t *nbr,
                                                             const int64_t *g_v0, int ngraphs, int *bad)
{
    for (int g = blockIdx.x; g < ngraphs; g += gridDim.x) {
        const int64_t v0 = g_v0[g], v1 = g_v0[g + 1];
        int b = 0;
        for (int64_t e = off[v0] + threadIdx.x; e < off[v1]; e += blockDim.x) {
            const int64_t u = nbr[e];
            b |= (u < v0 || u >= v1);
        }
        if (__any_sync(kFull, b) && (threadIdx.x & 31) == 0) atomicOr(bad, 1);
    }
}

__global__ void __launch_bounds__(kTB) batch_init_labels_kernel(const int64_t *g_v0, int ngraphs, int32_t *lab)
{
    for (int g = blockIdx.x; g < ngraphs; g += gridDim.x) {
        const int64_t v0 = g_v0[g], v1 = g_v0[g + 1];
        for (int64_t v = v0 + threadIdx.x; v < v1; v += blockDim.x) lab[v] = (int32_t)(v - v0);
    }
}

// Per-graph run bases after the scan: g_base[g] = run base of graph g's first vertex,
// g_base[ngraphs] = all runs.
__global__ void batch_bases_kernel(const int64_t *g_v0, int ngraphs, const int64_t *runbase, int64_t n, const Ctl *ctl,
                                   int64_t *g_base)
{
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g <= ngraphs; g += gridDim.x * blockDim.x) {
        const int64_t v = g_v0[g];
        g_base[g] = v < n ? runbase[v] : ctl->N;
    }
}

// After an iteration: per graph, the labels that changed and the reference's early exit
// (count <= n_g * 1e-5, dpp.cuh:88) per graph.  A graph that had already exited keeps its
// labels (lab_out = lab_in).  One block per graph (grid-stride).
__global__ void __launch_bounds__(kTB) batch_commit_kernel(const Ctl *ctl, const int64_t *g_v0, int ngraphs,
                                                           const int32_t *lab_in, int32_t *lab_out, int32_t *g_active,
                                                           int32_t *g_iters, long long *g_counts, int max_iter, int it,
                                                           int early_exit)
{
    __shared__ unsigned long long part[kTB / 32];
    if (!ctl_active(ctl)) return;  // every graph exited earlier: the final buffer is settled
    for (int g = blockIdx.x; g < ngraphs; g += gridDim.x) {
        const int64_t v0 = g_v0[g], v1 = g_v0[g + 1];
        if (!g_active[g]) {
            for (int64_t v = v0 + threadIdx.x; v < v1; v += blockDim.x) lab_out[v] = lab_in[v];
            continue;
        }
        unsigned long long c = 0;
        for (int64_t v = v0 + threadIdx.x; v < v1; v += blockDim.x) c += lab_out[v] != lab_in[v];
        c = __reduce_add_sync(kFull, (unsigned)c);
        if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = c;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long t = 0;
            for (int w = 0; w < kTB / 32; ++w) t += part[w];
            if (it < max_iter) g_counts[(int64_t)g * max_iter + it] = (long long)t;
            g_iters[g] = it + 1;
            if ((early_exit && (double)t <= (double)(v1 - v0) * 1e-5) || it + 1 >= max_iter) g_active[g] = 0;
        }
        __syncthreads();
    }
}

// Global bookkeeping after batch_commit: the run goes on while some graph is active.
__global__ void batch_finalize_kernel(Ctl *ctl, const int32_t *g_active, int ngraphs)
{
    __shared__ int any;
    if (threadIdx.x == 0) any = 0;
    __syncthreads();
    for (int g = threadIdx.x; g < ngraphs; g += blockDim.x)
        if (g_active[g]) any = 1;
    __syncthreads();
    if (threadIdx.x == 0) {
        if (ctl->active) {
            const unsigned long long c = ctl->changes;
            if (ctl->iter < 64) ctl->counts[ctl->iter] = c;
            ctl->iter += 1;
            if (!any || ctl->iter >= ctl->max_iter) ctl->active = 0;
        }
        ctl->changes = 0;
        ctl->ticket = 0;
    }
}

__global__ void batch_init_kernel(int32_t *g_active, int32_t *g_iters, int ngraphs, int active)
{
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ngraphs; g += gridDim.x * blockDim.x) {
        g_active[g] = active;
        g_iters[g] = 0;
    }
}

}  // namespace galp
