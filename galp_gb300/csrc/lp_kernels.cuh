// lp_kernels.cuh -- kernels of one exact label-propagation iteration (method-0 semantics).
//
// One iteration over a scope (whole graph in-core, one batch out-of-core, one graph
// of a batch) is:
//
//   big_insert -> big_combine -> [big_stats] -> lp_tile_kernel -> big_resolve -> finalize
//
// lp_tile_kernel is a persistent, single-pass kernel: CTAs take vertex tiles in
// vertex order from an atomic ticket, gather the tile's neighbour labels into shared
// memory once, count them (warp match for vertices of degree <= 32, a per-vertex
// shared-memory hash region for larger ones), publish the tile's distinct-label
// total, obtain the exclusive prefix (the run base of the tile's first vertex) by
// decoupled look-back over the preceding tiles, and resolve every vertex's winner
// with the positional tie rule while the tile is still on chip.  Vertices of degree
// above kTileSlots ("big") are counted beforehand into global hash tables by
// big_insert and big_combine (big_stats adds candidate ranks), take part in the scan
// as single-vertex tiles, and are resolved by big_resolve once their run base is known.
//
// Reference counterparts: DPPBase::perform_lp (label_propagation/src/dpp/dpp.cuh:104-138),
// gather_labels..update_labels (src/dpp/kernel.cuh:27-119), the segmented sort and
// scan (dpp.cuh:113-118) and SegmentedReducer::apply (src/common/segmented_reduce.cuh:586-615).
#pragma once

#include <cstdint>
#include <climits>

#include "lp_device.cuh"

namespace galp {

constexpr int kTB = 256;              // threads per CTA
constexpr int kNW = kTB / 32;         // warps per CTA
constexpr int kTileSlots = 2048;      // shared-memory label slots per tile
constexpr int kTileV = 512;           // vertices per tile
constexpr int kSmallMax = 32;         // degree handled by one warp pack
constexpr int kBigChunk = 1024;       // edges per big_insert CTA
constexpr int kBigSlotChunk = 8192;   // distinct-list entries per big_stats CTA
constexpr int kHubPartPairs = 8192;   // target pairs per hub partition (a hub of degree D: D / 8192 partitions)
constexpr int kHubTab = 16384;        // shared-memory table slots of a hub partition (distinct labels < 16384)
constexpr int kHubMaxParts = 1 << 20; // partitions of one hub at most
constexpr int kHubCountThreads = 1024;
constexpr int kHubBinMin = 256;       // a chunk with this many pairs bins them by partition in shared memory
constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr int kPickScratch = 8192;    // power of two >= kTile, for WarpTableQuery::tile_pick
constexpr long long kSpinLimit = 1ll << 20;  // default look-back give-up bound (about a second)

// error bits in Ctl::err
constexpr int kErrLookback = 1;
constexpr int kErrFormat = 2;
constexpr int kErrStage = 8;        // a bulk-copy wait of a counting kernel ran out (bounded wait)
constexpr int kErrHubOverflow = 4;  // a hub partition received more pairs, or more distinct labels, than it
                                    // holds (the run is redone with twice the partitions)

struct Ctl {
    int active;                 // 1 while iterations still run
    int iter;                   // iterations completed
    int err;                    // sticky error bits
    int pad0;
    unsigned long long ticket;  // tile ticket of the running lp_tile_kernel
    unsigned long long changes; // labels changed in the current iteration
    long long N;                // runs in the scope (written by the tile of last_v)
    long long thr;              // early-exit threshold: stop when changes <= thr
    int max_iter;               // iterations requested
    int pad1;
    unsigned long long counts[64];  // changes per iteration
    int tied_small;             // tied vertices listed by the count kernels (per scope)
    int tied_mid;
    int changed_n;              // vertices whose label changed (frontier mode)
    int frontier_off;           // frontier mode: this iteration recounts every vertex
};

// Per-big-vertex statistics (reset by big_resolve after use).
struct BigStat {
    int d;      // distinct labels
    int W;      // max count
    int k;      // candidates
    int cmin;   // smallest candidate label
    int cmax;   // largest candidate label
    int rmin;   // rank of cmin
    int rmax;   // rank of cmax
    int pad;
};

// Arguments of one iteration over one scope of run positions: the whole graph
// (in-core) or one batch (out-of-core).  Tile, big-vertex and chunk indices are
// relative to the scope's bases t0/b0/c0/s0; neighbour reads subtract nbr_shift
// (the first CSR entry held by the neighbour buffer).
struct IterArgs {
    const int32_t *nbr;        // CSR neighbours (global IDs), entries [nbr_shift, ...)
    int64_t nbr_shift;
    int32_t t0, b0, c0, s0;    // scope bases: tiles, big vertices, insert chunks, stats chunks
    const int64_t *off;        // CSR offsets (global)
    const uint16_t *vpos;      // slot position of each vertex in its tile
    const int32_t *tile_v0;    // ntiles+1: first vertex of each tile
    const int32_t *tile_big;   // ntiles: big-vertex index or -1
    const uint16_t *tile_used; // ntiles: slots used by the tile
    int32_t ntiles;
    int32_t last_v;            // last vertex that owns runs, or -1
    const int32_t *lab_in;
    int32_t *lab_out;
    unsigned long long *status;
    unsigned epoch;
    unsigned wait_xor;          // look-back accepts statuses of epoch ^ wait_xor (0; tests only)
    long long spin_limit;       // look-back polls before a wait gives up
    Ctl *ctl;
    // big vertices (hubs): each hub's labels are counted by hash partitions of its
    // distinct (label, count) pairs, one shared-memory table per partition
    int32_t nbig;
    const int32_t *big_v;       // vertex of each big entry
    const int32_t *chunk_big;   // insert chunk -> big index
    const int64_t *chunk_e0;    // insert chunk -> first edge
    const int64_t *chunk_e1;    // insert chunk -> end edge
    int32_t nchunks;
    const int32_t *schunk_big;  // stats chunk -> big index
    const int64_t *schunk_s0;   // stats chunk -> first entry of the vertex's distinct list
    const int64_t *schunk_s1;
    int32_t nschunks;
    const int32_t *hub_p0;      // first partition of each big vertex (global index; nbig + 1 entries)
    const int64_t *hub_pbase;   // pair-area offset of each big vertex's partitions (scope-relative)
    const int32_t *hub_pcap;    // pair capacity of each partition of the big vertex
    const int32_t *part_big;    // partition -> big index
    int32_t q0, nparts;         // the scope's partitions
    int *pfill;                 // pairs appended to each partition (hub_count_kernel resets it)
    int4 *psum;                 // per partition: max count, candidates, smallest, largest
    unsigned long long *pairs;  // pair area: label << 32 | count
    unsigned long long *big_list;  // distinct label << 32 | count of each big vertex (capacity = degree)
    const int64_t *big_ooff;    // offset of each big vertex's distinct list (scope-relative)
    BigStat *bstat;
    int64_t *big_a;             // run base of each big vertex (written by the scan)
    const int64_t *runbase;     // run base of every vertex when the scan precedes big_resolve
    int32_t *changed;           // frontier mode: vertices whose label changes (else null)
};

__device__ __forceinline__ int pad32(int x) { return (x + 31) & ~31; }

__device__ __forceinline__ bool ctl_active(const Ctl *c)
{
    return *((volatile const int *)&c->active) != 0;
}

// ---------------------------------------------------------------------------
// warp helpers
// ---------------------------------------------------------------------------

// max over the contiguous lane segment [first, last] containing this lane
__device__ __forceinline__ int seg_max(int val, int lane, int first, int last)
{
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        int o = __shfl_down_sync(kFull, val, off);
        if (lane + off <= last) val = max(val, o);
    }
    return __shfl_sync(kFull, val, first);
}

__device__ __forceinline__ int seg_min(int val, int lane, int first, int last)
{
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        int o = __shfl_down_sync(kFull, val, off);
        if (lane + off <= last) val = min(val, o);
    }
    return __shfl_sync(kFull, val, first);
}

__device__ __forceinline__ long long warp_sum_ll(long long v)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(kFull, v, off);
    return v;
}

// Block-wide decoupled look-back: all kTB threads read kTB predecessors per round
// trip, so a tile whose nearest published prefix lies a few hundred tiles back (the
// usual case with hundreds of resident CTAs) waits for one or two L2 round trips.
// Called by every thread of the block; returns the exclusive prefix to all.
struct LookbackSmem {
    long long wsum[kNW];
    int wfirst[kNW];
    long long P;
    int done;
};

// A wait gives up after spin_limit polls (or at once when another wait already gave
// up), sets kErrLookback and takes a zero prefix, so the kernel always returns; the host
// reports the error.  The wait accepts statuses of epoch (epoch ^ wait_xor): wait_xor is
// 0 except in the failure-detection test, where no tile publishes that epoch.
__device__ long long lookback_prefix_block(unsigned long long *status, long long t, unsigned epoch, long long D,
                                           Ctl *ctl, LookbackSmem &L, long long spin_limit, unsigned wait_xor)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (t == 0) {
        if (tid == 0) st_relaxed_u64(&status[0], pack_status(2, epoch, (unsigned long long)D));
        return 0;
    }
    if (tid == 0) st_relaxed_u64(&status[t], pack_status(1, epoch, (unsigned long long)D));
    const unsigned ep = (epoch ^ wait_xor) & kEpochMask;
    long long P = 0;
    long long j = t - 1;
    for (;;) {
        const long long jj = j - tid;
        unsigned long long w = 0;
        unsigned state = 2;
        if (jj >= 0) {
            long long spins = 0;
            unsigned ns = 32;
            for (;;) {
                w = ld_relaxed_u64(&status[jj]);
                state = (unsigned)(w >> kStateShift);
                if (state != 0 && (unsigned)((w >> kEpochShift) & kEpochMask) == ep) break;
                // give up after spin_limit polls, or at once when another wait already gave up
                if (++spins > spin_limit || *((volatile int *)&ctl->err)) {
                    atomicOr(&ctl->err, kErrLookback);
                    state = 2;
                    w = 0;
                    break;
                }
                __nanosleep(ns);
                if (ns < 1024) ns <<= 1;
            }
        } else {
            w = 0;  // before the first tile: prefix 0
        }
        // nearest predecessor holding an inclusive prefix = smallest tid with state 2
        const unsigned pm = __ballot_sync(kFull, state == 2);
        if (lane == 0) L.wfirst[warp] = pm ? (warp * 32 + __ffs(pm) - 1) : INT_MAX;
        __syncthreads();
        int first = INT_MAX;
#pragma unroll
        for (int w2 = 0; w2 < kNW; ++w2) first = min(first, L.wfirst[w2]);
        long long val = (tid <= first) ? (long long)(w & kValueMask) : 0;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) val += __shfl_xor_sync(kFull, val, off);
        if (lane == 0) L.wsum[warp] = val;
        __syncthreads();
        long long sum = 0;
#pragma unroll
        for (int w2 = 0; w2 < kNW; ++w2) sum += L.wsum[w2];
        P += sum;
        __syncthreads();  // L is rewritten by the next round
        if (first != INT_MAX) break;
        j -= kTB;
    }
    if (tid == 0) st_relaxed_u64(&status[t], pack_status(2, epoch, (unsigned long long)(P + D)));
    return P;
}

// ---------------------------------------------------------------------------
// warp-level queries used for tied vertices that the per-vertex summary cannot decide
// ---------------------------------------------------------------------------

// Vertex of degree <= 32 whose labels occupy lanes [0, deg) of the warp.
struct WarpSmallQuery {
    bool cand;
    int rk;
    __device__ int first_ge(int64_t x)
    {
        int m = __reduce_min_sync(kFull, (cand && rk >= x) ? rk : INT_MAX);
        return m == INT_MAX ? -1 : m;
    }
    __device__ int last_lt(int64_t y)
    {
        return __reduce_max_sync(kFull, (cand && rk < y) ? rk : -1);
    }
    __device__ int tile_pick(int64_t lo)
    {
        const bool in = cand && rk >= lo && rk < lo + kTile;
        const int key = __reduce_max_sync(kFull, in ? tile_priority(rk - lo) : -1);
        const unsigned m = __ballot_sync(kFull, in && tile_priority(rk - lo) == key);
        return m ? __shfl_sync(kFull, rk, __ffs(m) - 1) : -1;
    }
};

// Sorted run list (labels ascending, counts) of a vertex of degree <= 32, scanned by
// one thread.
struct RunListQuery {
    const uint32_t *lab;
    const uint32_t *cnt;
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
    __device__ int tile_pick(int64_t lo) const
    {
        int best = -1, br = -1;
        for (int r = 0; r < d; ++r)
            if ((int)cnt[r] == W && r >= lo && r < lo + kTile && tile_priority(r - lo) > best) {
                best = tile_priority(r - lo);
                br = r;
            }
        return br;
    }
};

// Table layouts a WarpTableQueryT reads: k(s) = label of slot s or kEmpty, c(s) = its count.
struct SplitTable {  // separate key and count arrays (shared-memory regions)
    const uint32_t *key;
    const uint32_t *cnt;
    __device__ uint32_t k(int s) const { return key[s]; }
    __device__ uint32_t c(int s) const { return cnt[s]; }
};
struct DenseTable {  // a big vertex's distinct list: label << 32 | count, every entry occupied
    const unsigned long long *list;
    __device__ uint32_t k(int s) const { return (uint32_t)(list[s] >> 32); }
    __device__ uint32_t c(int s) const { return (uint32_t)list[s]; }
};

// Open-addressed table region of one vertex, scanned by one warp.
// hist: 256 ints of warp-private shared memory.
template <class T>
struct WarpTableQueryT {
    T t;
    int cap;
    int d, W, rmin, rmax;
    int *hist;
    int lane;
    uint32_t *scratch;  // kPickScratch entries for tile_pick (only vertices with >= kTile distinct labels)

    __device__ int nslots() const { return cap; }
    __device__ int slot(int i) const { return i; }

    // x-th smallest key (0-based) among the occupied slots
    __device__ uint32_t select(int x)
    {
        uint32_t prefix = 0;
        int remaining = x;
        for (int shift = 24; shift >= 0; shift -= 8) {
            for (int b = lane; b < 256; b += 32) hist[b] = 0;
            __syncwarp();
            const uint32_t hi_mask = (shift == 24) ? 0u : (0xFFFFFFFFu << (shift + 8));
            for (int i = lane; i < nslots(); i += 32) {
                uint32_t k = t.k(slot(i));
                if (k != kEmpty && (k & hi_mask) == (prefix & hi_mask)) atomicAdd(&hist[(k >> shift) & 255], 1);
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
                int o = __shfl_up_sync(kFull, incl, off);
                if (lane >= off) incl += o;
            }
            const int excl = incl - local;
            // the bin holding the target lies in the lane whose range covers `remaining`
            const bool mine = remaining >= excl && remaining < incl;
            const unsigned who = __ballot_sync(kFull, mine);
            const int src = who ? (__ffs(who) - 1) : 31;
            int digit = 0, before = 0;
            if (lane == src) {
                int acc = excl;
                int i = 0;
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
    __device__ int rank_of(uint32_t c)
    {
        int n = 0;
        for (int i = lane; i < nslots(); i += 32) {
            uint32_t k = t.k(slot(i));
            n += (k != kEmpty && k < c);
        }
        return __reduce_add_sync(kFull, n);
    }
    __device__ int first_ge(int64_t x)
    {
        if (x >= d) return -1;
        if (x <= rmin) return rmin;
        const uint32_t L = select((int)x);
        uint32_t best = kEmpty;
        for (int i = lane; i < nslots(); i += 32) {
            const int s = slot(i);
            uint32_t k = t.k(s);
            if (k != kEmpty && (int)t.c(s) == W && k >= L && k < best) best = k;
        }
        best = __reduce_min_sync(kFull, best);
        if (best == kEmpty) return -1;
        return rank_of(best);
    }
    __device__ int last_lt(int64_t y)
    {
        if (y > rmax) return rmax;
        if (y <= rmin) return -1;
        const uint32_t L = select((int)y);
        int best = -1;
        for (int i = lane; i < nslots(); i += 32) {
            const int s = slot(i);
            uint32_t k = t.k(s);
            if (k != kEmpty && (int)t.c(s) == W && k < L && (int)k > best) best = (int)k;
        }
        best = __reduce_max_sync(kFull, best);
        if (best < 0) return -1;
        return rank_of((uint32_t)best);
    }
    // Sort the tile's kTile distinct labels (ranks [lo, lo + kTile)) in scratch and
    // pick the candidate of highest tile_priority.  Entries are label << 1 | candidate
    // (labels are below 2^31 - 1, so they sort by label and stay below kEmpty).
    __device__ int tile_pick(int64_t lo)
    {
        if (!scratch) return -1;
        const uint32_t Llo = select((int)lo);
        const uint32_t Lhi = (lo + kTile < d) ? select((int)(lo + kTile)) : kEmpty;
        int base = 0;
        for (int i0 = 0; i0 < nslots(); i0 += 32) {
            const int i = i0 + lane;
            const int s = (i < nslots()) ? slot(i) : 0;
            const uint32_t k = (i < nslots()) ? t.k(s) : kEmpty;
            const bool in = k != kEmpty && k >= Llo && k < Lhi;
            const unsigned m = __ballot_sync(kFull, in);
            if (in && base + __popc(m & ((1u << lane) - 1)) < kPickScratch)
                scratch[base + __popc(m & ((1u << lane) - 1))] = (k << 1) | ((int)t.c(s) == W ? 1u : 0u);
            base += __popc(m);
        }
        const int nin = min(base, kPickScratch);
        for (int i = nin + lane; i < kPickScratch; i += 32) scratch[i] = kEmpty;
        __syncwarp();
        for (int kk = 2; kk <= kPickScratch; kk <<= 1) {
            for (int j = kk >> 1; j > 0; j >>= 1) {
                for (int i = lane; i < kPickScratch; i += 32) {
                    const int ixj = i ^ j;
                    if (ixj > i) {
                        const uint32_t x = scratch[i], y = scratch[ixj];
                        const bool up = (i & kk) == 0;
                        if ((x > y) == up) {
                            scratch[i] = y;
                            scratch[ixj] = x;
                        }
                    }
                }
                __syncwarp();
            }
        }
        int best = -1, bi = -1;
        for (int i = lane; i < nin; i += 32) {
            if ((scratch[i] & 1u) && tile_priority(i) > best) {
                best = tile_priority(i);
                bi = i;
            }
        }
        const int top = __reduce_max_sync(kFull, best);
        const unsigned m = __ballot_sync(kFull, best == top && bi >= 0);
        if (top < 0 || !m) return -1;
        return (int)lo + __shfl_sync(kFull, bi, __ffs(m) - 1);
    }
};
using WarpTableQuery = WarpTableQueryT<SplitTable>;

// ---------------------------------------------------------------------------
// the tile kernel
// ---------------------------------------------------------------------------
struct TileSmem {
    int32_t lab[kTileSlots];
    uint32_t hkey[2 * kTileSlots];
    uint32_t hcnt[2 * kTileSlots];
    int16_t svid[kTileSlots];
    int64_t voff[kTileV + 1];
    uint16_t vpos[kTileV];
    int32_t vd[kTileV];
    int32_t vW[kTileV];
    int32_t vk[kTileV];
    int32_t vcmin[kTileV];
    int32_t vcmax[kTileV];
    int32_t vrmin[kTileV];
    int32_t vrmax[kTileV];
    int16_t vpref[kTileV];
    int16_t hard[kTileV];
    int16_t hard_rank[kTileV];
    int32_t wtmp[kNW];
    LookbackSmem lb;
    long long tile;
    long long P;
    long long N;
    int D;
    int nhard;
    int has_mid;
};

__device__ __forceinline__ int vdeg(const TileSmem &S, int i) { return (int)(S.voff[i + 1] - S.voff[i]); }

__global__ void __launch_bounds__(kTB, 3) lp_tile_kernel(IterArgs p)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TileSmem &S = *reinterpret_cast<TileSmem *>(smem_raw);
    if (!ctl_active(p.ctl)) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    unsigned long long changes = 0;

    for (;;) {
        if (tid == 0) S.tile = (long long)atomicAdd(&p.ctl->ticket, 1ull);
        __syncthreads();
        const long long t = S.tile;
        if (t >= p.ntiles) break;
        const long long tg = p.t0 + t;
        const int v0 = p.tile_v0[tg], v1 = p.tile_v0[tg + 1];
        const int bi = p.tile_big[tg];

        if (bi >= 0) {
            // single big vertex: its distinct count was computed by big_insert
            const long long D = *((volatile int *)&p.bstat[bi].d);
            const long long P = lookback_prefix_block(p.status, t, p.epoch, D, p.ctl, S.lb, p.spin_limit, p.wait_xor);
            if (tid == 0) {
                p.big_a[bi] = P;
                if (v0 == p.last_v) p.ctl->N = P + D;
            }
            __syncthreads();
            continue;
        }

        const int nv = v1 - v0;
        const int used = p.tile_used[tg];
        // P1: per-vertex metadata, slot map and hash regions reset
        for (int i = tid; i <= nv; i += kTB) S.voff[i] = __ldg(&p.off[v0 + i]);
        for (int i = tid; i < nv; i += kTB) {
            S.vpos[i] = __ldg(&p.vpos[v0 + i]);
            S.vd[i] = 0;
            S.vW[i] = 0;
            S.vk[i] = 0;
            S.vcmin[i] = INT_MAX;
            S.vcmax[i] = -1;
            S.vrmin[i] = 0;
            S.vrmax[i] = 0;
        }
        for (int s = tid; s < used; s += kTB) S.svid[s] = -1;
        if (tid == 0) {
            S.nhard = 0;
            S.has_mid = 0;
        }
        __syncthreads();
        // P2: slot -> vertex map (vertex starts, then an inclusive max-scan); hash
        // regions of vertices above 32 edges cleared
        {
            int mid_here = 0;
            for (int i = tid; i < nv; i += kTB) {
                const int dg = vdeg(S, i);
                if (dg > 0) S.svid[S.vpos[i]] = (int16_t)i;
                if (dg > kSmallMax) mid_here = 1;
            }
            if (__any_sync(kFull, mid_here) && lane == 0) S.has_mid = 1;
        }
        __syncthreads();
        if (S.has_mid)
            for (int s = tid; s < 2 * used; s += kTB) {
                S.hkey[s] = kEmpty;
                S.hcnt[s] = 0;
            }
        {
            constexpr int PER = kTileSlots / kTB;
            const int s0 = tid * PER;
            int run = -1;
            int loc[PER];
#pragma unroll
            for (int i = 0; i < PER; ++i) {
                int x = (s0 + i < used) ? S.svid[s0 + i] : -1;
                run = max(run, x);
                loc[i] = run;
            }
            int incl = run;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                int o = __shfl_up_sync(kFull, incl, off);
                if (lane >= off) incl = max(incl, o);
            }
            if (lane == 31) S.wtmp[warp] = incl;
            __syncthreads();
            int carry = -1;
            for (int w = 0; w < warp; ++w) carry = max(carry, S.wtmp[w]);
            int up = __shfl_up_sync(kFull, incl, 1);
            if (lane > 0) carry = max(carry, up);
#pragma unroll
            for (int i = 0; i < PER; ++i)
                if (s0 + i < used) S.svid[s0 + i] = (int16_t)max(loc[i], carry);
        }
        __syncthreads();
        // P3: gather labels with all of a thread's loads in flight together; insert
        // the labels of vertices with degree > 32 into their hash region
        {
            constexpr int PER = kTileSlots / kTB;
            int nb[PER];
#pragma unroll
            for (int i = 0; i < PER; ++i) {
                const int s = tid + i * kTB;
                nb[i] = -1;
                if (s < used) {
                    const int v = S.svid[s];
                    if (v >= 0) {
                        const int64_t o = S.voff[v];
                        const int j = s - (int)S.vpos[v];
                        if (j < (int)(S.voff[v + 1] - o)) nb[i] = __ldg(&p.nbr[o + j - p.nbr_shift]);
                    }
                }
            }
            int lb[PER];
#pragma unroll
            for (int i = 0; i < PER; ++i) lb[i] = (nb[i] >= 0) ? __ldg(&p.lab_in[nb[i]]) : -1;
#pragma unroll
            for (int i = 0; i < PER; ++i) {
                if (nb[i] < 0) continue;
                const int s = tid + i * kTB;
                const int32_t L = lb[i];
                S.lab[s] = L;
                const int v = S.svid[s];
                const int deg = vdeg(S, v);
                if (deg > kSmallMax) {
                    const uint32_t cap = 2u * (uint32_t)pad32(deg);
                    const uint32_t base = 2u * (uint32_t)S.vpos[v];
                    uint32_t h = hslot((uint32_t)L, cap);
                    for (;;) {
                        uint32_t prev = atomicCAS(&S.hkey[base + h], kEmpty, (uint32_t)L);
                        if (prev == kEmpty || prev == (uint32_t)L) {
                            atomicAdd(&S.hcnt[base + h], 1u);
                            break;
                        }
                        h = (h + 1 == cap) ? 0 : h + 1;
                    }
                }
            }
        }
        __syncthreads();
        // P4: counting summaries per pack of 32 slots (passes 1 and 2 only for tiles
        // holding a vertex above 32 edges)
        const int npk = (used + 31) >> 5;
        const int npass = S.has_mid ? 3 : 1;
        for (int pass = 0; pass < npass; ++pass) {
            for (int pk = warp; pk < npk; pk += kNW) {
                const int s = pk * 32 + lane;
                const int v = (s < used) ? S.svid[s] : -1;
                const int vl0 = __shfl_sync(kFull, v, 0);
                bool mid = false;
                if (vl0 >= 0) {
                    const int dg = vdeg(S, vl0);
                    mid = dg > kSmallMax && (pk * 32 - (int)S.vpos[vl0]) < pad32(dg);
                }
                if (mid) {
                    const int h0 = pk * 64 + lane, h1 = h0 + 32;
                    const uint32_t k0 = S.hkey[h0], k1 = S.hkey[h1];
                    const int c0 = (int)S.hcnt[h0], c1 = (int)S.hcnt[h1];
                    if (pass == 0) {
                        int dp = (k0 != kEmpty) + (k1 != kEmpty);
                        int wp = max(c0, c1);
                        dp = __reduce_add_sync(kFull, dp);
                        wp = __reduce_max_sync(kFull, wp);
                        if (lane == 0) {
                            atomicAdd(&S.vd[vl0], dp);
                            atomicMax(&S.vW[vl0], wp);
                        }
                    } else if (pass == 1) {
                        const int W = S.vW[vl0];
                        const bool q0 = k0 != kEmpty && c0 == W, q1 = k1 != kEmpty && c1 == W;
                        int kp = (int)q0 + (int)q1;
                        int mn = min(q0 ? (int)k0 : INT_MAX, q1 ? (int)k1 : INT_MAX);
                        int mx = max(q0 ? (int)k0 : -1, q1 ? (int)k1 : -1);
                        kp = __reduce_add_sync(kFull, kp);
                        mn = __reduce_min_sync(kFull, mn);
                        mx = __reduce_max_sync(kFull, mx);
                        if (lane == 0) {
                            atomicAdd(&S.vk[vl0], kp);
                            atomicMin(&S.vcmin[vl0], mn);
                            atomicMax(&S.vcmax[vl0], mx);
                        }
                    } else {
                        if (S.vk[vl0] == 1) continue;  // a unique winner needs no ranks
                        const int cmn = S.vcmin[vl0], cmx = S.vcmax[vl0];
                        int a0 = (k0 != kEmpty && (int)k0 < cmn) + (k1 != kEmpty && (int)k1 < cmn);
                        int a1 = (k0 != kEmpty && (int)k0 < cmx) + (k1 != kEmpty && (int)k1 < cmx);
                        a0 = __reduce_add_sync(kFull, a0);
                        a1 = __reduce_add_sync(kFull, a1);
                        if (lane == 0) {
                            atomicAdd(&S.vrmin[vl0], a0);
                            atomicAdd(&S.vrmax[vl0], a1);
                        }
                    }
                } else if (pass == 0) {
                    bool valid = false;
                    int lab = 0;
                    if (v >= 0) valid = (s - (int)S.vpos[v]) < vdeg(S, v);
                    if (valid) lab = S.lab[s];
                    const unsigned long long key =
                        valid ? (((unsigned long long)(unsigned)v << 32) | (unsigned)lab) : (0xFFFFFFFF00000000ull | (unsigned)lane);
                    const unsigned eq = __match_any_sync(kFull, key);
                    const unsigned vm = __match_any_sync(kFull, valid ? v : (-1 - lane));
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
                        // every vertex of the pack has a unique winner: no ranks needed
                        const unsigned m = cm & vm;
                        cmin = cmax = __shfl_sync(kFull, lab, m ? (__ffs(m) - 1) : lane);
                    } else {
                        // Sort the pack by (vertex, label); vertices keep their lanes, equal
                        // labels become adjacent runs in ascending order.  Each vertex's runs
                        // (label, count) are written to its slots of hkey/hcnt (unused by
                        // vertices of degree <= 32) for per-thread resolution later.
                        unsigned long long sk = key;
                        int sc = valid ? cnt : 0;
#pragma unroll
                        for (int kk = 2; kk <= 32; kk <<= 1) {
#pragma unroll
                            for (int j = kk >> 1; j > 0; j >>= 1) {
                                const unsigned long long ok = __shfl_xor_sync(kFull, sk, j);
                                const int oc = __shfl_xor_sync(kFull, sc, j);
                                const bool up = (lane & kk) == 0, lower = (lane & j) == 0;
                                const bool take = (lower == up) ? (ok < sk) : (ok > sk);
                                if (take) {
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
                        const unsigned cr = __ballot_sync(kFull, head && sc == W) & vm;
                        if (head) {
                            const int base = 2 * (int)S.vpos[v];
                            S.hkey[base + rank] = (uint32_t)slab;
                            S.hcnt[base + rank] = (uint32_t)sc;
                        }
                        const int lo = cr ? (__ffs(cr) - 1) : lane, hi = cr ? (31 - __clz(cr)) : lane;
                        cmin = __shfl_sync(kFull, slab, lo);
                        cmax = __shfl_sync(kFull, slab, hi);
                        rmin = __popc(hm & ((1u << lo) - 1));
                        rmax = __popc(hm & ((1u << hi) - 1));
                    }
                    if (valid && lane == first) {
                        S.vd[v] = d;
                        S.vW[v] = W;
                        S.vk[v] = k;
                        S.vcmin[v] = cmin;
                        S.vcmax[v] = cmax;
                        S.vrmin[v] = rmin;
                        S.vrmax[v] = rmax;
                    }
                }
            }
            __syncthreads();
        }
        // P5: exclusive scan of distinct counts over the tile's vertices
        {
            const int i0 = 2 * tid, i1 = 2 * tid + 1;
            const int x0 = i0 < nv ? S.vd[i0] : 0, x1 = i1 < nv ? S.vd[i1] : 0;
            const int sum = x0 + x1;
            int incl = sum;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                int o = __shfl_up_sync(kFull, incl, off);
                if (lane >= off) incl += o;
            }
            if (lane == 31) S.wtmp[warp] = incl;
            __syncthreads();
            int base = 0, tot = 0;
            for (int w = 0; w < kNW; ++w) {
                if (w < warp) base += S.wtmp[w];
                tot += S.wtmp[w];
            }
            const int excl = base + incl - sum;
            if (i0 < nv) S.vpref[i0] = (int16_t)excl;
            if (i1 < nv) S.vpref[i1] = (int16_t)(excl + x0);
            if (tid == 0) S.D = tot;
        }
        __syncthreads();
        // P6: the tile's run base by block-wide look-back, then the vertices whose
        // winner is unique (no position needed)
        {
            const long long P = lookback_prefix_block(p.status, t, p.epoch, S.D, p.ctl, S.lb, p.spin_limit, p.wait_xor);
            if (tid == 0) {
                S.P = P;
                if (p.last_v >= v0 && p.last_v < v1) {
                    S.N = P + S.D;
                    p.ctl->N = P + S.D;
                } else {
                    S.N = -1;
                }
            }
        }
        for (int i = tid; i < nv; i += kTB) {
            const int v = v0 + i;
            if (vdeg(S, i) == 0 || S.vk[i] == 1) {
                const int32_t old = __ldg(&p.lab_in[v]);
                const int32_t nl = vdeg(S, i) == 0 ? old : S.vcmin[i];
                p.lab_out[v] = nl;
                changes += (nl != old);
            }
        }
        __syncthreads();
        // P7: resolve tied vertices: from the summary when it decides, from the sorted
        // run list for vertices of degree <= 32, else by a warp query in P8
        for (int i = tid; i < nv; i += kTB) {
            if (vdeg(S, i) == 0 || S.vk[i] == 1) continue;
            const int v = v0 + i;
            const int32_t old = __ldg(&p.lab_in[v]);
            int32_t nl;
            const int k = S.vk[i], d = S.vd[i];
            const long long a = S.P + S.vpref[i];
            SummaryQuery q(k, d, S.vrmin[i], S.vrmax[i]);
            int r = resolve_rank(a, d, S.N, v == p.last_v, q);
            if (!q.fail && r == S.vrmin[i]) {
                nl = S.vcmin[i];
            } else if (!q.fail && r == S.vrmax[i]) {
                nl = S.vcmax[i];
            } else if (vdeg(S, i) <= kSmallMax) {
                const int base = 2 * (int)S.vpos[i];
                RunListQuery rq{&S.hkey[base], &S.hcnt[base], d, S.vW[i]};
                if (q.fail) r = resolve_rank(a, d, S.N, v == p.last_v, rq);
                nl = (int32_t)S.hkey[base + r];
            } else {
                const int h = atomicAdd(&S.nhard, 1);
                S.hard[h] = (int16_t)i;
                S.hard_rank[h] = (int16_t)(q.fail ? -1 : r);
                continue;
            }
            p.lab_out[v] = nl;
            changes += (nl != old);
        }
        __syncthreads();
        // P8: tied vertices above 32 edges whose summary does not decide: warp queries
        // over the vertex's hash region (radix-select histograms alias the label slots,
        // which are no longer needed)
        if (S.nhard) {
            int *hist = reinterpret_cast<int *>(S.lab) + warp * 256;
            for (int h = warp; h < S.nhard; h += kNW) {
                const int i = S.hard[h];
                int r = S.hard_rank[h];
                const int v = v0 + i;
                const int deg = vdeg(S, i);
                const int d = S.vd[i], W = S.vW[i];
                const long long a = S.P + S.vpref[i];
                WarpTableQuery q{{&S.hkey[2 * S.vpos[i]], &S.hcnt[2 * S.vpos[i]]}, 2 * pad32(deg), d, W,
                                 S.vrmin[i], S.vrmax[i], hist, lane, nullptr};
                if (r < 0) r = resolve_rank(a, d, S.N, v == p.last_v, q);
                const int32_t label =
                    (r == S.vrmin[i]) ? S.vcmin[i] : (r == S.vrmax[i]) ? S.vcmax[i] : (int32_t)q.select(r);
                if (lane == 0) {
                    const int32_t old = __ldg(&p.lab_in[v]);
                    p.lab_out[v] = label;
                    changes += (label != old);
                }
            }
        }
        __syncthreads();
    }
    // one global update of the change counter per CTA
    unsigned long long c = changes;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) c += __shfl_xor_sync(kFull, c, off);
    if (lane == 0 && c) atomicAdd(&p.ctl->changes, c);
}

// ---------------------------------------------------------------------------
// big vertices
// ---------------------------------------------------------------------------

// Partition of a hub's label: the high bits of a hash independent of the one that places
// labels in a partition's table (hslot).
__device__ __forceinline__ uint32_t hub_part(uint32_t label, uint32_t nparts)
{
    return __umulhi(mix32(label ^ 0x9E3779B9u), nparts);
}

// Count the labels of one chunk of a big vertex's edges in shared memory, then append
// the chunk's distinct (label, count) pairs to the vertex's hash partitions (one
// reservation per warp and partition; appends to a partition are contiguous, so its
// sectors fill in L2).  A partition that is full drops the pair and flags the run, which
// the host then redoes with twice the partitions.
__global__ void __launch_bounds__(kTB, 8) big_insert_kernel(IterArgs p)
{
    // 18 KB of shared memory: the rest of the unified L1 caches the label gathers
    __shared__ uint32_t skey[2 * kBigChunk];
    __shared__ uint32_t scnt[2 * kBigChunk];
    __shared__ uint16_t sused[kBigChunk];     // occupied local slots, compacted
    __shared__ int nused;
    if (!ctl_active(p.ctl)) return;
    if ((int)blockIdx.x >= p.nchunks) return;
    const int ch = p.c0 + blockIdx.x;
    const int bi = p.chunk_big[ch];
    const int64_t e0 = p.chunk_e0[ch] - p.nbr_shift, e1 = p.chunk_e1[ch] - p.nbr_shift;
    const uint32_t cap = 2u * kBigChunk;
    for (int s = threadIdx.x; s < (int)cap; s += kTB) {
        skey[s] = kEmpty;
        scnt[s] = 0;
    }
    if (threadIdx.x == 0) nused = 0;
    __syncthreads();
    {
        // all of a thread's neighbour loads, then all its label gathers, in flight together
        constexpr int PER = kBigChunk / kTB;
        int nb[PER];
#pragma unroll
        for (int i = 0; i < PER; ++i) {
            const int64_t e = e0 + threadIdx.x + (int64_t)i * kTB;
            nb[i] = (e < e1) ? ld_nbr(&p.nbr[e]) : -1;
        }
        uint32_t lb[PER];
#pragma unroll
        for (int i = 0; i < PER; ++i) lb[i] = (nb[i] >= 0) ? (uint32_t)__ldg(&p.lab_in[nb[i]]) : kEmpty;
#pragma unroll
        for (int i = 0; i < PER; ++i) {
            const uint32_t L = lb[i];
            const unsigned same = __match_any_sync(kFull, L);
            if (L == kEmpty || (int)(threadIdx.x & 31) != __ffs(same) - 1) continue;
            uint32_t h = hslot(L, cap);
            for (;;) {
                uint32_t prev = atomicCAS(&skey[h], kEmpty, L);
                if (prev == kEmpty || prev == L) {
                    atomicAdd(&scnt[h], (uint32_t)__popc(same));
                    break;
                }
                h = (h + 1 == cap) ? 0 : h + 1;
            }
        }
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    // compact the occupied local slots, so the append rounds below run on full warps
    for (int s0 = 0; s0 < (int)cap; s0 += kTB) {
        const int s = s0 + threadIdx.x;
        const bool used = skey[s] != kEmpty;
        const unsigned m = __ballot_sync(kFull, used);
        if (!m) continue;
        int at = 0;
        if (lane == __ffs(m) - 1) at = atomicAdd(&nused, __popc(m));
        at = __shfl_sync(kFull, at, __ffs(m) - 1);
        if (used) sused[at + __popc(m & ((1u << lane) - 1))] = (uint16_t)s;
    }
    __syncthreads();
    const int nloc = nused;
    const int q = p.hub_p0[bi];
    const int np = p.hub_p0[bi + 1] - q;
    const int pcap = p.hub_pcap[bi];
    unsigned long long *area = p.pairs + p.hub_pbase[bi];
    if (nloc >= kHubBinMin && np <= kBigChunk) {
        // many pairs (labels still mostly distinct): bin them by partition, then one
        // reservation per partition touched; the chunk's pairs of a partition land side by
        // side.  The pairs move to the front of the table arrays (nloc <= kBigChunk); the back
        // halves then hold the bins (skey) and each pair's partition and rank (scnt).
        constexpr int PAIRS = kBigChunk / kTB;
        uint32_t kk[PAIRS], cc[PAIRS];
#pragma unroll
        for (int r = 0; r < PAIRS; ++r) {
            const int i = threadIdx.x + r * kTB;
            if (i < nloc) {
                kk[r] = skey[sused[i]];
                cc[r] = scnt[sused[i]];
            }
        }
        __syncthreads();
        int *sbin = reinterpret_cast<int *>(skey + kBigChunk);
        uint32_t *spr = scnt + kBigChunk;  // partition << 16 | rank
#pragma unroll
        for (int r = 0; r < PAIRS; ++r) {
            const int i = threadIdx.x + r * kTB;
            if (i < nloc) {
                skey[i] = kk[r];
                scnt[i] = cc[r];
            }
        }
        for (int b = threadIdx.x; b < np; b += kTB) sbin[b] = 0;
        __syncthreads();
        for (int i = threadIdx.x; i < nloc; i += kTB) {
            const uint32_t part = hub_part(skey[i], (uint32_t)np);
            spr[i] = (part << 16) | (uint32_t)atomicAdd(&sbin[part], 1);
        }
        __syncthreads();
        for (int b = threadIdx.x; b < np; b += kTB) {
            const int cnt = sbin[b];
            if (cnt) sbin[b] = atomicAdd(&p.pfill[q + b], cnt);
        }
        __syncthreads();
        for (int i = threadIdx.x; i < nloc; i += kTB) {
            const int part = (int)(spr[i] >> 16);
            const int at = sbin[part] + (int)(spr[i] & 0xFFFFu);
            if (at < pcap) area[(int64_t)part * pcap + at] = ((unsigned long long)skey[i] << 32) | scnt[i];
            else atomicOr(&p.ctl->err, kErrHubOverflow);
        }
        return;
    }
    // few pairs (labels repeat): one reservation per partition among a warp's pairs
    for (int base = 0; base < nloc; base += kTB) {  // block-uniform trip count
        const int i = base + threadIdx.x;
        uint32_t L = kEmpty, c = 0;
        int part = -1;
        if (i < nloc) {
            const uint32_t ls = sused[i];
            L = skey[ls];
            c = scnt[ls];
            part = (int)hub_part(L, (uint32_t)np);
        }
        const unsigned grp = __match_any_sync(kFull, part);
        const int leader = __ffs(grp) - 1;
        int at = 0;
        if (part >= 0 && lane == leader) at = atomicAdd(&p.pfill[q + part], __popc(grp));
        at = __shfl_sync(kFull, at, leader) + __popc(grp & ((1u << lane) - 1));
        if (part >= 0) {
            if (at < pcap) area[(int64_t)part * pcap + at] = ((unsigned long long)L << 32) | c;
            else atomicOr(&p.ctl->err, kErrHubOverflow);
        }
    }
}

// Ranks of each big vertex's smallest and largest candidate among its distinct labels,
// over its distinct list, one CTA per stats chunk; only vertices with some but not all
// distinct labels tied at the maximum need them.
__global__ void __launch_bounds__(kTB) big_stats_kernel(IterArgs p)
{
    __shared__ int red[2][kNW];
    if (!ctl_active(p.ctl)) return;
    if ((int)blockIdx.x >= p.nschunks) return;
    const int c = p.s0 + blockIdx.x;
    const int bi = p.schunk_big[c];
    BigStat &st = p.bstat[bi];
    const int d = *((volatile int *)&st.d);
    const int64_t i0 = p.schunk_s0[c];
    const int64_t i1 = min(p.schunk_s1[c], (int64_t)d);
    if (st.k == 1 || st.k == d || i0 >= i1) return;
    const unsigned long long *list = p.big_list + p.big_ooff[bi];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int cmn = st.cmin, cmx = st.cmax;
    int r0 = 0, r1 = 0;
    for (int64_t i = i0 + threadIdx.x; i < i1; i += kTB) {
        const int lab = (int)(list[i] >> 32);
        r0 += lab < cmn;
        r1 += lab < cmx;
    }
    r0 = __reduce_add_sync(kFull, r0);
    r1 = __reduce_add_sync(kFull, r1);
    if (lane == 0) {
        red[0][warp] = r0;
        red[1][warp] = r1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int a0 = 0, a1 = 0;
        for (int w = 0; w < kNW; ++w) {
            a0 += red[0][w];
            a1 += red[1][w];
        }
        atomicAdd(&st.rmin, a0);
        atomicAdd(&st.rmax, a1);
    }
}

// One warp per big vertex: fold its partitions' summaries; when every distinct label is
// a candidate the ranks are 0 and d - 1.
__global__ void big_combine_kernel(IterArgs p)
{
    if (!ctl_active(p.ctl)) return;
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < p.nbig; i += nw) {
        const int bi = p.b0 + i;
        int W = 0, k = 0, mn = INT_MAX, mx = -1;
        for (int c = p.hub_p0[bi] + lane; c < p.hub_p0[bi + 1]; c += 32) {
            const int4 o = p.psum[c];
            if (o.x > W) {
                W = o.x;
                k = o.y;
                mn = o.z;
                mx = o.w;
            } else if (o.x == W) {
                k += o.y;
                mn = min(mn, o.z);
                mx = max(mx, o.w);
            }
        }
        const int Ww = __reduce_max_sync(kFull, W);
        const bool top = W == Ww;
        k = __reduce_add_sync(kFull, top ? k : 0);
        mn = __reduce_min_sync(kFull, top ? mn : INT_MAX);
        mx = __reduce_max_sync(kFull, top ? mx : -1);
        if (lane == 0) {
            BigStat &st = p.bstat[bi];
            st.W = Ww;
            st.k = k;
            st.cmin = mn;
            st.cmax = mx;
            if (k == st.d) {
                st.rmin = 0;
                st.rmax = st.d - 1;
            }
        }
    }
}

// One warp per big vertex: resolve its winner (its run base is known now), write the
// label and count the change.
__global__ void __launch_bounds__(32) big_resolve_kernel(IterArgs p)
{
    __shared__ int hist[256];
    extern __shared__ uint32_t pick_scratch[];  // kPickScratch entries
    if (!ctl_active(p.ctl)) return;
    if ((int)blockIdx.x >= p.nbig) return;
    const int bi = p.b0 + blockIdx.x;
    BigStat &st = p.bstat[bi];
    const int v = p.big_v[bi];
    const int lane = threadIdx.x;
    const int k = st.k, d = st.d;
    int32_t label;
    if (k == 1) {
        label = st.cmin;
    } else {
        const long long a = p.runbase ? p.runbase[v] : p.big_a[bi];
        const long long N = p.ctl->N;
        SummaryQuery sq(k, d, st.rmin, st.rmax);
        int r = resolve_rank(a, d, N, v == p.last_v, sq);
        if (!sq.fail && r == st.rmin) {
            label = st.cmin;
        } else if (!sq.fail && r == st.rmax) {
            label = st.cmax;
        } else {
            WarpTableQueryT<DenseTable> q{{p.big_list + p.big_ooff[bi]}, d, d, st.W, st.rmin, st.rmax, hist, lane,
                                          pick_scratch};
            if (sq.fail) r = resolve_rank(a, d, N, v == p.last_v, q);
            label = (r == st.rmin) ? st.cmin : (r == st.rmax) ? st.cmax : (int32_t)q.select(r);
        }
    }
    if (lane == 0) {
        const int32_t old = p.lab_in[v];
        p.lab_out[v] = label;
        if (label != old) {
            atomicAdd(&p.ctl->changes, 1ull);
            if (p.changed) p.changed[atomicAdd(&p.ctl->changed_n, 1)] = v;
        }
    }
}

// Reset the per-big-vertex statistics for the next iteration.
__global__ void big_reset_kernel(IterArgs p)
{
    if (!ctl_active(p.ctl)) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < p.nbig; i += gridDim.x * blockDim.x) {
        BigStat &b = p.bstat[p.b0 + i];
        b.d = 0;
        b.W = 0;
        b.k = 0;
        b.cmin = INT_MAX;
        b.cmax = -1;
        b.rmin = 0;
        b.rmax = 0;
    }
}

// End of an iteration: record the change count, apply the early exit
// (DPPBase::run, dpp.cuh:83-90: break once count <= n * 1e-5) and reset the
// per-launch counters.
__global__ void finalize_kernel(Ctl *ctl)
{
    if (ctl->active) {
        const unsigned long long c = ctl->changes;
        if (ctl->iter < 64) ctl->counts[ctl->iter] = c;
        ctl->iter += 1;
        if ((long long)c <= ctl->thr || ctl->iter >= ctl->max_iter) ctl->active = 0;
    }
    ctl->changes = 0;
    ctl->ticket = 0;
}

__global__ void init_labels_kernel(int32_t *lab, int64_t n)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        lab[i] = (int32_t)i;
}

__global__ void init_ctl_kernel(Ctl *ctl, long long thr, int max_iter)
{
    ctl->active = max_iter > 0;
    ctl->iter = 0;
    ctl->err = 0;
    ctl->ticket = 0;
    ctl->changes = 0;
    ctl->N = 0;
    ctl->thr = thr;
    ctl->max_iter = max_iter;
    ctl->changed_n = 0;
    ctl->frontier_off = 0;
    for (int i = 0; i < 64; ++i) ctl->counts[i] = 0;
}

__global__ void init_bigstat_kernel(BigStat *b, int nbig)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nbig; i += gridDim.x * blockDim.x) {
        b[i].d = 0;
        b[i].W = 0;
        b[i].k = 0;
        b[i].cmin = INT_MAX;
        b[i].cmax = -1;
        b[i].rmin = 0;
        b[i].rmax = 0;
    }
}

// Input validation on the device: neighbours in [0, n).  (Offsets are checked on
// the host before the schedule is built.)
__global__ void validate_kernel(const int32_t *nbr, int64_t m, int64_t n, int *bad)
{
    int b = 0;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t x = nbr[e];
        if (x < 0 || (int64_t)x >= n) b = 1;
    }
    if (__any_sync(kFull, b) && (threadIdx.x & 31) == 0) atomicOr(bad, 1);
}

// Out-of-core: validate a streamed batch before its kernels run; a bad neighbour stops
// the run (every later kernel returns at once) and is reported as a format error.
__global__ void validate_batch_kernel(const int32_t *nbr, int64_t cnt, int64_t n, Ctl *ctl)
{
    int b = 0;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < cnt; e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t x = nbr[e];
        if (x < 0 || (int64_t)x >= n) b = 1;
    }
    if (__any_sync(kFull, b) && (threadIdx.x & 31) == 0) {
        atomicOr(&ctl->err, kErrFormat);
        atomicExch(&ctl->active, 0);
    }
}

}  // namespace galp
