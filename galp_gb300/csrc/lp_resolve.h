// lp_resolve.h -- closed form of the reference's method-0 tie-break, shared by
// the device kernels and a host-side test hook.
//
// The reference's segmented arg-max (label_propagation/src/common/segmented_reduce.cuh)
// decides ties between equally heavy runs by their global position in the run
// array.  This header states that decision as a function of the run base `a`,
// the distinct count `d`, the scope size `N` and the ranks of the candidate runs.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define GALP_HD __host__ __device__ __forceinline__
#else
#define GALP_HD inline
#endif

namespace galp {

// Reduction geometry of the reference's SegmentedReducer (segmented_reduce.cuh:559-562):
// 256 threads x 17 elements per tile, spine blocks of 256 tiles, level-2 chunks of
// 256 spine blocks.
constexpr int64_t kChunk = 17;
constexpr int64_t kTile = 256 * 17;
constexpr int64_t kSpine = 256;
constexpr int64_t kSpine2 = 256;

GALP_HD int64_t imax64(int64_t a, int64_t b) { return a > b ? a : b; }

// Priority of position i (0 <= i < kTile) inside a tile that lies wholly within one
// vertex's runs.  The reference reduces such a tile (segmented_reduce.cuh:263-304)
// with a per-thread '<=' scan over 17 elements (rightmost maximum of the thread)
// followed by a tree over the 256 threads in which v[t] absorbs v[t+i] for
// i = 128, 64, ..., 1 and the absorbed (higher) thread wins ties.  Among tied
// threads the winner is therefore the one whose index, bit-reversed over 8 bits, is
// largest.  The tied position with the largest key wins.
GALP_HD int tile_priority(int64_t i)
{
    unsigned t = (unsigned)(i / kChunk), r = 0;
    for (int b = 0; b < 8; ++b) {
        r = (r << 1) | (t & 1u);
        t >>= 1;
    }
    return (int)(r * kChunk + (unsigned)(i % kChunk));
}

// Winning candidate rank for a vertex whose runs are [a, a+d) in a scope of N
// runs.  is_last marks the scope's last run-owning vertex: the reference pads
// the last tile with zero-weight elements and closes the last segment at the
// tile's end (segmented_reduce.cuh:102-126), so its chunk/tile geometry uses the
// padded end.  Q answers, over the candidates' ranks (0-based among the vertex's
// distinct labels):
//   first_ge(x):  smallest candidate rank >= x, or -1
//   last_lt(y):   largest candidate rank < y, or -1
//   tile_pick(lo): among candidates with rank in [lo, lo + kTile) (a whole tile), the
//                  one whose position lo' = rank - lo has the largest tile_priority
// Rules (all candidates weigh the same, so every max/argmax step is positional):
//  * in-tile (segmented_reduce :166-257): the leftmost candidate of the last
//    17-run chunk if any, else the leftmost candidate in the rest of the last tile;
//  * earlier tiles: a tile the segment starts inside contributes its leftmost
//    candidate (carry-out of the partial scan, :198-225), a tile wholly inside the
//    segment the candidate of highest tile_priority (the <= tree reduction, :263-304);
//  * level-1 spine (:308-411) takes the last tile's value if it has one, else the
//    first earlier tile (within the same 256-tile spine block) that has a candidate;
//  * level-2 spine (:415-556) the same over spine blocks, except that across
//    chunks of 256 spine blocks the carry keeps the later chunk (:534-543).
template <class Q>
GALP_HD int resolve_rank(int64_t a, int64_t d, int64_t N, bool is_last, Q &q)
{
    const int64_t b = a + d;
    const int64_t e = is_last ? ((N + kTile - 1) / kTile) * kTile - 1 : b - 1;
    const int64_t ke = e / kTile, ce = e / kChunk, sb = ke / kSpine, qe = sb / kSpine2;
    const int64_t ka = a / kTile;

    const int64_t rho = imax64(0, ce * kChunk - a);
    if (rho < d) {
        int r = q.first_ge(rho);
        if (r >= 0) return r;
    }
    const int64_t tau = imax64(0, ke * kTile - a);
    {
        int r = q.first_ge(tau);
        if (r >= 0) return r;
    }
    // no candidate in the last tile: the segment spans earlier tiles (ka < ke)
    auto pick_in_tile = [&](int c) -> int {
        const int64_t j = (a + c) / kTile;
        if (a > j * kTile) return c;           // partial first tile: leftmost candidate
        return q.tile_pick(j * kTile - a);     // whole tile: tree-reduction winner
    };
    const int64_t lo1 = imax64(0, imax64(ka, sb * kSpine) * kTile - a);
    {
        int c = q.first_ge(lo1);
        if (c >= 0 && c < tau) return pick_in_tile(c);
    }
    const int64_t qa = (ka / kSpine) / kSpine2;
    const int64_t chunk_runs = kSpine2 * kSpine * kTile;
    if (qa < qe) {
        int cl = q.last_lt(qe * chunk_runs - a);
        if (cl >= 0) {
            const int64_t qs = (a + cl) / chunk_runs;
            int c = q.first_ge(imax64(0, qs * chunk_runs - a));
            return pick_in_tile(c);
        }
    }
    int c = q.first_ge(imax64(0, qe * chunk_runs - a));
    return pick_in_tile(c);
}

// Query over the summary a counting pass leaves per vertex: candidate count k,
// distinct count d, and the ranks of the smallest and largest candidate.
// Answers exactly when k <= 2 or k == d (every distinct label is a candidate);
// otherwise sets `fail` for the queries it cannot answer.
struct SummaryQuery {
    int k, d, rmin, rmax;
    bool fail;
    GALP_HD SummaryQuery(int k_, int d_, int rmin_, int rmax_) : k(k_), d(d_), rmin(rmin_), rmax(rmax_), fail(false) {}
    GALP_HD int first_ge(int64_t x)
    {
        if (x <= rmin) return rmin;
        if (x > rmax) return -1;
        if (k == 2) return rmax;
        if (k == d) return (int)x;
        fail = true;
        return -1;
    }
    GALP_HD int last_lt(int64_t y)
    {
        if (y > rmax) return rmax;
        if (y <= rmin) return -1;
        if (k == 2) return rmin;
        if (k == d) return (int)(y - 1);
        fail = true;
        return -1;
    }
    GALP_HD int tile_pick(int64_t lo)
    {
        if (k == d) return (int)(lo + kTile - 1);  // every position is a candidate
        if (k <= 2) {
            const bool in0 = rmin >= lo && rmin < lo + kTile, in1 = rmax >= lo && rmax < lo + kTile;
            if (in0 && in1) return tile_priority(rmin - lo) > tile_priority(rmax - lo) ? rmin : rmax;
            if (in0) return rmin;
            if (in1) return rmax;
            return -1;
        }
        fail = true;
        return -1;
    }
};

}  // namespace galp
