/*
 * lp_oracle.c -- CPU oracle for galp's method-0 ("DPP") label-propagation update.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links or calls this
 * file: it is the checker that the parity tests, the smoke check and the CPU
 * baseline leg of the benchmark compare the CUDA path against.
 *
 * Two restatements of the same semantics live here:
 *
 *  (1) oracle_perform_lp_literal(): a literal, sequential restatement of
 *      DPPBase::perform_lp (label_propagation/src/dpp/dpp.cuh:104-138) and of
 *      every kernel it launches (src/dpp/kernel.cuh:27-119), with the modified
 *      segmented arg-max of src/common/segmented_reduce.cuh:26-626 emulated at
 *      thread/tile granularity (per-thread register scans, the Hillis-Steele
 *      block scan with its `my_delta` segment heads, the whole-tile tree
 *      reduction, the level-1 spine and the serial level-2 spine).  The
 *      moderngpu segmented sort (dpp/segmented_sort.cuh:35-64) and exclusive
 *      scan (dpp.cuh:118) are replaced by their uniquely defined results
 *      (ascending sort of each vertex's neighbour labels; exclusive integer sum).
 *      TB (threads per block, 256 in the reference) and ET (elements per thread,
 *      17 in the reference) are parameters so that tests can reach every level
 *      of the reduction with small inputs.
 *
 *  (2) oracle_perform_lp_closed(): the same update computed per vertex with the
 *      closed form of the tie-break (cf_winner below), in 64-bit run positions.
 *      It is the oracle for graphs whose run count exceeds int32 and is the
 *      fast CPU restatement used for larger parity cases.
 *
 * Parity pinning: (1) is checked bit-for-bit against the reference's own kernel
 * source (dpp/kernel.cuh + common/segmented_reduce.cuh) executed on the CPU by a
 * SIMT emulation harness (oracle/refsim/), on random graphs and on the committed
 * golden vectors in tests/golden/.  (2) is checked against (1).
 *
 * Degree-0 vertices: the reference's update is undefined for them
 * (set_boundary_case writes flags[offsets[v+1]-1], which is flags[-1] for a
 * leading isolated vertex, and empty segments corrupt the segmented reduce).
 * The literal path rejects them (returns -2).  The closed-form path gives them
 * the semantics the library implements: an isolated vertex keeps its label,
 * owns zero runs, and the "last segment" of a scope is the last vertex that
 * owns runs.  That equals running the reference on the graph with isolated
 * vertices deleted (label order is preserved by the deletion).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int32_t w; /* weight (run length); 0 = identity */
    int64_t x; /* satellite: run index; -1 = identity */
} wx_t;

static const wx_t WX_ID = {0, -1};

/* L: earlier operand wins ties.  R: later operand wins ties. */
static inline wx_t opL(wx_t e, wx_t l) { return (e.w >= l.w) ? e : l; }
static inline wx_t opR(wx_t e, wx_t l) { return (l.w >= e.w) ? l : e; }

static int cmp_i32(const void *a, const void *b)
{
    int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

/* upper_bound over data[0..n) (segmented_reduce.cuh:8-23: binary_search) */
static int64_t upper_bound64(int64_t key, const int64_t *data, int64_t n)
{
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t mid = lo + (hi - lo) / 2;
        if (!(key < data[mid])) lo = mid + 1; else hi = mid;
    }
    return lo;
}

/* Last thread t' <= t whose flag is set, else 0.  This is what the warp/block
 * ballot + __clz sequence computes for `start` (segmented_reduce.cuh:130-157,
 * 330-359, 437-467). */
static void seg_heads_delta(const char *flag, int TB, int *delta)
{
    int last = -1;
    for (int t = 0; t < TB; ++t) {
        if (flag[t]) last = t;
        delta[t] = t - (last >= 0 ? last : 0);
    }
}

/* Hillis-Steele inclusive scan with the "earlier wins ties" update
 * (segmented_reduce.cuh:198-213, 370-385, 480-495).  In-place over v[0..TB). */
static void hs_scan_L(wx_t *v, wx_t *tmp, const int *delta, int TB)
{
    for (int off = 1; off < TB; off += off) {
        for (int t = 0; t < TB; ++t) {
            wx_t s = v[t];
            if (delta[t] >= off && s.w <= v[t - off].w) s = v[t - off];
            tmp[t] = s;
        }
        memcpy(v, tmp, sizeof(wx_t) * (size_t)TB);
    }
}

/*
 * Literal emulation of SegmentedReducer::apply (segmented_reduce.cuh:586-615):
 * block_partition (:26-45), segmented_reduce<TB,ET> (:49-305),
 * segmented_reduce_spine<TB> (:308-411) and segmented_reduce_spine2<TB>
 * (:415-556).  data[N] = run weights, ptr[M] = segment starts.  Writes the
 * reduced (weight, run index) of every segment into dstw/dsts.
 */
static int seg_reduce_literal(const int32_t *data, int64_t N, const int64_t *ptr, int64_t M,
                              int TB, int ET, int32_t *dstw, int64_t *dsts)
{
    const int64_t EB = (int64_t)TB * ET;
    const int64_t BIG = INT64_MAX;
    int64_t nt = (N + EB - 1) / EB;
    int rc = -1;

    int64_t *part = malloc(sizeof(int64_t) * (size_t)(nt + 1));
    char *mid = malloc((size_t)(nt + 1));
    wx_t *carry = malloc(sizeof(wx_t) * (size_t)(nt > 0 ? nt : 1));
    int32_t *reg = malloc(sizeof(int32_t) * (size_t)EB);
    int64_t *segs = malloc(sizeof(int64_t) * (size_t)TB * (ET + 1));
    wx_t *my_scan = malloc(sizeof(wx_t) * (size_t)EB);
    wx_t *v = malloc(sizeof(wx_t) * (size_t)TB);
    wx_t *tmp = malloc(sizeof(wx_t) * (size_t)TB);
    wx_t *loc = malloc(sizeof(wx_t) * (size_t)(EB + 2));
    wx_t *dd = malloc(sizeof(wx_t) * (size_t)TB);
    int64_t *s1 = malloc(sizeof(int64_t) * (size_t)TB);
    int64_t *s2 = malloc(sizeof(int64_t) * (size_t)TB);
    char *flag = malloc((size_t)TB);
    int *delta = malloc(sizeof(int) * (size_t)TB);
    if (!part || !mid || !carry || !reg || !segs || !my_scan || !v || !tmp || !loc || !dd ||
        !s1 || !s2 || !flag || !delta)
        goto out;

    /* block_partition */
    for (int64_t t = 0; t <= nt; ++t) {
        int64_t p = t * EB < N ? t * EB : N;
        if (p == N) {
            part[t] = M;
            mid[t] = 0;
        } else {
            int64_t i = upper_bound64(p, ptr, M) - 1;
            part[t] = i;
            mid[t] = (p != ptr[i]);
        }
    }

    /* segmented_reduce, one tile (= one CUDA block) at a time */
    for (int64_t b = 0; b < nt; ++b) {
        const int64_t tile_offset = EB * b;
        for (int64_t k = 0; k < EB; ++k) reg[k] = (tile_offset + k < N) ? data[tile_offset + k] : 0;

        int64_t seg_begin = part[b];
        int64_t seg_end = part[b + 1];
        int64_t seg_total = seg_end - seg_begin;
        int flush = !mid[b + 1];
        seg_end += !flush;
        int64_t nsegs = seg_end - seg_begin;

        if (seg_total > 0) {
            const int64_t *sh = ptr + seg_begin;
            int64_t end = flush ? (tile_offset + EB) : BIG;
            for (int t = 0; t < TB; ++t) {
                int64_t my_offset = tile_offset + (int64_t)ET * t;
                int64_t seg = upper_bound64(my_offset, sh, nsegs) - 1;
                int64_t next_offset = (seg + 1 < nsegs) ? sh[seg + 1] : end;
                int64_t *sg = segs + (size_t)t * (ET + 1);
                sg[0] = seg;
                for (int i = 1; i <= ET; ++i) {
                    if (my_offset + i == next_offset) {
                        ++seg;
                        next_offset = (seg + 1 < nsegs) ? sh[seg + 1] : end;
                    }
                    sg[i] = seg;
                }
                flag[t] = sg[0] != sg[ET];
            }
            seg_heads_delta(flag, TB, delta);

            /* per-thread scan, strict '<' (leftmost max), reset at segment ends */
            for (int t = 0; t < TB; ++t) {
                int64_t *sg = segs + (size_t)t * (ET + 1);
                wx_t s = WX_ID;
                for (int i = 0; i < ET; ++i) {
                    int64_t k = (int64_t)ET * t + i;
                    wx_t r = {reg[k], tile_offset + k};
                    if (i > 0) {
                        if (s.w < r.w) s = r;
                    } else {
                        s = r;
                    }
                    my_scan[k] = s;
                    if (sg[i] != sg[i + 1]) s = WX_ID;
                }
                v[t] = s;
            }
            hs_scan_L(v, tmp, delta, TB);
            wx_t carry_out = v[TB - 1];
            carry[b] = carry_out;
            for (int t = 0; t < TB; ++t) {
                int64_t *sg = segs + (size_t)t * (ET + 1);
                wx_t ci = t > 0 ? v[t - 1] : WX_ID;
                for (int i = 0; i < ET; ++i) {
                    wx_t ms = my_scan[(int64_t)ET * t + i];
                    wx_t s2v = (ci.w <= ms.w) ? ms : ci;
                    if (sg[i] != sg[i + 1]) {
                        loc[sg[i]] = s2v;
                        ci = WX_ID;
                    }
                }
            }
            for (int64_t i = 0; i < seg_total; ++i) {
                dstw[seg_begin + i] = loc[i].w;
                dsts[seg_begin + i] = loc[i].x;
            }
        } else {
            /* whole tile inside one segment: '<=' everywhere (rightmost max) */
            for (int t = 0; t < TB; ++t) {
                wx_t s = WX_ID;
                for (int i = 0; i < ET; ++i) {
                    int64_t k = (int64_t)ET * t + i;
                    wx_t r = {reg[k], tile_offset + k};
                    if (i > 0) {
                        if (s.w <= r.w) s = r;
                    } else {
                        s = r;
                    }
                }
                v[t] = s;
            }
            for (int i = TB / 2; i >= 1; i >>= 1)
                for (int t = 0; t < i; ++t)
                    if (v[t].w <= v[t + i].w) v[t] = v[t + i];
            carry[b] = v[0];
        }
    }

    /* level-1 spine over blocks of TB tiles */
    int64_t nsb = (nt + TB - 1) / TB;
    wx_t *carry2 = malloc(sizeof(wx_t) * (size_t)(nsb > 0 ? nsb : 1));
    if (!carry2) goto out;
    for (int64_t sb = 0; sb < nsb; ++sb) {
        for (int t = 0; t < TB; ++t) {
            int64_t g = sb * TB + t;
            s1[t] = g < nt ? part[g] : BIG;
            s2[t] = g + 1 < nt ? part[g + 1] : BIG;
            v[t] = g < nt ? carry[g] : WX_ID;
            if (g < nt) {
                dd[t].w = dstw[s1[t]];
                dd[t].x = dsts[s1[t]];
            } else {
                dd[t] = WX_ID;
            }
            flag[t] = s1[t] != s2[t];
        }
        seg_heads_delta(flag, TB, delta);
        hs_scan_L(v, tmp, delta, TB);
        carry2[sb] = v[TB - 1];
        for (int t = TB - 1; t >= 0; --t) {
            if (!flag[t]) continue;
            wx_t s = t ? v[t - 1] : WX_ID;
            wx_t r = (s.w <= dd[t].w) ? dd[t] : s;
            dstw[s1[t]] = r.w;
            dsts[s1[t]] = r.x;
        }
    }

    /* level-2 spine: one block walks the spine blocks in chunks of TB */
    if (nsb > 1) {
        const int64_t eb = TB;
        wx_t s_carry_in = WX_ID;
        int64_t s_carry_in_seg = -1;
        for (int64_t i = 0; i < nsb; i += TB) {
            for (int t = 0; t < TB; ++t) {
                int64_t gid = (i + t) * eb;
                s1[t] = gid < nt ? part[gid] : BIG;
                s2[t] = gid + eb < nt ? part[gid + eb] : BIG;
                if (i + t < nsb) {
                    v[t] = carry2[i + t];
                } else {
                    v[t].w = 0;
                    v[t].x = 0;
                }
                if (gid < nt) {
                    dd[t].w = dstw[s1[t]];
                    dd[t].x = dsts[s1[t]];
                } else {
                    dd[t] = WX_ID;
                }
                flag[t] = s1[t] != s2[t];
            }
            seg_heads_delta(flag, TB, delta);
            hs_scan_L(v, tmp, delta, TB);
            wx_t carry_out = v[TB - 1];
            for (int t = 0; t < TB; ++t) {
                if (!flag[t]) continue;
                wx_t s = t ? v[t - 1] : WX_ID;
                if (i > 0 && s1[t] == s_carry_in_seg) {
                    if (s.w <= s_carry_in.w) s = s_carry_in;
                }
                wx_t r = (s.w <= dd[t].w) ? dd[t] : s;
                dstw[s1[t]] = r.w;
                dsts[s1[t]] = r.x;
            }
            if (i + TB < nsb) {
                int64_t seg2 = s2[TB - 1];
                if (i > 0) {
                    if (s_carry_in_seg == seg2) {
                        if (s_carry_in.w <= carry_out.w) s_carry_in = carry_out;
                    } else {
                        s_carry_in = carry_out;
                    }
                } else {
                    s_carry_in = carry_out;
                }
                s_carry_in_seg = seg2;
            }
        }
    }
    free(carry2);
    rc = 0;
out:
    free(part); free(mid); free(carry); free(reg); free(segs); free(my_scan); free(v); free(tmp);
    free(loc); free(dd); free(s1); free(s2); free(flag); free(delta);
    return rc;
}

/*
 * Literal restatement of DPPBase::perform_lp (dpp.cuh:104-138) for one scope of
 * n vertices whose CSR offsets are rebased to 0 (offsets[0] == 0).  neighbors
 * hold global vertex IDs; labels is the global label array; the scope's
 * vertices are labels[lbl_offset .. lbl_offset+n).  Returns the number of
 * labels that changed (update_labels' counter, kernel.cuh:95-119), -1 on
 * allocation failure, -2 if the scope has a degree-0 vertex.
 */
int64_t oracle_perform_lp_literal(int64_t n, const int64_t *offsets, const int32_t *neighbors,
                                  int32_t *labels, int64_t lbl_offset, int TB, int ET)
{
    if (n <= 0) return 0;
    const int64_t m = offsets[n] - offsets[0];
    for (int64_t v = 0; v < n; ++v)
        if (offsets[v + 1] == offsets[v]) return -2;

    int32_t *adj = malloc(sizeof(int32_t) * (size_t)m);
    int64_t *run = malloc(sizeof(int64_t) * (size_t)(m + 1));
    int64_t *bnd = malloc(sizeof(int64_t) * (size_t)(m + 1));
    int64_t *bo = malloc(sizeof(int64_t) * (size_t)(n + 1));
    int32_t *wts = malloc(sizeof(int32_t) * (size_t)(m + 1));
    int32_t *dstw = malloc(sizeof(int32_t) * (size_t)n);
    int64_t *dsts = malloc(sizeof(int64_t) * (size_t)n);
    int64_t count = -1;
    if (!adj || !run || !bnd || !bo || !wts || !dstw || !dsts) goto out;

    /* gather_labels (kernel.cuh:27-37) */
    for (int64_t e = 0; e < m; ++e) adj[e] = labels[neighbors[e]];
    /* segmented sort, heads = offsets[1..n-1] (dpp.cuh:113) */
    for (int64_t v = 0; v < n; ++v)
        qsort(adj + offsets[v], (size_t)(offsets[v + 1] - offsets[v]), sizeof(int32_t), cmp_i32);
    /* find_boundaries + set_boundary_case (kernel.cuh:41-63); flags[m] is
     * never written by the reference and does not influence an exclusive scan */
    for (int64_t e = 0; e + 1 < m; ++e) run[e] = adj[e] != adj[e + 1];
    for (int64_t v = 0; v < n; ++v) run[offsets[v + 1] - 1] = 1;
    run[m] = 0;
    /* ScanExc over m+1 flags (dpp.cuh:118), in place */
    {
        int64_t acc = 0;
        for (int64_t e = 0; e <= m; ++e) {
            int64_t f = run[e];
            run[e] = acc;
            acc += f;
        }
    }
    /* scatter_indexes (kernel.cuh:66-82) */
    for (int64_t e = 0; e < m; ++e)
        if (run[e] != run[e + 1]) bnd[run[e]] = e;
    bo[0] = 0;
    for (int64_t v = 0; v < n; ++v) bo[v + 1] = run[offsets[v + 1]];
    const int64_t N = bo[n];
    /* compute_label_weights (kernel.cuh:85-92) */
    for (int64_t t = 0; t < N; ++t) wts[t] = (int32_t)(t == 0 ? bnd[t] + 1 : bnd[t] - bnd[t - 1]);

    if (seg_reduce_literal(wts, N, bo, n, TB, ET, dstw, dsts) != 0) goto out;

    /* update_labels (kernel.cuh:95-119) */
    count = 0;
    for (int64_t v = 0; v < n; ++v) {
        int32_t lbl = adj[bnd[dsts[v]]];
        if (lbl != labels[lbl_offset + v]) ++count;
        labels[lbl_offset + v] = lbl;
    }
out:
    free(adj); free(run); free(bnd); free(bo); free(wts); free(dstw); free(dsts);
    return count;
}

/* ---------------------------------------------------------------------- */
/* Closed form of the tie-break                                            */
/* ---------------------------------------------------------------------- */

/* Run weights of a segment, addressed by global run index: at(i) = p[i - base].
 * Only indexes inside the segment being resolved are ever read. */
typedef struct {
    const int32_t *p;
    int64_t base;
} wseg_t;

static inline int32_t wat(wseg_t w, int64_t i) { return w.p[i - w.base]; }

static wx_t lmax_range(wseg_t w, int64_t lo, int64_t hi)
{
    wx_t r = WX_ID;
    for (int64_t i = lo; i < hi; ++i)
        if (wat(w, i) > r.w) { r.w = wat(w, i); r.x = i; }
    return r;
}

/* Whole-tile reduction (segmented_reduce.cuh:263-304): each thread keeps its
 * rightmost maximum ('<=' scan over its ET elements), then a tree over the TB
 * threads combines v[t] with v[t+i] for i = TB/2 .. 1, the higher thread winning
 * ties.  Among the threads that hold the tile maximum this selects the one whose
 * index, bit-reversed over log2(TB) bits, is largest (bit 0 is decided last and
 * prefers 1, then bit 1, ...), not the rightmost one. */
static int64_t bitrev(int64_t t, int TB)
{
    int64_t r = 0;
    for (int b = 1; b < TB; b <<= 1) {
        r = (r << 1) | (t & 1);
        t >>= 1;
    }
    return r;
}

static wx_t tree_pick(wseg_t w, int64_t lo, int TB, int ET)
{
    wx_t r = WX_ID;
    int64_t best_key = -1;
    const int64_t E = (int64_t)TB * ET;
    for (int64_t i = 0; i < E; ++i) {
        const int32_t x = wat(w, lo + i);
        if (x > r.w) {
            r.w = x;
            best_key = -1;
        }
        if (x == r.w) {
            int64_t key = bitrev(i / ET, TB) * ET + (i % ET);
            if (key > best_key) {
                best_key = key;
                r.x = lo + i;
            }
        }
    }
    return r;
}

static inline int64_t max64(int64_t a, int64_t b) { return a > b ? a : b; }
static inline int64_t min64(int64_t a, int64_t b) { return a < b ? a : b; }

/* contribution of an earlier tile j of segment [a, ...): the trailing-partial
 * carry (leftmost max) when the segment starts inside tile j, otherwise the
 * whole-tile tree reduction (tree_pick). */
static wx_t tile_contrib(wseg_t w, int64_t a, int64_t j, int TB, int ET)
{
    const int64_t E = (int64_t)TB * ET;
    if (a > j * E) return lmax_range(w, a, (j + 1) * E);
    return tree_pick(w, j * E, TB, ET);
}

static wx_t tiles_fold_L(wseg_t w, int64_t a, int64_t j0, int64_t j1, int TB, int ET)
{
    wx_t acc = WX_ID;
    for (int64_t j = j0; j < j1; ++j) acc = opL(acc, tile_contrib(w, a, j, TB, ET));
    return acc;
}

/*
 * Winning run index of the segment [a, b) in a scope of N runs, for a reduction
 * with TB threads x ET elements per tile; w_seg[i] is the weight of run a + i.
 * Derived from segmented_reduce.cuh; chunk = ET runs, tile = TB*ET runs,
 * spine block = TB tiles, level-2 chunk = TB spine blocks.  TB must be a power
 * of two.  Every run index it reads lies in [a, b).
 */
int64_t oracle_cf_winner_seg(const int32_t *w_seg, int64_t a, int64_t b, int64_t N, int TB, int ET)
{
    const wseg_t w = {w_seg, a};
    const int64_t C = ET, E = (int64_t)TB * ET, SB = TB, Q = TB;
    const int64_t e = (b == N) ? ((N + E - 1) / E) * E - 1 : b - 1;
    const int64_t ke = e / E, ce = e / C, sb = ke / SB, qe = sb / Q;
    const int64_t ka = a / E;

    wx_t X = lmax_range(w, max64(a, ke * E), min64(ce * C, b));
    wx_t Y = lmax_range(w, max64(a, ce * C), b);
    wx_t d = opR(X, Y);
    if (ka == ke) return d.x;

    wx_t d1 = opR(tiles_fold_L(w, a, max64(ka, sb * SB), ke, TB, ET), d);
    if (ka >= sb * SB) return d1.x;

    const int64_t qa = (ka / SB) / Q;
    wx_t s_in = tiles_fold_L(w, a, max64(ka, qe * Q * SB), sb * SB, TB, ET);
    wx_t s = s_in;
    if (qa < qe) {
        wx_t acc = WX_ID;
        for (int64_t q = qa; q < qe; ++q) {
            wx_t cc = tiles_fold_L(w, a, max64(ka, q * Q * SB), (q + 1) * Q * SB, TB, ET);
            acc = (q == qa) ? cc : opR(acc, cc);
        }
        s = opL(acc, s_in);
    }
    return opR(s, d1).x;
}

/* The same over a scope-wide weight array w[N]. */
int64_t oracle_cf_winner(const int32_t *w, int64_t a, int64_t b, int64_t N, int TB, int ET)
{
    return oracle_cf_winner_seg(w + a, a, b, N, TB, ET);
}

/*
 * Closed-form update of one scope (semantics of oracle_perform_lp_literal,
 * extended to degree-0 vertices as described in the file header).  Run
 * positions are 64-bit.  Returns the change count, -1 on allocation failure.
 */
int64_t oracle_perform_lp_closed(int64_t n, const int64_t *offsets, const int32_t *neighbors,
                                 int32_t *labels, int64_t lbl_offset, int TB, int ET)
{
    if (n <= 0) return 0;
    const int64_t base = offsets[0];
    const int64_t m = offsets[n] - base;
    int32_t *adj = malloc(sizeof(int32_t) * (size_t)(m > 0 ? m : 1));
    int32_t *rl = malloc(sizeof(int32_t) * (size_t)(m > 0 ? m : 1)); /* run labels */
    int32_t *rw = malloc(sizeof(int32_t) * (size_t)(m > 0 ? m : 1)); /* run weights */
    int64_t *ra = malloc(sizeof(int64_t) * (size_t)(n + 1));          /* run base per vertex */
    int32_t *nl = malloc(sizeof(int32_t) * (size_t)n);
    int64_t count = -1;
    if (!adj || !rl || !rw || !ra || !nl) goto out;

    for (int64_t e = 0; e < m; ++e) adj[e] = labels[neighbors[base + e]];
    int64_t N = 0;
    for (int64_t v = 0; v < n; ++v) {
        int64_t lo = offsets[v] - base, hi = offsets[v + 1] - base;
        qsort(adj + lo, (size_t)(hi - lo), sizeof(int32_t), cmp_i32);
        ra[v] = N;
        for (int64_t e = lo; e < hi; ++e) {
            if (e == lo || adj[e] != adj[e - 1]) {
                rl[N] = adj[e];
                rw[N] = 1;
                ++N;
            } else {
                rw[N - 1]++;
            }
        }
    }
    ra[n] = N;
    count = 0;
    for (int64_t v = 0; v < n; ++v) {
        int64_t a = ra[v], b = ra[v + 1];
        int32_t cur = labels[lbl_offset + v];
        nl[v] = (a == b) ? cur : rl[oracle_cf_winner(rw, a, b, N, TB, ET)];
        if (nl[v] != cur) ++count;
    }
    for (int64_t v = 0; v < n; ++v) labels[lbl_offset + v] = nl[v];
out:
    free(adj); free(rl); free(rw); free(ra); free(nl);
    return count;
}

/* Segmented-reduce literal vs closed form on an arbitrary segmentation; used
 * by the tie-break unit tests.  seg_start[M] (ascending, non-empty segments),
 * weights w[N].  Writes the literal winner and the closed-form winner of each
 * segment.  Returns 0 on success. */
int oracle_seg_reduce_check(const int32_t *w, int64_t N, const int64_t *seg_start, int64_t M,
                            int TB, int ET, int64_t *lit_out, int64_t *cf_out)
{
    int32_t *dstw = malloc(sizeof(int32_t) * (size_t)(M > 0 ? M : 1));
    if (!dstw) return -1;
    int rc = seg_reduce_literal(w, N, seg_start, M, TB, ET, dstw, lit_out);
    free(dstw);
    if (rc) return rc;
    for (int64_t s = 0; s < M; ++s) {
        int64_t a = seg_start[s], b = (s + 1 < M) ? seg_start[s + 1] : N;
        cf_out[s] = oracle_cf_winner(w, a, b, N, TB, ET);
    }
    return 0;
}

/* ---------------------------------------------------------------------- */
/* Policies and the run loop                                               */
/* ---------------------------------------------------------------------- */

/*
 * OutOfCore::compute_batch_boundaries (src/common/outofcore.cuh:38-60): batch j
 * is vertices [bbs[j], bbs[j+1]) with fewer than 2^buffer_pow edges.  Returns
 * the number of batches, or -3 when a vertex of degree >= 2^buffer_pow makes the
 * reference loop forever (the reference hangs there; this reports it).
 */
int64_t oracle_batch_boundaries(int64_t n, const int64_t *offsets, int buffer_pow, int64_t *bbs,
                                int64_t cap)
{
    const int64_t B = (int64_t)1 << buffer_pow;
    const int64_t m = offsets[n];
    int64_t nb = 0;
    if (cap < 2) return -1;
    bbs[nb++] = 0;
    int64_t batch_offset = B;
    while (batch_offset < m) {
        int64_t left = 0, right = n + 1;
        while (left < right) {
            int64_t mid = (left + right) / 2;
            if (offsets[mid] < batch_offset) left = mid + 1; else right = mid;
        }
        if (left - 1 <= bbs[nb - 1]) return -3;
        if (nb + 1 >= cap) return -1;
        bbs[nb++] = left - 1;
        batch_offset = offsets[left - 1] + B;
    }
    bbs[nb++] = n;
    return nb - 1;
}

/*
 * DPPBase::run (dpp.cuh:64-102) with InCoreLP (policy 0, common/incore.cuh:41-48)
 * or SyncLP/AsyncLP (policies 1/2, common/sync.cuh:42-59, common/async.cuh:65-89;
 * same labels).  labels_out[n] receives the final labels, counts_out[niter] the
 * per-iteration change counts.  literal != 0 selects the literal reduction
 * (TB/ET as given), else the closed form.  Returns the number of iterations run
 * (with early_exit, the loop breaks once count <= n * 1e-5, dpp.cuh:88; without it,
 * all niter iterations run), or a negative error.
 */
int64_t oracle_run(int64_t n, const int64_t *offsets, const int32_t *neighbors, int niter,
                   int policy, int buffer_pow, int literal, int TB, int ET, int early_exit,
                   int32_t *labels_out, int64_t *counts_out)
{
    for (int64_t i = 0; i < n; ++i) labels_out[i] = (int32_t)i;
    int64_t nb = 1;
    int64_t *bbs = NULL;
    int64_t *loff = NULL;
    if (policy == 1 || policy == 2) {
        bbs = malloc(sizeof(int64_t) * (size_t)(n + 2));
        if (!bbs) return -1;
        nb = oracle_batch_boundaries(n, offsets, buffer_pow, bbs, n + 2);
        if (nb < 0) { free(bbs); return nb; }
        loff = malloc(sizeof(int64_t) * (size_t)(n + 1));
        if (!loff) { free(bbs); return -1; }
    }
    int64_t it;
    for (it = 0; it < niter; ++it) {
        int64_t count = 0;
        if (!bbs) {
            count = literal ? oracle_perform_lp_literal(n, offsets, neighbors, labels_out, 0, TB, ET)
                            : oracle_perform_lp_closed(n, offsets, neighbors, labels_out, 0, TB, ET);
            if (count < 0) return count;
        } else {
            for (int64_t j = 0; j < nb; ++j) {
                int64_t v0 = bbs[j], v1 = bbs[j + 1];
                int64_t bn = v1 - v0;
                int64_t e0 = offsets[v0];
                for (int64_t k = 0; k <= bn; ++k) loff[k] = offsets[v0 + k] - e0;
                int64_t c = literal
                    ? oracle_perform_lp_literal(bn, loff, neighbors + e0, labels_out, v0, TB, ET)
                    : oracle_perform_lp_closed(bn, loff, neighbors + e0, labels_out, v0, TB, ET);
                if (c < 0) { free(bbs); free(loff); return c; }
                count += c;
            }
        }
        counts_out[it] = count;
        if (early_exit && (double)count <= (double)n * 1e-5) { ++it; break; }
    }
    free(bbs);
    free(loff);
    return it;
}
