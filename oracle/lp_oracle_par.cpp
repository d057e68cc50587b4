// lp_oracle_par.cpp -- multi-threaded closed-form oracle for the method-0 update.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links or calls this
// file; the parity tests use it to check the CUDA path at the benchmark sizes
// (R-MAT scale 24 and 26, billions of CSR entries), where the sequential
// restatement in lp_oracle.c would take hours.
//
// Semantics are those of oracle_perform_lp_closed / oracle_run in lp_oracle.c,
// which restate DPPBase::perform_lp (label_propagation/src/dpp/dpp.cuh:104-138),
// DPPBase::run (dpp.cuh:64-102) and the out-of-core batching of
// OutOfCore::compute_batch_boundaries / AsyncLP::iterate
// (src/common/outofcore.cuh:38-97, src/common/async.cuh:65-89):
//
//   * per vertex, its neighbours' labels sorted ascending form runs; the runs of
//     a scope (the whole graph in-core, one batch out-of-core) are numbered from 0
//     in vertex order, so vertex v owns runs [a_v, a_v + d_v), a_v = sum of the
//     distinct counts of the scope's earlier vertices;
//   * the new label is the label of the run the reference's segmented arg-max
//     picks (oracle_cf_winner_seg, the closed form of
//     src/common/segmented_reduce.cuh:26-626);
//   * out-of-core batches update in place, in batch order: a batch reads the new
//     labels of the batches before it.
//
// The work is split in two passes so that no run array of the whole scope is
// ever stored (memory stays O(n) plus one buffer per thread):
//   pass 1: distinct count d_v, maximum count W_v and the number of labels k_v
//           reaching it; a vertex with k_v == 1 is decided here (the arg-max of
//           a unique maximum does not depend on positions);
//   scan:   a_v = exclusive sum of d_v (64-bit), N = total runs of the scope;
//   pass 2: tied vertices (k_v > 1) rebuild their runs and apply the closed form.
// Parity: tests/test_oracle.py compares it with oracle_run (closed form and the
// literal emulation) on random graphs, every policy.
#include <omp.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

extern "C" int64_t oracle_cf_winner_seg(const int32_t *w_seg, int64_t a, int64_t b, int64_t N, int TB, int ET);
extern "C" int64_t oracle_batch_boundaries(int64_t n, const int64_t *offsets, int buffer_pow, int64_t *bbs,
                                           int64_t cap);

namespace {

struct Range {
    int64_t v0, v1;
};

// Vertex ranges of about `grain` CSR entries (a vertex above it is a range of its own).
std::vector<Range> plan(int64_t v0, int64_t v1, const int64_t *off, int64_t grain)
{
    std::vector<Range> r;
    int64_t s = v0;
    while (s < v1) {
        int64_t e = s + 1;
        const int64_t lim = off[s] + grain;
        while (e < v1 && off[e + 1] <= lim && e - s < 65536) ++e;
        r.push_back({s, e});
        s = e;
    }
    return r;
}

inline void sort_small(int32_t *p, int64_t d)
{
    if (d <= 24) {
        for (int64_t i = 1; i < d; ++i) {
            int32_t x = p[i];
            int64_t j = i - 1;
            while (j >= 0 && p[j] > x) {
                p[j + 1] = p[j];
                --j;
            }
            p[j + 1] = x;
        }
    } else {
        std::sort(p, p + d);
    }
}

// Gathers and sorts v's neighbour labels into buf; returns the degree.
inline int64_t gather_sorted(int64_t v, const int64_t *off, const int32_t *nbr, const int32_t *lab,
                             std::vector<int32_t> &buf)
{
    const int64_t lo = off[v], d = off[v + 1] - lo;
    if ((int64_t)buf.size() < d) buf.resize((size_t)d);
    int32_t *p = buf.data();
    for (int64_t i = 0; i < d; ++i) p[i] = lab[nbr[lo + i]];
    sort_small(p, d);
    return d;
}

// One synchronous update of scope [v0, v1): reads lab (labels before the scope's
// update), writes out[v - v0].  Returns the number of labels that changed.
int64_t scope_step(int64_t v0, int64_t v1, const int64_t *off, const int32_t *nbr, const int32_t *lab,
                   int32_t *out, int TB, int ET)
{
    const int64_t ns = v1 - v0;
    if (ns <= 0) return 0;
    std::vector<int32_t> dcnt((size_t)ns);
    std::vector<uint8_t> tied((size_t)ns);
    const std::vector<Range> work = plan(v0, v1, off, int64_t(1) << 16);
    const int64_t nw = (int64_t)work.size();

#pragma omp parallel
    {
        std::vector<int32_t> buf;
#pragma omp for schedule(dynamic, 1)
        for (int64_t wi = 0; wi < nw; ++wi) {
            for (int64_t v = work[wi].v0; v < work[wi].v1; ++v) {
                const int64_t i = v - v0;
                const int64_t d = gather_sorted(v, off, nbr, lab, buf);
                if (d == 0) {
                    dcnt[i] = 0;
                    tied[i] = 0;
                    out[i] = lab[v];
                    continue;
                }
                const int32_t *p = buf.data();
                int32_t distinct = 0, W = 0, k = 0, best = 0;
                int64_t s = 0;
                while (s < d) {
                    int64_t e = s + 1;
                    while (e < d && p[e] == p[s]) ++e;
                    const int32_t c = (int32_t)(e - s);
                    ++distinct;
                    if (c > W) {
                        W = c;
                        k = 1;
                        best = p[s];
                    } else if (c == W) {
                        ++k;
                    }
                    s = e;
                }
                dcnt[i] = distinct;
                tied[i] = k > 1;
                out[i] = best;
            }
        }
    }

    std::vector<int64_t> base((size_t)ns + 1);
    int64_t acc = 0;
    for (int64_t i = 0; i < ns; ++i) {
        base[i] = acc;
        acc += dcnt[i];
    }
    base[ns] = acc;
    const int64_t N = acc;

#pragma omp parallel
    {
        std::vector<int32_t> buf, rw, rl;
#pragma omp for schedule(dynamic, 1)
        for (int64_t wi = 0; wi < nw; ++wi) {
            for (int64_t v = work[wi].v0; v < work[wi].v1; ++v) {
                const int64_t i = v - v0;
                if (!tied[i]) continue;
                const int64_t d = gather_sorted(v, off, nbr, lab, buf);
                const int32_t dc = dcnt[i];
                if ((int64_t)rw.size() < dc) {
                    rw.resize((size_t)dc);
                    rl.resize((size_t)dc);
                }
                const int32_t *p = buf.data();
                int64_t s = 0, r = 0;
                while (s < d) {
                    int64_t e = s + 1;
                    while (e < d && p[e] == p[s]) ++e;
                    rl[(size_t)r] = p[s];
                    rw[(size_t)r] = (int32_t)(e - s);
                    ++r;
                    s = e;
                }
                const int64_t a = base[i];
                const int64_t x = oracle_cf_winner_seg(rw.data(), a, a + dc, N, TB, ET);
                out[i] = rl[(size_t)(x - a)];
            }
        }
    }

    int64_t changed = 0;
#pragma omp parallel for reduction(+ : changed) schedule(static)
    for (int64_t i = 0; i < ns; ++i) changed += out[i] != lab[v0 + i];
    return changed;
}

}  // namespace

extern "C" {

int oracle_par_threads(void) { return omp_get_max_threads(); }

// One iteration of the update (policy 0: one scope; policies 1/2: batches of fewer
// than 2^buffer_pow edges, in place, in batch order) applied to labels[n] in place.
// Returns the change count, or a negative error (-3: a vertex does not fit a batch).
int64_t oracle_step_par(int64_t n, const int64_t *offsets, const int32_t *neighbors, int policy, int buffer_pow,
                        int TB, int ET, int32_t *labels, int threads)
{
    if (threads > 0) omp_set_num_threads(threads);
    if (n <= 0) return 0;
    if (policy == 1 || policy == 2) {
        std::vector<int64_t> bbs((size_t)n + 2);
        const int64_t nb = oracle_batch_boundaries(n, offsets, buffer_pow, bbs.data(), n + 2);
        if (nb < 0) return nb;
        std::vector<int32_t> out;
        int64_t count = 0;
        for (int64_t j = 0; j < nb; ++j) {
            const int64_t v0 = bbs[(size_t)j], v1 = bbs[(size_t)j + 1];
            out.resize((size_t)(v1 - v0));
            count += scope_step(v0, v1, offsets, neighbors, labels, out.data(), TB, ET);
            std::memcpy(labels + v0, out.data(), sizeof(int32_t) * (size_t)(v1 - v0));
        }
        return count;
    }
    std::vector<int32_t> out((size_t)n);
    const int64_t count = scope_step(0, n, offsets, neighbors, labels, out.data(), TB, ET);
    std::memcpy(labels, out.data(), sizeof(int32_t) * (size_t)n);
    return count;
}

// DPPBase::run: labels from vertex IDs (init_ids != 0) or as given, up to niter
// iterations, early exit once count <= n * 1e-5 (dpp.cuh:88) when early_exit != 0.
// Returns the number of iterations run, or a negative error.
int64_t oracle_run_par(int64_t n, const int64_t *offsets, const int32_t *neighbors, int niter, int policy,
                       int buffer_pow, int TB, int ET, int early_exit, int init_ids, int32_t *labels,
                       int64_t *counts_out, int threads)
{
    if (init_ids)
        for (int64_t i = 0; i < n; ++i) labels[i] = (int32_t)i;
    int64_t it;
    for (it = 0; it < niter; ++it) {
        const int64_t c = oracle_step_par(n, offsets, neighbors, policy, buffer_pow, TB, ET, labels, threads);
        if (c < 0) return c;
        counts_out[it] = c;
        if (early_exit && (double)c <= (double)n * 1e-5) {
            ++it;
            break;
        }
    }
    return it;
}

}  // extern "C"
