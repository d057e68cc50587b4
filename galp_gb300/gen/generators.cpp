// generators.cpp -- seeded synthetic graphs for galp-gb300.
//
// The reference ships no graphs beyond a 7-vertex sample; its experiments ran on
// SNAP and LFR files that are not available here.  These generators produce the
// benchmark families used to exercise and measure the label-propagation update:
//
//   * planted-partition SBM (Bernoulli edges inside/between equal or given blocks)
//   * an LFR-style benchmark (power-law degrees and community sizes, mixing mu),
//     written from the published model description, not from the LFR code
//   * R-MAT (recursive quadrant sampling, a/b/c/d)
//   * batches of independent SBMs
//
// Every generator emits an undirected simple graph the way the reference's own
// converters prepare inputs (utils/edgelist2bin.cpp:13-65, utils/normalize.py):
// self-loops and duplicate edges removed, both directions stored, adjacency
// sorted by (source, target), and vertices that have no edge deleted with the
// remaining IDs compacted in order.  The reference's .bin loader
// (include/graph.h:119-150) silently renumbers around missing sources and its
// update is undefined on degree-0 vertices, so compaction is part of the format.
//
// Randomness: R-MAT uses a counter-based generator (a SplitMix64 finaliser over
// seed, edge index and level), so a GPU implementation can reproduce it edge for
// edge.  SBM and LFR use a SplitMix64-seeded xoshiro256** stream.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <vector>

#include "../../include/galp_gen.h"
#include "../csrc/rmat_rng.h"

namespace {

inline uint64_t splitmix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

struct Xoshiro {
    uint64_t s[4];
    explicit Xoshiro(uint64_t seed)
    {
        uint64_t z = seed;
        for (auto &w : s) {
            z += 0x9E3779B97F4A7C15ull;
            w = splitmix64(z);
        }
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next()
    {
        const uint64_t r = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    // uniform in [0, 1) with 53 random bits
    double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }
    // uniform integer in [0, n)
    uint64_t below(uint64_t n) { return (uint64_t)(((__uint128_t)next() * n) >> 64); }
};

// LSD radix sort of 64-bit keys, 16 bits per pass.
void radix_sort_u64(std::vector<uint64_t> &a)
{
    std::vector<uint64_t> b(a.size());
    std::vector<size_t> cnt(65536);
    for (int shift = 0; shift < 64; shift += 16) {
        std::fill(cnt.begin(), cnt.end(), 0);
        for (uint64_t x : a) cnt[(x >> shift) & 0xFFFF]++;
        size_t acc = 0;
        for (auto &c : cnt) {
            size_t t = c;
            c = acc;
            acc += t;
        }
        for (uint64_t x : a) b[cnt[(x >> shift) & 0xFFFF]++] = x;
        a.swap(b);
    }
}

galp_graph *alloc_graph(int64_t n, int64_t m)
{
    galp_graph *g = (galp_graph *)std::calloc(1, sizeof(galp_graph));
    if (!g) return nullptr;
    g->n = n;
    g->m = m;
    g->offsets = (int64_t *)std::malloc(sizeof(int64_t) * (size_t)(n + 1));
    g->neighbors = (int32_t *)std::malloc(sizeof(int32_t) * (size_t)(m > 0 ? m : 1));
    g->community = (int32_t *)std::malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    if (!g->offsets || !g->neighbors || !g->community) {
        galp_graph_free(g);
        return nullptr;
    }
    return g;
}

// Undirected edge keys (u<<32 | v, any orientation) over raw IDs [0, n_raw) ->
// compacted, symmetric, deduplicated CSR.  comm_raw[n_raw] (may be null) is
// carried over to the compacted IDs.
galp_graph *finish_graph(std::vector<uint64_t> &keys, int64_t n_raw, const int32_t *comm_raw)
{
    // symmetrise and drop self-loops
    const size_t k0 = keys.size();
    size_t w = 0;
    for (size_t i = 0; i < k0; ++i) {
        uint32_t u = (uint32_t)(keys[i] >> 32), v = (uint32_t)keys[i];
        if (u != v) keys[w++] = keys[i];
    }
    keys.resize(w);
    keys.reserve(2 * w);
    for (size_t i = 0; i < w; ++i) {
        uint32_t u = (uint32_t)(keys[i] >> 32), v = (uint32_t)keys[i];
        keys.push_back(((uint64_t)v << 32) | u);
    }
    radix_sort_u64(keys);
    keys.erase(std::unique(keys.begin(), keys.end()), keys.end());

    // compact away vertices without edges
    std::vector<int32_t> newid((size_t)n_raw, -1);
    for (uint64_t x : keys) newid[x >> 32] = 1;
    int64_t n = 0;
    for (int64_t v = 0; v < n_raw; ++v)
        if (newid[v] >= 0) newid[v] = (int32_t)n++;

    galp_graph *g = alloc_graph(n, (int64_t)keys.size());
    if (!g) return nullptr;
    std::fill(g->offsets, g->offsets + n + 1, 0);
    for (size_t i = 0; i < keys.size(); ++i) {
        int32_t u = newid[keys[i] >> 32], v = newid[(uint32_t)keys[i]];
        g->offsets[u + 1]++;
        g->neighbors[i] = v;  // keys are sorted by (u, v) and the map is monotone
    }
    for (int64_t v = 0; v < n; ++v) g->offsets[v + 1] += g->offsets[v];
    for (int64_t v = 0; v < n_raw; ++v)
        if (newid[v] >= 0) g->community[newid[v]] = comm_raw ? comm_raw[v] : -1;
    return g;
}

// Bernoulli(p) over the pair index range [0, count): append selected indices.
template <class F>
void bernoulli_skip(Xoshiro &rng, uint64_t count, double p, F &&emit)
{
    if (p <= 0.0 || count == 0) return;
    if (p >= 1.0) {
        for (uint64_t i = 0; i < count; ++i) emit(i);
        return;
    }
    const double lq = std::log1p(-p);
    uint64_t i = 0;
    for (;;) {
        double u = rng.uniform();
        double skip = std::floor(std::log1p(-u) / lq);
        if (skip >= (double)(count - i)) return;
        i += (uint64_t)skip;
        emit(i);
        if (++i >= count) return;
    }
}

// unordered pair index -> (i, j), i < j, for pairs within [0, s)
inline void tri_pair(uint64_t idx, uint64_t s, uint64_t &i, uint64_t &j)
{
    // row i holds s-1-i pairs; solve by search on the row start
    double si = (double)s;
    double r = std::floor(((2.0 * si - 1.0) - std::sqrt((2.0 * si - 1.0) * (2.0 * si - 1.0) - 8.0 * (double)idx)) / 2.0);
    uint64_t row = (uint64_t)std::max(0.0, r);
    auto start = [&](uint64_t rr) { return rr * (2 * s - rr - 1) / 2; };
    while (row > 0 && start(row) > idx) --row;
    while (start(row + 1) <= idx) ++row;
    i = row;
    j = row + 1 + (idx - start(row));
}

}  // namespace

extern "C" {

void galp_graph_free(galp_graph *g)
{
    if (!g) return;
    std::free(g->offsets);
    std::free(g->neighbors);
    std::free(g->community);
    std::free(g);
}

galp_graph *galp_gen_sbm(const int64_t *block_sizes, int32_t nblocks, double deg_in, double deg_out,
                         uint64_t seed)
{
    if (nblocks <= 0) return nullptr;
    std::vector<int64_t> start(nblocks + 1, 0);
    for (int b = 0; b < nblocks; ++b) start[b + 1] = start[b] + block_sizes[b];
    const int64_t n = start[nblocks];
    std::vector<int32_t> comm(n);
    for (int b = 0; b < nblocks; ++b)
        for (int64_t v = start[b]; v < start[b + 1]; ++v) comm[v] = b;
    Xoshiro rng(seed);
    std::vector<uint64_t> keys;
    keys.reserve((size_t)(n * (deg_in + deg_out) / 2 * 1.1) + 16);
    for (int b = 0; b < nblocks; ++b) {
        const uint64_t s = (uint64_t)block_sizes[b];
        if (s < 2) continue;
        const double p_in = deg_in / (double)(s - 1);
        bernoulli_skip(rng, s * (s - 1) / 2, p_in, [&](uint64_t idx) {
            uint64_t i, j;
            tri_pair(idx, s, i, j);
            keys.push_back(((uint64_t)(start[b] + i) << 32) | (uint64_t)(start[b] + j));
        });
    }
    for (int b = 0; b < nblocks; ++b) {
        const uint64_t s = (uint64_t)block_sizes[b];
        const uint64_t rest = (uint64_t)(n - start[b + 1]);  // vertices in later blocks
        const uint64_t outside = (uint64_t)(n - (int64_t)s);
        if (s == 0 || rest == 0 || outside == 0) continue;
        const double p_out = deg_out / (double)outside;
        bernoulli_skip(rng, s * rest, p_out, [&](uint64_t idx) {
            uint64_t i = idx / rest, j = idx % rest;
            keys.push_back(((uint64_t)(start[b] + i) << 32) | (uint64_t)(start[b + 1] + j));
        });
    }
    return finish_graph(keys, n, comm.data());
}

galp_graph *galp_gen_rmat(int32_t scale, int64_t edge_factor, double a, double b, double c,
                          uint64_t seed)
{
    const int64_t n_raw = (int64_t)1 << scale;
    const int64_t ne = edge_factor << scale;
    const uint32_t ta = (uint32_t)std::llround(a * 4294967296.0);
    const uint32_t tb = (uint32_t)std::llround((a + b) * 4294967296.0);
    const uint32_t tc = (uint32_t)std::llround((a + b + c) * 4294967296.0);
    std::vector<uint64_t> keys((size_t)ne);
    for (int64_t e = 0; e < ne; ++e) keys[e] = galp_rmat_edge(seed, (uint64_t)e, scale, ta, tb, tc);
    return finish_graph(keys, n_raw, nullptr);
}

uint64_t galp_rmat_edge(uint64_t seed, uint64_t e, int32_t scale, uint32_t ta, uint32_t tb, uint32_t tc)
{
    return galp::rmat_edge_key(seed, e, scale, ta, tb, tc);
}

// Truncated discrete power law on [lo, hi] with exponent tau (P(k) ~ k^-tau).
static int64_t sample_powerlaw(Xoshiro &rng, double tau, double lo, double hi)
{
    double u = rng.uniform();
    double e = 1.0 - tau;
    double x = std::pow(std::pow(lo, e) + u * (std::pow(hi + 1.0, e) - std::pow(lo, e)), 1.0 / e);
    int64_t k = (int64_t)std::floor(x);
    if (k < (int64_t)lo) k = (int64_t)lo;
    if (k > (int64_t)hi) k = (int64_t)hi;
    return k;
}

static double powerlaw_mean(double tau, double lo, double hi)
{
    // mean of floor(x) for the continuous law on [lo, hi+1); numerically
    double e = 1.0 - tau, num = 0, den = 0;
    for (int64_t k = (int64_t)lo; k <= (int64_t)hi; ++k) {
        double p = std::pow(k + 1.0, e) - std::pow((double)k, e);
        num += p * (double)k;
        den += p;
    }
    return num / den;
}

galp_graph *galp_gen_lfr(int64_t n, double tau1, double kmean, int64_t kmax, double tau2,
                         int64_t cmin, int64_t cmax, double mu, uint64_t seed)
{
    Xoshiro rng(seed);
    // choose the minimum degree so that the mean degree is kmean
    double lo = 1.0, hi = (double)kmax;
    for (int it = 0; it < 60; ++it) {
        double mid = 0.5 * (lo + hi);
        if (powerlaw_mean(tau1, mid, (double)kmax) < kmean) lo = mid; else hi = mid;
    }
    const double kmin = 0.5 * (lo + hi);
    std::vector<int64_t> deg(n);
    for (auto &d : deg) d = sample_powerlaw(rng, tau1, kmin, (double)kmax);

    // community sizes summing to n
    std::vector<int64_t> csize;
    int64_t tot = 0;
    while (tot < n) {
        int64_t s = sample_powerlaw(rng, tau2, (double)cmin, (double)cmax);
        if (tot + s > n) s = n - tot;
        csize.push_back(s);
        tot += s;
    }
    if (csize.size() > 1 && csize.back() < cmin) {  // fold a short tail into another block
        int64_t t = csize.back();
        csize.pop_back();
        for (size_t i = 0; t > 0; i = (i + 1) % csize.size()) {
            csize[i]++;
            t--;
        }
    }
    const int32_t nc = (int32_t)csize.size();

    // internal degree of each vertex; assign vertices to communities large enough
    std::vector<int64_t> kin(n);
    for (int64_t v = 0; v < n; ++v) kin[v] = (int64_t)std::llround((1.0 - mu) * (double)deg[v]);
    std::vector<int64_t> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](int64_t x, int64_t y) { return kin[x] > kin[y]; });
    std::vector<int32_t> cidx(nc);
    std::iota(cidx.begin(), cidx.end(), 0);
    std::sort(cidx.begin(), cidx.end(), [&](int32_t x, int32_t y) { return csize[x] > csize[y]; });
    std::vector<int64_t> room(csize.begin(), csize.end());
    std::vector<int32_t> comm(n, -1);
    // largest internal degrees first, each into a random community with room
    // whose size exceeds the internal degree (fall back to the largest with room)
    for (int64_t v : order) {
        int32_t chosen = -1;
        for (int tries = 0; tries < 64 && chosen < 0; ++tries) {
            int32_t c = (int32_t)rng.below((uint64_t)nc);
            if (room[c] > 0 && csize[c] > kin[v]) chosen = c;
        }
        if (chosen < 0)
            for (int32_t c : cidx)
                if (room[c] > 0) { chosen = c; break; }
        comm[v] = chosen;
        room[chosen]--;
        if (kin[v] > csize[chosen] - 1) kin[v] = csize[chosen] - 1;
    }
    // stubs: internal per community, external globally; random matching
    std::vector<std::vector<int64_t>> istubs(nc);
    std::vector<int64_t> estubs;
    for (int64_t v = 0; v < n; ++v) {
        for (int64_t k = 0; k < kin[v]; ++k) istubs[comm[v]].push_back(v);
        for (int64_t k = kin[v]; k < deg[v]; ++k) estubs.push_back(v);
    }
    std::vector<uint64_t> keys;
    auto shuffle = [&](std::vector<int64_t> &s) {
        for (size_t i = s.size(); i > 1; --i) std::swap(s[i - 1], s[rng.below(i)]);
    };
    for (auto &s : istubs) {
        shuffle(s);
        for (size_t i = 0; i + 1 < s.size(); i += 2)
            keys.push_back(((uint64_t)s[i] << 32) | (uint64_t)s[i + 1]);
    }
    shuffle(estubs);
    for (size_t i = 0; i + 1 < estubs.size(); i += 2) {
        int64_t u = estubs[i], v = estubs[i + 1];
        if (comm[u] == comm[v]) {  // try to re-pair with a later stub from another community
            for (size_t j = i + 2; j < std::min(estubs.size(), i + 66); ++j)
                if (comm[estubs[j]] != comm[u]) {
                    std::swap(estubs[i + 1], estubs[j]);
                    break;
                }
            v = estubs[i + 1];
        }
        keys.push_back(((uint64_t)u << 32) | (uint64_t)v);
    }
    return finish_graph(keys, n, comm.data());
}

int galp_graph_write_bin(const galp_graph *g, const char *path)
{
    FILE *f = std::fopen(path, "wb");
    if (!f) return -1;
    std::vector<int32_t> buf;
    buf.reserve(1 << 20);
    for (int64_t u = 0; u < g->n; ++u) {
        for (int64_t e = g->offsets[u]; e < g->offsets[u + 1]; ++e) {
            buf.push_back((int32_t)u);
            buf.push_back(g->neighbors[e]);
            if (buf.size() >= (1 << 20)) {
                if (std::fwrite(buf.data(), 4, buf.size(), f) != buf.size()) { std::fclose(f); return -1; }
                buf.clear();
            }
        }
    }
    if (!buf.empty() && std::fwrite(buf.data(), 4, buf.size(), f) != buf.size()) { std::fclose(f); return -1; }
    return std::fclose(f) == 0 ? 0 : -1;
}

int galp_graph_write_gt(const galp_graph *g, const char *path)
{
    int32_t nc = 0;
    for (int64_t v = 0; v < g->n; ++v) nc = std::max(nc, g->community[v] + 1);
    std::vector<std::vector<int64_t>> members(nc);
    for (int64_t v = 0; v < g->n; ++v)
        if (g->community[v] >= 0) members[g->community[v]].push_back(v);
    FILE *f = std::fopen(path, "w");
    if (!f) return -1;
    for (auto &mem : members) {
        if (mem.empty()) continue;
        for (size_t i = 0; i < mem.size(); ++i) std::fprintf(f, i ? " %lld" : "%lld", (long long)mem[i]);
        std::fprintf(f, "\n");
    }
    return std::fclose(f) == 0 ? 0 : -1;
}

}  // extern "C"
