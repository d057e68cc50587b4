// graph_io.cpp -- .txt/.dat and .bin edge-list loaders producing galp's CSR.
//
// Same CSR as the reference's CSRGraph<int32,int64> (include/graph.h:65-150):
//  * text: every line "u v" appends v to u's list and u to v's list, in file order;
//    the vertex count is one past the largest ID seen; CSR = the lists concatenated
//  * binary: int32 pairs (u, v); a new vertex starts whenever u differs from the
//    previous pair's u (so vertices are numbered by group order, not by u); each
//    pair appends v to the current vertex.
// Files are read in bulk; parsing of the text format is a hand-written integer
// scanner over the whole buffer.
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/galp_host.h"

namespace {

bool read_file(const char *path, std::vector<char> &buf)
{
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    long long len = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (len < 0) {
        std::fclose(f);
        return false;
    }
    buf.resize((size_t)len);
    size_t got = len ? std::fread(buf.data(), 1, (size_t)len, f) : 0;
    std::fclose(f);
    return got == (size_t)len;
}

galp_host_graph *make_graph(int64_t n, int64_t m)
{
    auto *g = (galp_host_graph *)std::calloc(1, sizeof(galp_host_graph));
    if (!g) return nullptr;
    g->n = n;
    g->m = m;
    g->offsets = (int64_t *)std::malloc(sizeof(int64_t) * (size_t)(n + 1));
    g->neighbors = (int32_t *)std::malloc(sizeof(int32_t) * (size_t)(m > 0 ? m : 1));
    if (!g->offsets || !g->neighbors) {
        galp_host_graph_free(g);
        return nullptr;
    }
    return g;
}

// Parse one non-negative or negative decimal integer; returns false if none.
inline bool parse_int(const char *&p, const char *end, long long &out)
{
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\r')) ++p;
    bool neg = false;
    if (p < end && (*p == '-' || *p == '+')) {
        neg = *p == '-';
        ++p;
    }
    if (p >= end || *p < '0' || *p > '9') return false;
    long long v = 0;
    while (p < end && *p >= '0' && *p <= '9') {
        v = v * 10 + (*p - '0');
        ++p;
    }
    out = neg ? -v : v;
    return true;
}

int load_txt(const std::vector<char> &buf, galp_host_graph **out)
{
    std::vector<int32_t> us, vs;
    const char *p = buf.data(), *end = p + buf.size();
    long long maxid = -1;
    while (p < end) {
        const char *line_end = (const char *)std::memchr(p, '\n', (size_t)(end - p));
        if (!line_end) line_end = end;
        const char *q = p;
        long long u, v;
        if (parse_int(q, line_end, u) && parse_int(q, line_end, v)) {
            if (u < 0 || v < 0 || u > INT32_MAX - 1 || v > INT32_MAX - 1) return -5;
            us.push_back((int32_t)u);
            vs.push_back((int32_t)v);
            if (u > maxid) maxid = u;
            if (v > maxid) maxid = v;
        }
        p = line_end + 1;
    }
    const int64_t n = maxid + 1;
    std::vector<int64_t> deg((size_t)n + 1, 0);
    for (size_t i = 0; i < us.size(); ++i) {
        deg[(size_t)us[i] + 1]++;
        deg[(size_t)vs[i] + 1]++;
    }
    for (int64_t i = 0; i < n; ++i) deg[(size_t)i + 1] += deg[(size_t)i];
    galp_host_graph *g = make_graph(n, deg[(size_t)n]);
    if (!g) return -1;
    std::memcpy(g->offsets, deg.data(), sizeof(int64_t) * (size_t)(n + 1));
    // file order per list: line i appends v to u, then u to v
    std::vector<int64_t> cur(deg.begin(), deg.end() - 1);
    for (size_t i = 0; i < us.size(); ++i) {
        g->neighbors[cur[(size_t)us[i]]++] = vs[i];
        g->neighbors[cur[(size_t)vs[i]]++] = us[i];
    }
    *out = g;
    return 0;
}

int load_bin(const std::vector<char> &buf, galp_host_graph **out)
{
    const int64_t ints = (int64_t)(buf.size() / sizeof(int32_t));
    const int64_t pairs = ints / 2;
    const int32_t *a = (const int32_t *)buf.data();
    int64_t n = 0;
    int64_t prev = -1;  // the reference starts from cur = -1
    for (int64_t i = 0; i < pairs; ++i) {
        if (a[2 * i] != prev) {
            ++n;
            prev = a[2 * i];
        }
    }
    galp_host_graph *g = make_graph(n, pairs);
    if (!g) return -1;
    int64_t v = -1;
    prev = -1;
    for (int64_t i = 0; i < pairs; ++i) {
        if (a[2 * i] != prev) {
            g->offsets[++v] = i;
            prev = a[2 * i];
        }
        g->neighbors[i] = a[2 * i + 1];
    }
    g->offsets[n] = pairs;
    *out = g;
    return 0;
}

}  // namespace

extern "C" {

void galp_host_graph_free(galp_host_graph *g)
{
    if (!g) return;
    std::free(g->offsets);
    std::free(g->neighbors);
    std::free(g);
}

int galp_load_graph(const char *path, galp_host_graph **out)
{
    if (!path || !out) return -1;
    *out = nullptr;
    std::vector<char> buf;
    if (!read_file(path, buf)) return -1;
    std::string s(path);
    const size_t dot = s.find_last_of('.');
    const std::string ext = dot == std::string::npos ? std::string() : s.substr(dot);
    if (ext == ".txt" || ext == ".dat") return load_txt(buf, out);
    return load_bin(buf, out);
}

}  // extern "C"
