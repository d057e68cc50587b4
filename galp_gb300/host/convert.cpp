// convert.cpp -- native converters into galp's two input formats.
//
//   galp_convert edgelist2bin EDGES.txt [OUT.bin] [--one-direction] [--dedup]
//   galp_convert normalize EDGES.txt [GROUND_TRUTH.txt] [--out OUT.txt] [--gt-out OUT_GT.txt]
//
// edgelist2bin replaces the reference's utils/edgelist2bin.cpp:13-65 and normalize
// replaces utils/normalize.py:12-76.  Both read a SNAP-style edge list: one "u v" pair
// per line separated by blanks or tabs, lines starting with '#' skipped, vertex IDs any
// non-negative integers.  Both "normalise" the IDs the same way: the distinct IDs that
// appear, sorted, are renumbered 0..n-1 (so the result has no isolated vertices).
//
// edgelist2bin writes the binary format the loaders read (include/graph.h:119-150):
// int32 pairs (x, y) grouped by x ascending, each group's y ascending.  Every input
// line is an undirected edge; self-loops are dropped.  By default both directions are
// written, which is the format the reference's README describes ("including edges of
// both directions") and its loader expects for a symmetric graph; the reference's
// converter itself writes only x < y (edgelist2bin.cpp:60), which --one-direction
// reproduces byte for byte.  Parallel edges are kept as the reference keeps them
// (std::vector adjacency); --dedup drops them.  Default output: graph.bin, as the
// reference writes.
//
// normalize writes the text format (include/graph.h:166-188): one "x y" line per
// distinct undirected edge with x < y, grouped by x ascending, y ascending (sets, as
// normalize.py uses).  With a ground-truth file of "vertex community" lines it also
// writes one community per line, members renumbered and ascending, communities in the
// order of their first appearance.  Default outputs: normalized_<name> next to the
// input file (normalize.py prefixes the path it was given).
#include <algorithm>
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

namespace {

bool read_all(const char *path, std::vector<char> &buf)
{
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    const long sz = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    buf.resize(sz > 0 ? (size_t)sz : 0);
    const size_t got = sz > 0 ? std::fread(buf.data(), 1, (size_t)sz, f) : 0;
    std::fclose(f);
    return got == buf.size();
}

// Pairs of the edge list; false on a malformed line (reported with its number).
bool parse_pairs(const std::vector<char> &buf, std::vector<int64_t> &us, std::vector<int64_t> &vs)
{
    const char *p = buf.data(), *end = p + buf.size();
    long line = 0;
    while (p < end) {
        ++line;
        const char *eol = (const char *)std::memchr(p, '\n', (size_t)(end - p));
        if (!eol) eol = end;
        const char *q = p;
        while (q < eol && (*q == ' ' || *q == '\t' || *q == '\r')) ++q;
        if (q < eol && *q != '#') {
            int64_t x[2];
            for (int k = 0; k < 2; ++k) {
                while (q < eol && (*q == ' ' || *q == '\t')) ++q;
                if (q >= eol || *q < '0' || *q > '9') {
                    std::fprintf(stderr, "galp_convert: line %ld: expected two non-negative vertex IDs\n", line);
                    return false;
                }
                int64_t v = 0;
                while (q < eol && *q >= '0' && *q <= '9') v = v * 10 + (*q++ - '0');
                x[k] = v;
            }
            us.push_back(x[0]);
            vs.push_back(x[1]);
        }
        p = eol + 1;
    }
    return true;
}

struct Normalised {
    std::vector<int64_t> ids;  // sorted distinct original IDs; new ID = index
    std::vector<int32_t> u, v; // renumbered pairs
};

bool normalise(const std::vector<int64_t> &us, const std::vector<int64_t> &vs, Normalised &out)
{
    out.ids.reserve(us.size() * 2);
    out.ids.insert(out.ids.end(), us.begin(), us.end());
    out.ids.insert(out.ids.end(), vs.begin(), vs.end());
    std::sort(out.ids.begin(), out.ids.end());
    out.ids.erase(std::unique(out.ids.begin(), out.ids.end()), out.ids.end());
    if (out.ids.size() > (size_t)INT32_MAX) {
        std::fprintf(stderr, "galp_convert: more than 2^31-1 vertices\n");
        return false;
    }
    auto id = [&](int64_t x) {
        return (int32_t)(std::lower_bound(out.ids.begin(), out.ids.end(), x) - out.ids.begin());
    };
    out.u.resize(us.size());
    out.v.resize(vs.size());
    for (size_t i = 0; i < us.size(); ++i) {
        out.u[i] = id(us[i]);
        out.v[i] = id(vs[i]);
    }
    return true;
}

// Symmetric adjacency (both directions of every non-loop pair), lists sorted.
void adjacency(const Normalised &g, bool dedup, std::vector<int64_t> &off, std::vector<int32_t> &adj)
{
    const size_t n = g.ids.size();
    off.assign(n + 1, 0);
    for (size_t i = 0; i < g.u.size(); ++i) {
        if (g.u[i] == g.v[i]) continue;
        ++off[(size_t)g.u[i] + 1];
        ++off[(size_t)g.v[i] + 1];
    }
    for (size_t i = 0; i < n; ++i) off[i + 1] += off[i];
    adj.resize((size_t)off[n]);
    std::vector<int64_t> pos(off.begin(), off.end() - 1);
    for (size_t i = 0; i < g.u.size(); ++i) {
        if (g.u[i] == g.v[i]) continue;
        adj[(size_t)pos[(size_t)g.u[i]]++] = g.v[i];
        adj[(size_t)pos[(size_t)g.v[i]]++] = g.u[i];
    }
    size_t w = 0;
    for (size_t x = 0; x < n; ++x) {
        const int64_t a = off[x], b = off[x + 1];
        std::sort(adj.begin() + a, adj.begin() + b);
        const size_t start = w;
        for (int64_t k = a; k < b; ++k)
            if (!dedup || w == start || adj[w - 1] != adj[(size_t)k]) adj[w++] = adj[(size_t)k];
        off[x] = (int64_t)start;
    }
    off[n] = (int64_t)w;
    adj.resize(w);
}

std::string sibling(const std::string &path, const std::string &prefix)
{
    const size_t slash = path.find_last_of('/');
    if (slash == std::string::npos) return prefix + path;
    return path.substr(0, slash + 1) + prefix + path.substr(slash + 1);
}

int edgelist2bin(int argc, char **argv)
{
    const char *in = nullptr, *outp = "graph.bin";
    bool one_dir = false, dedup = false;
    int pos = 0;
    for (int i = 2; i < argc; ++i) {
        if (!std::strcmp(argv[i], "--one-direction")) one_dir = true;
        else if (!std::strcmp(argv[i], "--dedup")) dedup = true;
        else if (pos == 0) { in = argv[i]; ++pos; }
        else if (pos == 1) { outp = argv[i]; ++pos; }
        else return 2;
    }
    if (!in) return 2;
    std::vector<char> buf;
    if (!read_all(in, buf)) {
        std::fprintf(stderr, "galp_convert: cannot read %s: %s\n", in, std::strerror(errno));
        return 1;
    }
    std::vector<int64_t> us, vs;
    if (!parse_pairs(buf, us, vs)) return 1;
    buf.clear();
    buf.shrink_to_fit();
    Normalised g;
    if (!normalise(us, vs, g)) return 1;
    us.clear();
    vs.clear();
    std::vector<int64_t> off;
    std::vector<int32_t> adj;
    adjacency(g, dedup, off, adj);
    FILE *f = std::fopen(outp, "wb");
    if (!f) {
        std::fprintf(stderr, "galp_convert: cannot write %s: %s\n", outp, std::strerror(errno));
        return 1;
    }
    std::vector<int32_t> out;
    out.reserve(1 << 20);
    int64_t pairs = 0;
    for (size_t x = 0; x + 1 < off.size(); ++x) {
        for (int64_t k = off[x]; k < off[x + 1]; ++k) {
            if (one_dir && (int64_t)x >= adj[(size_t)k]) continue;
            out.push_back((int32_t)x);
            out.push_back(adj[(size_t)k]);
            ++pairs;
            if (out.size() >= (1 << 20)) {
                std::fwrite(out.data(), sizeof(int32_t), out.size(), f);
                out.clear();
            }
        }
    }
    std::fwrite(out.data(), sizeof(int32_t), out.size(), f);
    const bool ok = std::fclose(f) == 0;
    std::fprintf(stderr, "galp_convert: %zu vertices, %lld pairs -> %s\n", g.ids.size(), (long long)pairs, outp);
    return ok ? 0 : 1;
}

int normalize(int argc, char **argv)
{
    std::string in, gt, outp, gtoutp;
    for (int i = 2; i < argc; ++i) {
        if (!std::strcmp(argv[i], "--out") && i + 1 < argc) outp = argv[++i];
        else if (!std::strcmp(argv[i], "--gt-out") && i + 1 < argc) gtoutp = argv[++i];
        else if (in.empty()) in = argv[i];
        else if (gt.empty()) gt = argv[i];
        else return 2;
    }
    if (in.empty()) return 2;
    if (outp.empty()) outp = sibling(in, "normalized_");
    std::vector<char> buf;
    if (!read_all(in.c_str(), buf)) {
        std::fprintf(stderr, "galp_convert: cannot read %s: %s\n", in.c_str(), std::strerror(errno));
        return 1;
    }
    std::vector<int64_t> us, vs;
    if (!parse_pairs(buf, us, vs)) return 1;
    Normalised g;
    if (!normalise(us, vs, g)) return 1;
    std::vector<int64_t> off;
    std::vector<int32_t> adj;
    adjacency(g, true, off, adj);
    FILE *f = std::fopen(outp.c_str(), "w");
    if (!f) {
        std::fprintf(stderr, "galp_convert: cannot write %s: %s\n", outp.c_str(), std::strerror(errno));
        return 1;
    }
    for (size_t x = 0; x + 1 < off.size(); ++x)
        for (int64_t k = off[x]; k < off[x + 1]; ++k)
            if ((int64_t)x < adj[(size_t)k]) std::fprintf(f, "%zu %d\n", x, adj[(size_t)k]);
    if (std::fclose(f) != 0) return 1;
    if (gt.empty()) return 0;

    if (gtoutp.empty()) gtoutp = sibling(gt, "normalized_");
    if (!read_all(gt.c_str(), buf)) {
        std::fprintf(stderr, "galp_convert: cannot read %s: %s\n", gt.c_str(), std::strerror(errno));
        return 1;
    }
    std::vector<int64_t> vtx, com;
    if (!parse_pairs(buf, vtx, com)) return 1;
    std::unordered_map<int64_t, size_t> order;  // community -> its first appearance
    std::vector<std::vector<int32_t>> members;
    for (size_t i = 0; i < vtx.size(); ++i) {
        auto it = std::lower_bound(g.ids.begin(), g.ids.end(), vtx[i]);
        if (it == g.ids.end() || *it != vtx[i]) {
            std::fprintf(stderr, "galp_convert: ground truth names vertex %lld, which has no edge\n",
                         (long long)vtx[i]);
            return 1;
        }
        auto ins = order.emplace(com[i], members.size());
        if (ins.second) members.emplace_back();
        members[ins.first->second].push_back((int32_t)(it - g.ids.begin()));
    }
    f = std::fopen(gtoutp.c_str(), "w");
    if (!f) return 1;
    for (auto &c : members) {
        std::sort(c.begin(), c.end());
        c.erase(std::unique(c.begin(), c.end()), c.end());
        for (size_t k = 0; k < c.size(); ++k) std::fprintf(f, k ? " %d" : "%d", c[k]);
        std::fputc('\n', f);
    }
    return std::fclose(f) == 0 ? 0 : 1;
}

}  // namespace

int main(int argc, char **argv)
{
    int rc = 2;
    if (argc >= 3 && !std::strcmp(argv[1], "edgelist2bin")) rc = edgelist2bin(argc, argv);
    else if (argc >= 3 && !std::strcmp(argv[1], "normalize")) rc = normalize(argc, argv);
    if (rc == 2)
        std::fprintf(stderr,
                     "usage: galp_convert edgelist2bin EDGES.txt [OUT.bin] [--one-direction] [--dedup]\n"
                     "       galp_convert normalize EDGES.txt [GROUND_TRUTH.txt] [--out OUT] [--gt-out OUT_GT]\n");
    return rc;
}
