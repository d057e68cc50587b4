// accuracy.cpp -- NMI, F-measure and ARI of a labelling against ground-truth communities.
//
// Same quantities as the reference's include/accuracy.h:
//  * ground truth: line i of the file is community i (a set of vertex IDs);
//  * found clusters: vertices grouped by label (accuracy.h:68-90);
//  * N_ij = |gt_i ∩ found_j|.
//  NMI  (accuracy.h:92-157):  -2 sum N_ij log2(N_ij Nt / (Ni. N.j)) /
//                             (sum Ni. log2(Ni./Nt) + sum N.j log2(N.j/Nt))
//  F    (accuracy.h:204-235): sum_i |gt_i| max_j 2 N_ij / (|gt_i| + |found_j|) / n
//  ARI  (accuracy.h:282-318): Hubert-Arabie adjusted Rand index over N_ij with the
//                             reference's v1/v2/v3 and n = number of labels.
// The reference intersects every pair of sets (O(ca cb min|set|)); here the sparse
// contingency table is built in one pass over the ground-truth members.
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <limits>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/galp_host.h"

namespace {

struct Table {
    int64_t ca = 0, cb = 0;
    std::vector<int64_t> gt_size;                  // |gt_i| (IDs as a set, including IDs >= n)
    std::vector<int64_t> my_size;                  // |found_j|
    std::vector<std::vector<std::pair<int32_t, int64_t>>> rows;  // i -> (j, N_ij), N_ij > 0
};

bool build_table(const char *gt_path, const int32_t *labels, int64_t n, Table &T)
{
    std::ifstream f(gt_path);
    if (!f) return false;
    // found clusters: labels mapped to 0..cb-1 in ascending label order
    std::vector<int32_t> sorted(labels, labels + n);
    std::sort(sorted.begin(), sorted.end());
    sorted.erase(std::unique(sorted.begin(), sorted.end()), sorted.end());
    T.cb = (int64_t)sorted.size();
    std::vector<int32_t> cl((size_t)n);
    T.my_size.assign((size_t)T.cb, 0);
    for (int64_t v = 0; v < n; ++v) {
        cl[(size_t)v] = (int32_t)(std::lower_bound(sorted.begin(), sorted.end(), labels[v]) - sorted.begin());
        T.my_size[(size_t)cl[(size_t)v]]++;
    }
    std::string line;
    std::vector<long long> mem;
    std::unordered_map<int32_t, int64_t> row;
    while (std::getline(f, line)) {
        std::istringstream ss(line);
        mem.clear();
        long long x;
        while (ss >> x) mem.push_back(x);
        std::sort(mem.begin(), mem.end());
        mem.erase(std::unique(mem.begin(), mem.end()), mem.end());
        T.gt_size.push_back((int64_t)mem.size());
        row.clear();
        for (long long v : mem)
            if (v >= 0 && v < n) row[cl[(size_t)v]]++;
        std::vector<std::pair<int32_t, int64_t>> r(row.begin(), row.end());
        std::sort(r.begin(), r.end());
        T.rows.push_back(std::move(r));
    }
    T.ca = (int64_t)T.rows.size();
    return true;
}

}  // namespace

extern "C" {

double galp_nmi(const char *gt_path, const int32_t *labels, int64_t n)
{
    Table T;
    if (!build_table(gt_path, labels, n, T)) return std::numeric_limits<double>::quiet_NaN();
    std::vector<double> Ni((size_t)T.ca, 0.0), Nj((size_t)T.cb, 0.0);
    double Nt = 0.0;
    for (int64_t i = 0; i < T.ca; ++i)
        for (auto &e : T.rows[(size_t)i]) {
            Nt += (double)e.second;
            Ni[(size_t)i] += (double)e.second;
            Nj[(size_t)e.first] += (double)e.second;
        }
    double v1 = 0.0;
    for (int64_t i = 0; i < T.ca; ++i)
        for (auto &e : T.rows[(size_t)i]) {
            const double Nij = (double)e.second;
            v1 += Nij * std::log2((Nij * Nt) / (Ni[(size_t)i] * Nj[(size_t)e.first]));
        }
    v1 *= -2;
    double v2 = 0.0;
    for (double x : Ni)
        if (x > 0.0) v2 += x * std::log2(x / Nt);
    for (double x : Nj)
        if (x > 0.0) v2 += x * std::log2(x / Nt);
    std::printf("%lld, %lld\n", (long long)T.ca, (long long)T.cb);  // as accuracy.h:156
    return v1 / v2;
}

double galp_f_measure(const char *gt_path, const int32_t *labels, int64_t n)
{
    Table T;
    if (!build_table(gt_path, labels, n, T)) return std::numeric_limits<double>::quiet_NaN();
    double v = 0.0;
    for (int64_t i = 0; i < T.ca; ++i) {
        double max_f = 0.0;
        const double gi = (double)T.gt_size[(size_t)i];
        for (auto &e : T.rows[(size_t)i])
            max_f = std::max(max_f, 2.0 * (double)e.second / (gi + (double)T.my_size[(size_t)e.first]));
        v += max_f * gi;
    }
    return v / (double)n;
}

double galp_ari(const char *gt_path, const int32_t *labels, int64_t n)
{
    Table T;
    if (!build_table(gt_path, labels, n, T)) return std::numeric_limits<double>::quiet_NaN();
    double v1 = 0.0, v2 = 0.0, v3 = 0.0;
    std::vector<double> sj((size_t)T.cb, 0.0);
    for (int64_t i = 0; i < T.ca; ++i) {
        double s = 0.0;
        for (auto &e : T.rows[(size_t)i]) {
            const double c = (double)e.second;
            v1 += c * (c - 1.0) / 2.0;
            s += c;
            sj[(size_t)e.first] += c;
        }
        v2 += s * (s - 1.0) / 2.0;
    }
    for (double s : sj) v3 += s * (s - 1.0) / 2.0;
    const double nn = (double)n;
    return (v1 - 2.0 * v2 * v3 / (nn * (nn - 1.0))) / ((v2 + v3) / 2.0 - 2.0 * v2 * v3 / (nn * (nn - 1.0)));
}

}  // extern "C"
