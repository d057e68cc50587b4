// ref_harness.cpp -- drive the reference's own method-0 kernels on the CPU.
//
// TEST INFRASTRUCTURE ONLY (part of the oracle; built into oracle/_ref/ by
// oracle/build_ref.sh, and only where the reference sources are present).
//
// The kernels executed here are compiled straight from the reference tree:
//   src/dpp/kernel.cuh               gather_labels, find_boundaries,
//                                    set_boundary_case, scatter_indexes,
//                                    compute_label_weights, update_labels
//   src/common/segmented_reduce.cuh  block_partition, segmented_reduce<TB,ET>,
//                                    segmented_reduce_spine<TB>,
//                                    segmented_reduce_spine2<TB>
//   include/graph.h                  CSRGraph loaders (.txt/.dat/.bin)
//   src/common/outofcore.cuh         OutOfCore batching (policies 1/2)
// through simt_shim.h.  The two moderngpu primitives that the reference calls
// and that are missing from its tree (segmented sort, dpp.cuh:113; exclusive
// scan, dpp.cuh:118) are replaced by std::sort per segment and a sequential
// exclusive sum, whose results are uniquely defined.  The launch sequence
// below mirrors DPPBase::perform_lp (dpp.cuh:104-138), SegmentedReducer::apply
// (segmented_reduce.cuh:586-615) and DPPBase::run (dpp.cuh:64-102).
//
// Usage:
//   ref_harness lp <graph> <policy 0|1|2> <buffer_pow> <niter> <labels_out.bin> <counts_out.txt>
//      labels_out.bin: int32 labels after each executed iteration, concatenated
//   ref_harness segreduce <TB> <ET> <in.bin> <out.bin>
//      in.bin: int64 N, int64 M, int32 w[N], int32 seg_start[M]; out.bin: int32 sat[M]
//   ref_harness csr <graph> <offsets_out.bin> <neighbors_out.bin>    CSRGraph loaders
//   ref_harness acc <ground_truth> <labels.bin>                      compute_nmi/f_measure/ari
// simt_shim.h and the kernel part of segmented_reduce.cuh (everything before
// `struct SegmentedReducer`, whose host code uses <<<>>> launch syntax) are
// force-included by oracle/build_ref.sh ahead of this file.
#include "dpp/kernel.cuh"
#include "graph.h"
#include "accuracy.h"
#include "common/outofcore.cuh"

#include <fstream>
#include <memory>
#include <numeric>

namespace {

inline int divup_i(long x, long y) { return (int)((x + y - 1) / y); }

// SegmentedReducer::apply with the reference kernels, for a given TB/ET.
template <int TB, int ET>
void seg_reduce_apply(int *data, int N, int *ptr, int M, int *dst, int *satellite_dst)
{
    constexpr int EB = TB * ET;
    int num_tiles = (N + EB - 1) / EB;
    int num_tiles2 = (num_tiles + TB - 1) / TB;
    std::vector<int> partitions(num_tiles + 2), carry_outs(num_tiles + 1),
        satellite_carry_outs(num_tiles + 1), carry_outs2(num_tiles2 + 1),
        satellite_carry_outs2(num_tiles2 + 1);
    {
        const int nt = (N + EB - 1) / EB + 1;
        const int nb = (nt + 64 - 1) / 64;
        simt::launch_flat(dim3(nb), dim3(64), [&] {
            block_partition(N, ptr, M, EB, partitions.data(), nt);
        });
    }
    {
        const int nb = (N + EB - 1) / EB;
        simt::launch(dim3(nb), dim3(TB), [&] {
            segmented_reduce<TB, ET>(data, N, ptr, M, partitions.data(), nb, dst, satellite_dst,
                                     carry_outs.data(), satellite_carry_outs.data());
        });
    }
    {
        const int nt = (N + EB - 1) / EB;
        const int nb = (nt + TB - 1) / TB;
        simt::launch(dim3(nb), dim3(TB), [&] {
            segmented_reduce_spine<TB>(partitions.data(), nt, dst, satellite_dst, carry_outs.data(),
                                       satellite_carry_outs.data(), carry_outs2.data(),
                                       satellite_carry_outs2.data());
        });
        if (nb > 1) {
            simt::launch(dim3(1), dim3(TB), [&] {
                segmented_reduce_spine2<TB>(partitions.data(), nb, nt, TB, dst, satellite_dst,
                                            carry_outs2.data(), satellite_carry_outs2.data());
            });
        }
    }
}

// DPPBase::perform_lp for one scope (offsets rebased, int32 as in the reference).
int perform_lp(int n, int m, int *d_offsets, int *d_neighbors, int *d_labels, int lbl_offset)
{
    const int nthreads = 128;
    const int n_blocks = divup_i(n, nthreads);
    const int m_blocks = divup_i(m, nthreads);
    std::vector<int> adj(m + 1), tmp1(m + 1, 0), boundaries(m + 1), boundary_offsets(n + 1),
        weights(m + 1), tmp_labels(n), counter(1, 0);

    simt::launch_flat(dim3(m_blocks), dim3(nthreads), [&] {
        gather_labels(d_neighbors, d_labels, adj.data(), m);
    });
    for (int v = 0; v < n; ++v) std::sort(adj.begin() + d_offsets[v], adj.begin() + d_offsets[v + 1]);
    simt::launch_flat(dim3(m_blocks), dim3(nthreads), [&] { find_boundaries(adj.data(), m, tmp1.data()); });
    simt::launch_flat(dim3(n_blocks), dim3(nthreads), [&] { set_boundary_case(d_offsets, n, tmp1.data()); });
    {
        int acc = 0;
        for (int e = 0; e <= m; ++e) {
            int f = tmp1[e];
            tmp1[e] = acc;
            acc += f;
        }
    }
    simt::launch_flat(dim3(m_blocks), dim3(nthreads), [&] {
        scatter_indexes(tmp1.data(), d_offsets, n, m, boundaries.data(), boundary_offsets.data() + 1);
    });
    simt::launch_flat(dim3(n_blocks), dim3(nthreads), [&] {
        compute_label_weights(boundaries.data(), boundary_offsets.data() + n, weights.data());
    });
    int N = boundary_offsets[n];
    seg_reduce_apply<256, 17>(weights.data(), N, boundary_offsets.data(), n, tmp1.data(),
                              tmp_labels.data());
    // update_labels' own counter is racy in the reference (kernel.cuh:95-119:
    // thread 0 reads s_count without a barrier after the other threads'
    // atomicAdd), so under this scheduler it holds thread 0's contribution
    // only.  The exact number of changed labels is counted here instead, by
    // comparing the scope's labels before and after the kernel.
    std::vector<int> before(d_labels + lbl_offset, d_labels + lbl_offset + n);
    simt::launch(dim3(n_blocks), dim3(nthreads), [&] {
        update_labels(adj.data(), boundaries.data(), tmp_labels.data(), n, d_labels + lbl_offset,
                      counter.data());
    });
    int changed = 0;
    for (int v = 0; v < n; ++v) changed += before[v] != d_labels[lbl_offset + v];
    return changed;
}

int run_lp(const char *graph_file, int policy, int bs, int niter, const char *labels_out,
           const char *counts_out)
{
    using GraphT = CSRGraph<int32_t, int64_t>;
    std::shared_ptr<GraphT> G(new GraphT(graph_file));
    const int n = G->n;
    const long m = G->m;
    std::vector<int> labels(n);
    simt::launch_flat(dim3(divup_i(n, 128)), dim3(128), [&] { initialize_labels(labels.data(), n); });
    std::vector<int> counts;
    std::vector<int> history;  // labels after every iteration, concatenated
    auto snap = [&] { history.insert(history.end(), labels.begin(), labels.end()); };

    if (policy == 0) {
        std::vector<int> offs(n + 1);
        for (int i = 0; i <= n; ++i) offs[i] = (int)G->offsets[i];  // incore.cuh:63-69
        std::vector<int> nbrs(G->neighbors.begin(), G->neighbors.end());
        for (int i = 0; i < niter; ++i) {
            int c = perform_lp(n, (int)m, offs.data(), nbrs.data(), labels.data(), 0);
            counts.push_back(c);
            snap();
            if (c <= n * 1e-5) break;
        }
    } else {
        OutOfCore<int32_t, int64_t> ooc(G, bs);
        ooc.compute_batch_boundaries();
        const int B = 1 << bs;
        std::vector<int> nbuf(B + 1), obuf(n + 2);
        for (int i = 0; i < niter; ++i) {
            int c = 0;
            for (int j = 0; j < ooc.get_num_batches(); ++j) {
                ooc.transfer_batch(j, nbuf.data(), obuf.data());
                c += perform_lp(ooc.get_num_batch_vertices(j), (int)ooc.get_num_batch_edges(j),
                                obuf.data(), nbuf.data(), labels.data(), ooc.bbs[j]);
            }
            counts.push_back(c);
            snap();
            if (c <= n * 1e-5) break;
        }
    }
    std::ofstream lo(labels_out, std::ios::binary);
    lo.write((const char *)history.data(), sizeof(int) * history.size());
    std::ofstream co(counts_out);
    for (int c : counts) co << c << "\n";
    return 0;
}

int run_segreduce(int TB, int ET, const char *in, const char *out)
{
    std::ifstream f(in, std::ios::binary);
    int64_t N = 0, M = 0;
    f.read((char *)&N, 8);
    f.read((char *)&M, 8);
    std::vector<int> w(N + 1), ptr(M + 1), dst(M + 1), sat(M + 1, -7);
    f.read((char *)w.data(), 4 * N);
    f.read((char *)ptr.data(), 4 * M);
    if (TB == 256 && ET == 17) seg_reduce_apply<256, 17>(w.data(), (int)N, ptr.data(), (int)M, dst.data(), sat.data());
    else if (TB == 32 && ET == 3) seg_reduce_apply<32, 3>(w.data(), (int)N, ptr.data(), (int)M, dst.data(), sat.data());
    else if (TB == 32 && ET == 1) seg_reduce_apply<32, 1>(w.data(), (int)N, ptr.data(), (int)M, dst.data(), sat.data());
    else if (TB == 64 && ET == 2) seg_reduce_apply<64, 2>(w.data(), (int)N, ptr.data(), (int)M, dst.data(), sat.data());
    else {
        std::fprintf(stderr, "unsupported TB/ET\n");
        return 2;
    }
    std::ofstream o(out, std::ios::binary);
    o.write((const char *)sat.data(), 4 * M);
    return 0;
}

int run_csr(const char *graph_file, const char *off_out, const char *nbr_out)
{
    CSRGraph<int32_t, int64_t> G(graph_file);
    std::ofstream o(off_out, std::ios::binary);
    o.write((const char *)G.offsets.data(), sizeof(int64_t) * G.offsets.size());
    std::ofstream nb(nbr_out, std::ios::binary);
    nb.write((const char *)G.neighbors.data(), sizeof(int32_t) * G.neighbors.size());
    return 0;
}

int run_acc(const char *gt, const char *labels_file)
{
    std::ifstream f(labels_file, std::ios::binary | std::ios::ate);
    const size_t n = (size_t)f.tellg() / sizeof(int);
    f.seekg(0);
    std::vector<int> labels(n);
    f.read((char *)labels.data(), sizeof(int) * n);
    const double nmi = compute_nmi(gt, labels);
    const double fm = compute_f_measure(gt, labels);
    const double ari = compute_ari(gt, labels);
    std::printf("ACC %.17g %.17g %.17g\n", nmi, fm, ari);
    return 0;
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc >= 5 && std::string(argv[1]) == "csr") return run_csr(argv[2], argv[3], argv[4]);
    if (argc >= 4 && std::string(argv[1]) == "acc") return run_acc(argv[2], argv[3]);
    if (argc >= 8 && std::string(argv[1]) == "lp")
        return run_lp(argv[2], atoi(argv[3]), atoi(argv[4]), atoi(argv[5]), argv[6], argv[7]);
    if (argc >= 6 && std::string(argv[1]) == "segreduce")
        return run_segreduce(atoi(argv[2]), atoi(argv[3]), argv[4], argv[5]);
    std::fprintf(stderr,
                 "usage: ref_harness lp <graph> <policy> <bpow> <niter> <labels.bin> <counts.txt>\n"
                 "       ref_harness segreduce <TB> <ET> <in.bin> <out.bin>\n");
    return 2;
}
