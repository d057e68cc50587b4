/* galp_gen.h -- seeded synthetic graph generators (C ABI).
 *
 * The reference has no generator: its experiments read SNAP/LFR files
 * (experiments/common.sh:14-17, experiments/lfr.sh:9-20) prepared by its
 * converters (utils/edgelist2bin.cpp:13-65, utils/normalize.py:12-76).  These
 * functions produce graphs in the same prepared form: undirected, simple, both
 * directions, adjacency sorted, isolated vertices deleted and IDs compacted.
 */
#ifndef GALP_GEN_H
#define GALP_GEN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int64_t n;          /* vertices */
    int64_t m;          /* directed CSR entries (2 x undirected edges) */
    int64_t *offsets;   /* n + 1 */
    int32_t *neighbors; /* m */
    int32_t *community; /* n: planted community, or -1 */
} galp_graph;

void galp_graph_free(galp_graph *g);

/* Planted partition: nblocks blocks of the given sizes; each pair inside a
 * block is an edge with probability deg_in/(size-1), each pair across blocks
 * with probability deg_out/(n-size_of_own_block). */
galp_graph *galp_gen_sbm(const int64_t *block_sizes, int32_t nblocks, double deg_in, double deg_out,
                         uint64_t seed);

/* R-MAT with edge_factor * 2^scale sampled edges and quadrant probabilities
 * a, b, c (d = 1-a-b-c). */
galp_graph *galp_gen_rmat(int32_t scale, int64_t edge_factor, double a, double b, double c,
                          uint64_t seed);

/* One R-MAT edge key (u << 32 | v) before symmetrisation; ta/tb/tc are the
 * cumulative quadrant thresholds scaled to 2^32.  Shared with the GPU generator. */
uint64_t galp_rmat_edge(uint64_t seed, uint64_t e, int32_t scale, uint32_t ta, uint32_t tb, uint32_t tc);

/* LFR-style benchmark: power-law degrees (exponent tau1, mean kmean, max kmax),
 * power-law community sizes (exponent tau2 in [cmin, cmax]), mixing mu. */
galp_graph *galp_gen_lfr(int64_t n, double tau1, double kmean, int64_t kmax, double tau2,
                         int64_t cmin, int64_t cmax, double mu, uint64_t seed);

/* .bin: int32 (u, v) pairs, both directions, grouped by u (include/graph.h:119-150). */
int galp_graph_write_bin(const galp_graph *g, const char *path);
/* ground truth: one community per line, space-separated vertex IDs (include/accuracy.h:53-66). */
int galp_graph_write_gt(const galp_graph *g, const char *path);

#ifdef __cplusplus
}
#endif

#endif
