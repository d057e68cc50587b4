/* galp_host.h -- galp's host front end as a C ABI: graph loaders and accuracy measures.
 *
 *   galp_load_graph     CSRGraph<int32,int64>(filename)   (label_propagation/include/graph.h:65-112)
 *                       .txt/.dat: load_edgelist_txt      (graph.h:166-188)
 *                       other:     load_symmetric_edgelist_bin (graph.h:119-150)
 *   galp_nmi            compute_nmi        (include/accuracy.h:49-158)
 *   galp_f_measure      compute_f_measure  (include/accuracy.h:161-236)
 *   galp_ari            compute_ari        (include/accuracy.h:239-319)
 *
 * The loaders produce the same CSR as the reference (same vertex numbering and
 * neighbour order) with bulk reads instead of per-edge stream reads.  Where the
 * reference's behaviour is undefined the loaders define it:
 *   .txt  a line that does not start with two integers is skipped; a source ID above
 *         every target grows the vertex count (the reference writes out of bounds);
 *   .bin  a trailing odd int32 is ignored (the reference re-reads a stale value);
 *   a file name without an extension is read as .bin (the reference throws).
 * The accuracy measures compute the same sums as the reference from a contingency
 * table instead of pairwise set intersections; results agree to rounding (the
 * reference's own OpenMP reductions are order-dependent).
 */
#ifndef GALP_HOST_H
#define GALP_HOST_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int64_t n;          /* vertices */
    int64_t m;          /* CSR entries */
    int64_t *offsets;   /* n + 1 */
    int32_t *neighbors; /* m */
} galp_host_graph;

/* Returns 0 on success, -1 if the file cannot be read, -5 on a malformed file. */
int galp_load_graph(const char *path, galp_host_graph **out);
void galp_host_graph_free(galp_host_graph *g);

/* Ground truth: one community per line, whitespace-separated vertex IDs.
 * Return NaN if the file cannot be read. */
double galp_nmi(const char *gt_path, const int32_t *labels, int64_t n);
double galp_f_measure(const char *gt_path, const int32_t *labels, int64_t n);
double galp_ari(const char *gt_path, const int32_t *labels, int64_t n);

#ifdef __cplusplus
}
#endif

#endif
