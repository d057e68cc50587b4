/* galp.h -- C ABI of galp-gb300, the GB300-native label-propagation update.
 *
 * This is the drop-in boundary for galp's propagator interface.  Each entry point
 * replaces a piece of the reference's C++ class hierarchy:
 *
 *   galp_create      LabelPropagator<V,E> constructor + policy preprocess()
 *                    (label_propagation/include/label_propagator.h:11-34,
 *                     src/common/incore.cuh:33-38 InCoreLP::preprocess,
 *                     src/common/async.cuh:53-62 AsyncLP::preprocess) and the
 *                    method*5+policy factory of src/main.cu:139-207
 *   galp_run         LabelPropagator::run(niter) -> (f1, f2)
 *                    (src/dpp/dpp.cuh:64-102 DPPBase::run)
 *   galp_get_labels  LabelPropagator::get_labels() (include/label_propagator.h:25-29)
 *   galp_destroy     postprocess() + destructor (src/common/incore.cuh:51-55)
 *   galp_run_batch   no reference counterpart: clusters many independent graphs
 *                    (galp_batch_create/_stats/_labels for the same as a context)
 *
 * All arguments are plain pointers and sizes.  The library never calls exit();
 * every entry point returns a status (0 = OK, negative = error, see galp_strerror).
 *
 * Semantics: every method/policy computes galp's method-0 ("DPP") update exactly:
 * each vertex takes the most frequent neighbour label; ties are broken by the
 * reference's segmented arg-max, which depends on the run's global position in the
 * sorted run array (src/common/segmented_reduce.cuh).  Method 1 (the reference's
 * lock-free hash path, src/lfht/) is racy and non-deterministic in the reference;
 * here method 1 selects the hash-based counting kernels and yields the same labels
 * as method 0.  The per-iteration change count is exact (the reference's
 * update_labels counter, src/dpp/kernel.cuh:95-119, reads its shared counter
 * without a barrier and may undercount).  Vertices without neighbours keep their
 * label (the reference's update is undefined for them).
 */
#ifndef GALP_H
#define GALP_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    GALP_OK = 0,
    GALP_EINVAL = -1,      /* bad argument or option */
    GALP_ENOMEM = -2,      /* device or pinned host allocation failed */
    GALP_ECUDA = -3,       /* CUDA runtime error */
    GALP_ETIMEOUT = -4,    /* a device-side wait gave up (watchdog); results invalid */
    GALP_EFORMAT = -5,     /* malformed graph (offsets not monotone, neighbour out of range) */
    GALP_EUNSUPPORTED = -6,/* method/policy combination not provided */
    GALP_ENODEV = -7,      /* no CUDA device */
    GALP_EBATCH = -8       /* out-of-core: a vertex has 2^buffer_pow or more edges */
};

/* Host CSR.  offsets[n+1] (offsets[0] == 0), neighbors[m] with values in [0, n).
 * The caller owns both arrays; for out-of-core policies they must outlive the context. */
typedef struct {
    const int32_t *neighbors;
    const int64_t *offsets;
    int64_t n;
    int64_t m;
} galp_csr;

typedef struct {
    int32_t method;       /* 0 = data-parallel primitives, 1 = lock-free hash (main.cu:114) */
    int32_t policy;       /* 0 = in-core, 1 = out-of-core, 2 = out-of-core with overlap */
    int32_t lfht_policy;  /* -l (main.cu:98-100); reported only */
    int32_t buffer_pow;   /* -b: out-of-core batch buffer 2^buffer_pow edges (main.cu:86-88) */
    int32_t frontier;     /* 1 = skip vertices whose neighbourhood and run base did not change */
    int32_t dispatch;     /* 0 = fixed thresholds, 1 = learned dispatcher */
    int32_t device;       /* CUDA device ordinal */
    int32_t early_exit;   /* 1 = stop when changes <= n * 1e-5 (dpp.cuh:88); 0 = run niter */
} galp_opts;

#define GALP_MAX_ITERS 64

typedef struct {
    double f1;                  /* main loop + final labels to host, seconds (dpp.cuh:78-96) */
    double f2;                  /* f1 + preprocess (allocation, upload), seconds */
    double device_ms;           /* device time of the iteration loop (CUDA events) */
    int32_t iters_run;          /* iterations executed (<= niter) */
    int32_t err;                /* device error bits (0 = none) */
    int64_t updates[GALP_MAX_ITERS]; /* labels changed per iteration */
    int64_t runs_last;          /* runs (distinct labels summed over vertices) in the last iteration */
    int64_t h2d_bytes;          /* bytes copied host -> device by this run */
    int64_t d2h_bytes;          /* bytes copied device -> host by this run */
} galp_stats;

typedef struct galp_ctx galp_ctx;

/* Default options: method 0, policy 0, lfht_policy 1, buffer_pow 24, no frontier,
 * fixed dispatch, device 0, early exit on. */
void galp_default_opts(galp_opts *opts);

int galp_create(const galp_csr *graph, const galp_opts *opts, galp_ctx **ctx);
/* Run up to niter iterations from labels = vertex IDs.  stats may be NULL. */
int galp_run(galp_ctx *ctx, int32_t niter, galp_stats *stats);
/* Copy the labels of the last run into out[n]. */
int galp_get_labels(galp_ctx *ctx, int32_t *out, int64_t n);
void galp_destroy(galp_ctx *ctx);
const char *galp_strerror(int code);

/* Launch on this CUDA stream (cudaStream_t passed as void*) instead of the
 * context's own stream. */
int galp_set_stream(galp_ctx *ctx, void *stream);

/* Enqueue niter iterations from labels = vertex IDs on the context's stream and
 * return without waiting (no host synchronisation, no copies).  Used to time the
 * device loop; galp_run is the complete call. */
int galp_enqueue(galp_ctx *ctx, int32_t niter);
/* Wait for enqueued work and fill stats (iterations, counts, errors). */
int galp_sync(galp_ctx *ctx, galp_stats *stats);

/* Label propagation without device allocation, for callers that cannot call
 * cudaMalloc (a host framework or external allocator owns all device memory, or an
 * allocation's synchronisation is not acceptable on the calling path).  No
 * counterpart in the reference.  Same labels, iteration count and change counts as
 * galp_create + galp_run + galp_get_labels with method 0, policy 0 (computed by a
 * different kernel: one single-pass tile kernel per iteration), but every device
 * buffer lives in one static device array of 12.5 MiB that each GPU loading the
 * library holds until the process exits; nothing is allocated on the device or the
 * host.
 *   graph       host CSR; at most GALP_NOALLOC_MAX_VERTICES vertices, at most
 *               GALP_NOALLOC_MAX_ENTRIES entries, no vertex above 2048 neighbours
 *               (GALP_EUNSUPPORTED otherwise)
 *   labels_out  host int32[n]; stats may be NULL; stream: cudaStream_t or NULL
 * Every call looks up the array's device address (cudaGetSymbolAddress, with the
 * call's device current) and waits for the work it queued before it returns, on
 * success and on error.  Never call it on a stream that is being captured (it copies
 * from pageable memory and synchronises; it returns GALP_EUNSUPPORTED there).  Calls
 * on a device share the array; calls that overlap on the GPU race on it (calls from
 * one process are serialised).  GALP_ETIMEOUT: a look-back wait of the kernel ran out
 * (bounded waits; the kernel returned and the labels are not valid). */
#define GALP_NOALLOC_MAX_VERTICES (1 << 17)
#define GALP_NOALLOC_MAX_ENTRIES (1 << 21)
int galp_run_noalloc(const galp_csr *graph, int32_t niter, int32_t early_exit, int32_t *labels_out,
                     galp_stats *stats, void *stream);

/* Batched mode (no counterpart in the reference): many independent graphs clustered
 * together, each with exactly the labels, iteration count and change counts of its own
 * in-core run (policy 0): labels start at graph-local IDs, run positions and the early
 * exit are per graph, and a graph that has exited keeps its labels while the others go
 * on.  A run is one CUDA-graph launch.  Vertices above 12288 neighbours are not
 * supported here (GALP_EUNSUPPORTED).
 *
 * galp_run_batch: one call over `count` host graphs; labels_out = int32[sum of n] in
 * graph order (graph-local labels), stats = galp_stats[count] or NULL. */
int galp_run_batch(const galp_csr *graphs, int32_t count, const galp_opts *opts, int32_t niter,
                   int32_t *labels_out, galp_stats *stats);
/* The batch as a context: one concatenated CSR (offsets int64[n+1], neighbours with
 * global IDs, host or device pointers), graph g = vertices [graph_v0[g],
 * graph_v0[g+1]) (host array of count+1), no edge leaving its graph.  Run it with
 * galp_run / galp_enqueue; read per-graph results with the two calls below. */
int galp_batch_create(const int64_t *offsets, const int32_t *neighbors, int64_t n, int64_t m,
                      const int64_t *graph_v0, int32_t count, const galp_opts *opts, galp_ctx **out);
int galp_batch_stats(galp_ctx *ctx, int32_t graph, galp_stats *stats);
int galp_batch_labels(galp_ctx *ctx, int32_t graph, int32_t *labels, int64_t n);

/* Host-side evaluation of the tie-break closed form, for tests: winning candidate
 * rank of a vertex with run base a, distinct count d, in a scope of N runs, given
 * its candidate ranks cand[k] (ascending). */
int32_t galp_debug_resolve_rank(int64_t a, int64_t d, int64_t N, int32_t is_last,
                                const int32_t *cand, int32_t k);

#ifdef __cplusplus
}
#endif

#endif
