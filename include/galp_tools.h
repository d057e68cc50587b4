/* galp_tools.h -- measurement and data-generation helpers exported by libgalp.so.
 *
 * None of these has a counterpart in the reference's propagator interface; they
 * serve the benchmark harness (per-kernel device times, schedule sizes for the
 * roofline arithmetic) and build large synthetic graphs on the device.
 */
#ifndef GALP_TOOLS_H
#define GALP_TOOLS_H

#include <stdint.h>

#include "galp.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int64_t n, m;          /* vertices, CSR entries */
    int64_t m_big;         /* CSR entries of vertices above 12288 neighbours (global-table path) */
    int64_t npacks;        /* packs of vertices with <= 32 neighbours (one warp each) */
    int64_t nmid;          /* vertices with 33..256 neighbours (one warp each) */
    int64_t nlarge;        /* vertices with 257..12288 neighbours (one CTA each, on-chip table) */
    int64_t nbig;          /* vertices on the global-table path */
    int64_t table_slots;   /* pair slots of those vertices' hash partitions (largest scope) */
    int32_t launches_per_iter; /* kernels launched per dense iteration (upper bound) */
    int32_t flags;         /* GALP_SCHED_* bits */
    int64_t launches;      /* kernels launched by the context's runs so far (setup excluded) */
    double setup_ms[5];    /* galp_create phases: host schedule, CSR upload, schedule upload and
                              per-vertex state, dispatch preparation, device checks */
} galp_sched_info;

#define GALP_SCHED_SORTED 1     /* every adjacency list strictly increasing */
#define GALP_SCHED_SYMMETRIC 2  /* edge multiset symmetric (checked by an edge checksum) */
#define GALP_SCHED_FRONTIER 4   /* frontier requested and usable (policy 0, symmetric graph) */

typedef struct {
    double pipe_ms;        /* count + scan + resolve kernels: summed device time */
    int32_t pipe_groups;   /* scopes timed */
    int32_t big_pre_groups;
    double big_pre_ms;     /* big_insert + big_stats + big_dcnt: summed device time */
    double big_post_ms;    /* big_resolve + big_clear + big_reset */
    int32_t big_post_groups;
    int32_t first_groups;  /* first-iteration shortcuts timed */
    double first_ms;       /* first_iteration_kernel (labels = IDs, sorted adjacency): summed
                              device time; not part of pipe_ms */
} galp_kernel_times;

typedef struct {
    char name[48];         /* kernel (or "memset") */
    double ms;             /* device time between the events around it, summed */
    int64_t launches;
} galp_kernel_stat;

/* Kernel variant knobs.  Every variant computes the same labels; they differ in speed. */
typedef struct {
    int32_t agg_mode;      /* warp-aggregated table inserts: 0 auto (by last distinct count, default),
                              1 always, 2 never */
    float frontier_frac;   /* fixed rule, frontier mode: an iteration after more than this fraction
                              of labels changed recounts every vertex (default 0.05) */
    float learned_margin;  /* learned rule: predicted log gain needed to leave the fixed rule's
                              choice (default 0.03) */
    int32_t small_sort;    /* vertices of at most 32 neighbours: 2 = one thread per vertex, labels sorted
                              in shared memory (default); 1 = packs of vertices per warp, sort-based
                              counting; 0 = packs per warp, match-based counting */
    int32_t hub_part_shift; /* hubs (above 12288 neighbours) count their labels in degree * 2^shift / 8192
                               hash partitions (default 1); a partition that overflows makes the run
                               redo itself with the shift raised by one (up to 6).  Shift 0 counts a
                               partition in a 1024-thread CTA with a 128 KB table, 1 in 512 threads
                               with 64 KB (three per SM), 2 and above in 256 threads with 32 KB (six) */
    int32_t cta_stage;      /* CTA counting of 257..2048 neighbours: 1 = the next vertex's neighbour IDs
                               staged in shared memory by a bulk copy, 0 = global loads (default: the
                               stage takes unified L1 from the label gathers; 1.7x slower on R-MAT 26) */
    int32_t cta_narrow;     /* 1 = vertices of 257..512 neighbours counted by 64-thread CTAs with 8 KB
                               tables, split off the 128-thread CTA range (default); 0 = all of that
                               range in 128-thread CTAs */
    int32_t mid_sort;       /* vertices of 33..256 neighbours (the warp range): 1 = the segmented
                               sort + reduce way (a 256-key bitonic sort per warp, runs from the
                               sorted keys: the reference's method-0 counting), 0 = hash tables
                               (default) */
} galp_variant;

/* One row of the in-core variant table (every row computes the same labels). */
typedef struct {
    int32_t agg_mode;          /* CTA-table inserts: 1 warp-aggregated, 2 plain */
    int32_t frontier;          /* 1 = skip vertices whose neighbour labels did not change */
    int32_t warp_max_degree;   /* mid vertices up to this degree: one warp each */
    int32_t cta256_max_degree; /* then 256-thread CTAs up to this degree, 1024-thread CTAs above */
    int32_t pos1, pos2;        /* the same split as positions in the degree-sorted mid list */
} galp_dispatch_row;

#define GALP_DISPATCH_FEATURES 24
#define GALP_DISPATCH_HIDDEN 64
#define GALP_DISPATCH_VARIANTS 16

typedef struct {
    int32_t small_blocks_per_sm, mid_blocks_per_sm, resolve_blocks_per_sm, trials;
    float best_ms;         /* probe run time with the chosen shapes */
    int32_t dispatch_row;  /* bucket shapes: the variant row forced on every iteration (degree splits
                              and insert aggregation), or -1 = the per-iteration fixed rule */
} galp_tune_result;

int galp_schedule_info(galp_ctx *ctx, galp_sched_info *info);
/* Gather floor of an in-core context: mean device time (ms, CUDA events on the context's
 * stream) of `reps` passes that stream every neighbour ID of the resident CSR and gather
 * its label, with the loads of the counting kernels and no other work. */
int galp_probe_gather(galp_ctx *ctx, int32_t reps, float *ms_per_pass);
/* Launch-shape autotuner of a batched context (galp_batch_create): times probe runs of
 * niter iterations and keeps the fastest blocks-per-SM of the counting/resolve kernels,
 * then the fastest bucket shapes (degree splits, insert aggregation) among the variant
 * rows against the per-iteration fixed rule. */
int galp_batch_tune(galp_ctx *ctx, int32_t niter, galp_tune_result *res);

/* Per-iteration dispatch: mode 0 = fixed rule (default), 1 = learned MLP (weights: the
 * galp_mlp_size(24, 64, 16) parameters of a galp_mlp, or NULL to keep those loaded; the
 * library's trained weights are loaded by opts.dispatch = 1), 2 = forced_variant every
 * iteration. */
int galp_dispatch_set(galp_ctx *ctx, int32_t mode, int32_t forced_variant, const float *weights, int64_t count);
/* Features (count x 24) and chosen variant (-1 = first-iteration shortcut) of the last
 * run's iterations. */
int galp_dispatch_log(galp_ctx *ctx, float *features, int32_t *variants, int32_t cap_iters, int32_t *count);
int galp_dispatch_table(galp_ctx *ctx, galp_dispatch_row *rows, int32_t cap, int32_t *count);
/* Device time of every in-core iteration since the last call (profile level >= 1). */
int galp_profile_iterations(galp_ctx *ctx, float *ms, int32_t cap, int32_t *count);

/* The dispatcher's network as a trainable object: nin -> nhid -> nhid -> nout, ReLU,
 * masked mean squared error, AdamW; forward, gradient and training run on the GPU. */
typedef struct galp_mlp galp_mlp;
int64_t galp_mlp_size(int32_t nin, int32_t nhid, int32_t nout);
int galp_mlp_create(int32_t nin, int32_t nhid, int32_t nout, uint64_t seed, galp_mlp **out);
int galp_mlp_set_weights(galp_mlp *mlp, const float *w, int64_t count);
int galp_mlp_get_weights(galp_mlp *mlp, float *w, int64_t count);
int galp_mlp_forward(galp_mlp *mlp, const float *x, int32_t batch, float *y);
/* loss and its gradient (parameter layout) on one batch; mask may be NULL (all ones) */
int galp_mlp_loss_grad(galp_mlp *mlp, const float *x, const float *target, const float *mask, int32_t batch,
                       float *loss, float *grad);
/* `steps` full-batch AdamW steps; loss_curve[steps] may be NULL */
int galp_mlp_train(galp_mlp *mlp, const float *x, const float *target, const float *mask, int32_t batch,
                   int32_t steps, float lr, float weight_decay, float *loss_curve);
void galp_mlp_destroy(galp_mlp *mlp);
int galp_set_variant(galp_ctx *ctx, const galp_variant *v);
int galp_get_variant(galp_ctx *ctx, galp_variant *v);
/* Record CUDA events around each kernel group of every following iteration. */
/* 0 = off, 1 = events around kernel groups, 2 = also around every kernel */
int galp_profile(galp_ctx *ctx, int32_t level);
/* Wait for the stream, sum and clear the recorded kernel times. */
int galp_profile_read(galp_ctx *ctx, galp_kernel_times *out);
/* Per-kernel totals since the last call (level 2), in order of first launch; writes up to
 * cap entries and the number of distinct kernels to *count. */
int galp_profile_kernels(galp_ctx *ctx, galp_kernel_stat *out, int32_t cap, int32_t *count);

/* Test hook of galp_run_noalloc's failure detection, process-wide: every look-back wait
 * of later calls gives up after spin_limit polls (<= 0: the default bound), and with
 * wait_unset != 0 the waits expect a status that no tile publishes, so that they run
 * out and the call returns GALP_ETIMEOUT.  (0, 0) restores the defaults. */
int galp_debug_noalloc_lookback(int64_t spin_limit, int32_t wait_unset);

/* Write nedges raw R-MAT edge keys (u << 32 | v) into device memory d_out, on
 * `stream` (cudaStream_t as void*), with the same sampler as galp_gen_rmat. */
int galp_gen_rmat_keys_device(uint64_t seed, int32_t scale, int64_t nedges, double a, double b, double c,
                              void *d_out, void *stream);

#ifdef __cplusplus
}
#endif

#endif
