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
    int64_t m_big;         /* CSR entries of vertices above 2048 neighbours (global-table path) */
    int64_t npacks;        /* packs of vertices with <= 32 neighbours (one warp each) */
    int64_t nmid;          /* vertices with 33..256 neighbours (one warp each) */
    int64_t nlarge;        /* vertices with 257..2048 neighbours (one CTA each) */
    int64_t nbig;          /* vertices on the global-table path */
    int64_t table_slots;   /* global hash-table slots of those vertices (largest scope) */
    int32_t launches_per_iter; /* kernels launched per iteration (upper bound) */
    int32_t pad;
} galp_sched_info;

typedef struct {
    double pipe_ms;        /* count + scan + resolve kernels: summed device time */
    int32_t pipe_groups;   /* scopes timed */
    int32_t big_pre_groups;
    double big_pre_ms;     /* big_insert + big_stats + big_dcnt: summed device time */
    double big_post_ms;    /* big_resolve + big_clear + big_reset */
    int32_t big_post_groups;
    int32_t pad;
} galp_kernel_times;

int galp_schedule_info(galp_ctx *ctx, galp_sched_info *info);
/* Record CUDA events around each kernel group of every following iteration. */
int galp_profile(galp_ctx *ctx, int32_t enable);
/* Wait for the stream, sum and clear the recorded kernel times. */
int galp_profile_read(galp_ctx *ctx, galp_kernel_times *out);

/* Write nedges raw R-MAT edge keys (u << 32 | v) into device memory d_out, on
 * `stream` (cudaStream_t as void*), with the same sampler as galp_gen_rmat. */
int galp_gen_rmat_keys_device(uint64_t seed, int32_t scale, int64_t nedges, double a, double b, double c,
                              void *d_out, void *stream);

#ifdef __cplusplus
}
#endif

#endif
