// cpu_worker_port.cpp -- port of the reference's CPU label update, the timed CPU baseline.
//
// TEST/BENCHMARK INFRASTRUCTURE ONLY (part of the oracle package).
//
// Follows CPUWorker::update_label (label_propagation/src/common/hybrid_cpu_worker.cuh:172-195):
// per vertex, count neighbour labels in a std::map, keep the label whose count
// reaches the running maximum last (`max_count <= c`), write the label in place.
// Driven as CPUWorker::run does (:123-129): `#pragma omp for schedule(dynamic, 1)`
// over the vertices, labels initialised to vertex IDs (:57-61).  The update is
// asynchronous (in place), so its labels differ from the synchronous method-0
// update; it is a speed baseline, not a parity reference.
#include <omp.h>

#include <chrono>
#include <cstdint>
#include <map>

extern "C" {

int cpu_lp_threads(void) { return omp_get_max_threads(); }

// niter sweeps over vertices [v_begin, v_end).  threads <= 0: all available.
// Returns the thread count used; *seconds = wall time of the sweeps.
int64_t cpu_lp_run(int64_t n, const int64_t *offsets, const int32_t *neighbors, int64_t v_begin, int64_t v_end,
                   int64_t niter, int threads, int32_t *labels, int64_t *counts, double *seconds)
{
    if (threads <= 0) threads = omp_get_max_threads();
    for (int64_t i = 0; i < n; ++i) labels[i] = (int32_t)i;
    auto t0 = std::chrono::steady_clock::now();
    for (int64_t it = 0; it < niter; ++it) {
        int64_t nupdated = 0;
#pragma omp parallel num_threads(threads) reduction(+ : nupdated)
        {
#pragma omp for schedule(dynamic, 1) nowait
            for (int64_t v = v_begin; v < v_end; ++v) {
                std::map<int32_t, int> label_count;
                int32_t max_label = labels[v];
                int max_count = 0;
                for (int64_t k = offsets[v]; k < offsets[v + 1]; ++k) {
                    const int32_t label = labels[neighbors[k]];
                    const int c = ++label_count[label];
                    if (max_count <= c) {
                        max_count = c;
                        max_label = label;
                    }
                }
                if (labels[v] != max_label) {
                    labels[v] = max_label;
                    ++nupdated;
                }
            }
        }
        counts[it] = nupdated;
    }
    *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return threads;
}

// The same update restricted to a strided vertex sample: vertices phase, phase + stride,
// phase + 2*stride, ... < n (a sample that covers every degree range in proportion, unlike
// a prefix, which after ID compaction holds R-MAT's hubs).  niter in-place sweeps over
// the sample in ascending order under the same dynamic schedule; labels start from vertex
// IDs; vertices outside the sample keep theirs.  *edges = CSR entries of the sample.
int64_t cpu_lp_run_strided(int64_t n, const int64_t *offsets, const int32_t *neighbors, int64_t stride,
                           int64_t phase, int64_t niter, int threads, int32_t *labels, int64_t *counts,
                           double *seconds, int64_t *edges)
{
    if (threads <= 0) threads = omp_get_max_threads();
    if (stride < 1) stride = 1;
    for (int64_t i = 0; i < n; ++i) labels[i] = (int32_t)i;
    const int64_t ns = phase < n ? (n - phase + stride - 1) / stride : 0;
    int64_t e = 0;
    for (int64_t s = 0; s < ns; ++s) e += offsets[phase + s * stride + 1] - offsets[phase + s * stride];
    *edges = e;
    auto t0 = std::chrono::steady_clock::now();
    for (int64_t it = 0; it < niter; ++it) {
        int64_t nupdated = 0;
#pragma omp parallel num_threads(threads) reduction(+ : nupdated)
        {
#pragma omp for schedule(dynamic, 1) nowait
            for (int64_t s = 0; s < ns; ++s) {
                const int64_t v = phase + s * stride;
                std::map<int32_t, int> label_count;
                int32_t max_label = labels[v];
                int max_count = 0;
                for (int64_t k = offsets[v]; k < offsets[v + 1]; ++k) {
                    const int32_t label = labels[neighbors[k]];
                    const int c = ++label_count[label];
                    if (max_count <= c) {
                        max_count = c;
                        max_label = label;
                    }
                }
                if (labels[v] != max_label) {
                    labels[v] = max_label;
                    ++nupdated;
                }
            }
        }
        counts[it] = nupdated;
    }
    *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return threads;
}

}  // extern "C"
