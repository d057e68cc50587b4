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

}  // extern "C"
