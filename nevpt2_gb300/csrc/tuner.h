// Autotuner of launch parameters (tile shapes, raster orders) for the
// library's own kernels.  A parameter is tuned the first time a call meets a
// new shape while tuning is on (nvpt_set_autotune): every candidate is timed
// with CUDA events on the caller's stream, the fastest is kept, and later
// launches of that shape use it whether tuning is on or not.  The candidates
// of a parameter only change the schedule of independent output tiles, so
// each trial writes the same results.  Choices are kept per device in a
// process-wide table (every context of the process shares them).
#pragma once
#include <cuda_runtime.h>

#include <string>

namespace nvpt {
namespace tune {

bool enabled();
void set_enabled(bool on);
// Cached choice of `key` on the current device, or -1.
int lookup(const std::string &key);
// Times launch(c) for each candidate c (one warm-up launch of the first
// candidate, then one timed launch per candidate; the last launch is of the
// winner, so the caller's outputs hold its result) and caches the fastest.
// Returns the winner.  Without tuning, returns the cached choice or `dflt`
// and launches nothing.
template <class F>
int choose(const std::string &key, const int *cand, int ncand, int dflt, cudaStream_t st, F &&launch);
void record(const std::string &key, int choice, const float *ms, const int *cand, int ncand);
std::string report();
void clear();

template <class F>
int choose(const std::string &key, const int *cand, int ncand, int dflt, cudaStream_t st, F &&launch) {
    const int c = lookup(key);
    if (c >= 0 || !enabled()) return c >= 0 ? c : dflt;
    float ms[16];
    cudaEvent_t a, b;
    if (ncand > 16 || cudaEventCreate(&a) != cudaSuccess) return dflt;
    if (cudaEventCreate(&b) != cudaSuccess) {
        cudaEventDestroy(a);
        return dflt;
    }
    launch(cand[0]);  // warm-up (module load, caches)
    int best = 0;
    for (int i = 0; i < ncand; ++i) {
        cudaEventRecord(a, st);
        launch(cand[i]);
        cudaEventRecord(b, st);
        if (cudaEventSynchronize(b) != cudaSuccess) ms[i] = 1e30f;
        else cudaEventElapsedTime(&ms[i], a, b);
        if (ms[i] < ms[best]) best = i;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (best != ncand - 1) launch(cand[best]);
    record(key, cand[best], ms, cand, ncand);
    return cand[best];
}

}  // namespace tune
}  // namespace nvpt
