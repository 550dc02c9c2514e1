/*
 * autotune.h — launch-configuration autotuner of libflipgpu.
 *
 * A kernel whose results do not depend on its tile shape or schedule (each
 * output's arithmetic is fixed; only the grouping of work changes) offers a
 * list of candidate configurations. The first launch for a key (the kernel
 * and its problem sizes) times every candidate on the caller's stream with
 * CUDA events (one warm-up launch, then the median of three) and keeps the
 * fastest; later launches use it. Nothing is tuned while the stream is
 * being captured into a graph (the default candidate, index 0, runs), and
 * FLIPGPU_AUTOTUNE=0 or flipgpu_set_autotune(0) turns tuning off.
 */
#pragma once
#include <cuda_runtime.h>

#include <functional>
#include <string>
#include <vector>

namespace autotune {

/* index of the configuration to run for key; run(i) launches candidate i */
int choose(const std::string &key, const std::vector<std::string> &names, cudaStream_t st,
           const std::function<cudaError_t(int)> &run);

/* the decision stored for key, or 0 (the default) when there is none; times
 * nothing, so it suits launches that must not wait for the device */
int cached(const std::string &key);

/* enter a decision timed elsewhere (ms < 0: the candidate failed) so that
 * flipgpu_autotune_report lists it */
void record(const std::string &key, const std::vector<std::string> &names,
            const std::vector<float> &ms, int choice);

} // namespace autotune
