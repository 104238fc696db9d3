// batch.h -- the many-shot form's own kernels (k_batch.cu); the step itself is the stencil pass
// over shot-stacked levels (k_stencil.cu with nshot > 1).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "host_util.h"

namespace semgb {

// Launch shape the autotuner picks (sem_batch_autotune): the CTAs of how many consecutive shots
// of a tile run as one thread-block cluster, and the y-chunk length; the stencil pass fixes the
// warps per CTA.
struct BatchTuning {
    int shots_per_cluster = 1;  // 1, 2, 4 or 8 (a divisor of the shot count)
    int warps_per_cta = 4;
    int ychunk = 0;             // planes per CTA along y (0: the stencil pass's own choice)
};

struct BatchSourceArgs {
    float *cur;            // shot-stacked level: shot s at cur + s * shot_stride
    const int64_t *node;   // device-layout node per shot (-1: no source)
    const float *coef;     // dt^2 c_e^2 per shot
    const float *wavelet;  // [nshot][nsamples]
    int nshot, nsamples;
    int64_t shot_stride;
    const int *ctr;
};

// Adds every shot's source sample of the current step, then advances the step counter
// (ctr[1] = step of the level being written, ctr[0] = next step).
cudaError_t launch_batch_source(const BatchSourceArgs &a, int *ctr, cudaStream_t st);

}  // namespace semgb
