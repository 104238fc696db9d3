// batch.h -- launch interface of the many-shot step (k_batch.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "host_util.h"

namespace semgb {

// Tuning knobs the autotuner picks (sem_batch_autotune).
struct BatchTuning {
    int shots_per_lane = 1;  // one shot per lane: a warp covers 32 shots
    int warps_per_cta = 8;   // z-rows of one element span per CTA (fixed at 8)
    int ychunk = 0;          // planes per CTA along y, rounded up to whole elements (0: all)
};

struct BatchArgs {
    const float *cur;   // [n_int][s_pad]
    float *prev;        // [n_int][s_pad], in: stored previous level, out: new level
    const float *a;     // [n_int] dt^2/M
    const float *sx, *sy, *sz;
    int64_t nx, nxp, ny, nz, s_pad;
    int ychunk;
    float g[3];
};

struct BatchSourceArgs {
    float *cur;
    const int64_t *node;   // device-layout node per shot (-1: no source)
    const float *coef;     // dt^2 c_e^2 per shot
    const float *wavelet;  // [nshot][nsamples]
    int nshot, nsamples;
    int64_t s_pad;
    const int *ctr;
};

struct BatchRecordArgs {
    const float *level;      // new level [n_int][s_pad]
    const int64_t *rec_node; // device-layout nodes
    int nrec, nshot;
    int64_t s_pad;
    float *traces;           // [step][nrec][nshot]
    const int *ctr;
};

cudaError_t batch_kernel_setup(const float *T_all, const float *wa_all);
cudaError_t launch_batch_step(int order, const BatchArgs &a, bool sponge, const BatchTuning &tune, cudaStream_t st);
cudaError_t launch_batch_source(const BatchSourceArgs &a, int *ctr, cudaStream_t st);
cudaError_t launch_batch_record(const BatchRecordArgs &a, cudaStream_t st);

}  // namespace semgb
