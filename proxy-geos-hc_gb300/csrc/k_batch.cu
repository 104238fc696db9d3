// k_batch.cu -- source injection of the many-shot form.  Shot s's source adds
// dt^2 c_e^2 r_s(t_n) at local node 0 of its element (SEMsolver.cpp:39-43 for one shot) in its
// own field of the shot-stacked level.
#include <cuda_runtime.h>

#include "batch.h"

namespace semgb {

namespace {

__global__ void k_batch_source(const BatchSourceArgs a)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = a.ctr[0];
    if (s < a.nshot && n < a.nsamples && a.node[s] >= 0)
        a.cur[(int64_t)s * a.shot_stride + a.node[s]] += a.coef[s] * a.wavelet[(int64_t)s * a.nsamples + n];
}

// Advances the step counter after the source launch (blocks of k_batch_source all read it).
__global__ void k_batch_tick(int *ctr)
{
    ctr[1] = ctr[0];
    ctr[0] = ctr[0] + 1;
}

}  // namespace

cudaError_t launch_batch_source(const BatchSourceArgs &a, int *ctr, cudaStream_t st)
{
    if (a.nshot > 0) {
        k_batch_source<<<(a.nshot + 127) / 128, 128, 0, st>>>(a);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    k_batch_tick<<<1, 1, 0, st>>>(ctr);
    return cudaGetLastError();
}

}  // namespace semgb
