// kernels.h -- launch interface between the C ABI (api.cu) and the device kernels.
//
// Data layout in HBM (reference node numbering, node = ix + iz*nx + iy*nx*nz):
//   p[2][N4]   float   the two pressure levels (N4 = N rounded up to 4, zero tail)
//   y[N4]      float   K.p accumulator of the element path (scratch, zero between steps)
//   a[N4]      float   dt^2 / M_i (mass with the velocity model folded in)
//   conn[NE][(o+1)^3] int32  element-to-node map (element path only)
//   sx[nx], sy[ny], sz[nz]   float  sponge factors per axis
// The level that a step reads as "previous" is stored without its last sponge factor; the
// step applies s_i when it reads it (fl(s_i * p) is the value the reference would have stored).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace semgb {

// Uniform-box geometry: J = diag(hx/2, hz/2, hy/2) for the reference directions
// (xi1 -> x, xi2 -> z, xi3 -> y).  g[d] = |detJ| / J_dd^2 (the diagonal of B, SEMQkGLIntegrals
// .hpp:344-349); off-diagonal terms are exactly zero on this mesh.
struct Geometry {
    double detJ;
    double g[3];
};

// Per-pencil coefficient table (device, float): tab[d][a + (o+1)*b] = g[d] * w_a * w_b, where
// (a, b) are the two local indices other than direction d in increasing axis order.
int coef_table_size(int order);

struct ElementArgs {
    const int32_t *conn;
    const float *p;      // current level
    float *y;            // accumulator
    const float *tab;    // coef table (device)
    int64_t n_elem;
    float D[6][6];       // D[i][l] = phi_l'(xi_i)
    float w[6];
};

struct UpdateArgs {
    const float *cur;
    float *prev;         // in: stored previous level; out: new level
    float *y;            // read then zeroed (element path)
    const float *a;      // dt^2/M
    const float *sx, *sy, *sz;
    int64_t nx, ny, nz, n;
    // receivers (sorted by node within each block's node range)
    const int64_t *rec_node;
    const int *rec_perm;
    const int *rec_off;  // [grid+1]
    int nrec;
    float *traces;       // [step][nrec]
    const int *ctr;      // ctr[1] = index of the step being run
};

struct SourceArgs {
    float *cur;
    const int64_t *node;
    const float *coef;     // dt^2 c_e^2 per source, rounded as the reference does
    const float *wavelet;  // [nsrc][nsamples]
    int nsrc, nsamples;
    int *ctr;              // ctr[0] = next step index (advanced here), ctr[1] = this step
};

constexpr int kUpdateThreads = 256;
constexpr int kUpdateNodesPerThread = 4;
inline int64_t update_grid(int64_t n)
{
    const int64_t per = (int64_t)kUpdateThreads * kUpdateNodesPerThread;
    return (n + per - 1) / per;
}

cudaError_t launch_element(int order, const ElementArgs &a, cudaStream_t s);
cudaError_t launch_update(const UpdateArgs &a, bool sponge, cudaStream_t s);
cudaError_t launch_source(const SourceArgs &a, cudaStream_t s);
cudaError_t launch_connectivity(int32_t *conn, int ex, int ey, int ez, int order, cudaStream_t s);
// a_i = dt^2 / M_i from per-element velocity (vel) or per-node squared slowness (slow2).
cudaError_t launch_mass(float *a, const float *vel, const float *slow2, int ex, int ey, int ez,
                        int order, const double *w_dev, double detJ, double dt2, cudaStream_t s);
cudaError_t element_kernel_setup();

}  // namespace semgb
