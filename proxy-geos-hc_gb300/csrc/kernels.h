// kernels.h -- launch interface between the C ABI (api.cu) and the element-path kernels.
//
// Data layout in HBM (device layout of host_util.h: rows along x padded to nxp, node index
// q = ix + iz*nxp + iy*nxp*nz, padding nodes zero):
//   p[2][n_int]   float   the two pressure levels
//   y[n_int]      float   K.p accumulator of the element path (scratch, zero between steps)
//   a[n_int]      float   dt^2 / M_i (mass with the velocity model folded in)
//   conn[NE][(o+1)^3] int32  element-to-node map in device-layout indices (element path)
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
    float S[6][6];       // 1-D element stiffness S[i][m] = sum_l w_l phi_i'(xi_l) phi_m'(xi_l)
    // SEM_ROUNDING_REFERENCE: the reference's element rows (device, float, layout of
    // reference_element_rows); null: the 1-D stiffness above in difference form
    const float *rtab;
    // > 0: connectivity entries come from the caller and are checked against [0, n_check):
    // an entry outside is never read or written through (its gather reads 0, its scatter is
    // dropped).  0: the library built the map, no checks.
    int64_t n_check;
};

struct UpdateArgs {
    const float *cur;
    float *prev;         // in: stored previous level; out: new level
    float *y;            // read then zeroed
    const float *a;      // dt^2/M
    const float *sx, *sy, *sz;
    int64_t nx, nxp, ny, nz, n_int;
    // receivers, node-sorted, grouped by update block: rec_off[b]..rec_off[b+1]
    const int64_t *rec_node;   // device-layout indices
    const int *rec_perm;
    const int *rec_off;
    int nrec;
    float *traces;       // [step][nrec]
    const int *ctr;      // ctr[1] = index of the step being run
    // SEM_ROUNDING_REFERENCE: the reference's float mass M (launch_mass_ref) and fl(dt*dt); the
    // update then rounds as the reference does.  Null: the precomputed a = dt^2/M.
    const float *mref;
    float dt2f;
};

struct SourceArgs {
    float *cur;
    const int64_t *node;   // device-layout indices
    const float *coef;     // dt^2 c_e^2 per source, rounded as the reference does
    const float *wavelet;  // [nsrc][nsamples]
    int nsrc, nsamples;
    int *ctr;              // ctr[0] = next step index (advanced here), ctr[1] = this step
    int distinct;          // 1: no two sources share a node, so they may be added in parallel
};

constexpr int kUpdateThreads = 256;
constexpr int kUpdateNodesPerThread = 4;
constexpr int64_t kUpdateNodesPerBlock = (int64_t)kUpdateThreads * kUpdateNodesPerThread;
inline int64_t update_grid(int64_t n) { return (n + kUpdateNodesPerBlock - 1) / kUpdateNodesPerBlock; }

cudaError_t launch_element(int order, const ElementArgs &a, cudaStream_t s);  // a.rtab selects the rows
cudaError_t launch_update(const UpdateArgs &a, bool sponge, cudaStream_t s);
cudaError_t launch_source(const SourceArgs &a, cudaStream_t s);
cudaError_t launch_connectivity(int32_t *conn, int ex, int ey, int ez, int order, int64_t nxp,
                                cudaStream_t s);
// Gradient with respect to the nodal mass parameter -> with respect to squared slowness: g /= m.
cudaError_t launch_grad_scale(float *g, const float *a, int ex, int ey, int ez, int order, int64_t nxp,
                              const double *w_dev, double detJ, double dt2, cudaStream_t s);
// a_i = dt^2 / M_i from per-element velocity (vel) or per-node squared slowness (slow2, device
// layout); zero on padding nodes.
cudaError_t launch_mass(float *a, const float *vel, const float *slow2, int ex, int ey, int ez,
                        int order, int64_t nxp, const double *w_dev, double detJ, double dt2,
                        cudaStream_t s);
// The reference's float mass M_i per node from per-element velocity (device layout; padding 1).
cudaError_t launch_mass_ref(float *m, const float *vel, int ex, int ey, int ez, int order, int64_t nxp,
                            const double *w_dev, double detJ, cudaStream_t s);
cudaError_t element_kernel_setup();

}  // namespace semgb
