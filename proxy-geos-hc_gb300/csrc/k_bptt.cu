// k_bptt.cu -- the adjoint of the time loop with the boundary network on the boundary nodes
// (layer 0), for training the network through it (sem_abc_bptt).
//
// Forward (stored levels; c = p^n after the source, q = p^{n-1}, s = (sx*sz)*sy per node):
//   interior i:  out_i = s_i ((2 c_i - s_i q_i) - a_i (K c)_i)            (the stencil pass)
//   boundary b:  out_b = N(f_b),  N(f) = scale clip(MLP(f / scale), -1, 1),  scale = max_k |f_k|
//   with the 81 features of b over its 3x3x3 neighbourhood j (the face kernel's):
//     level 0: out_j (j not on the boundary) or s_j (s_j q_j) (j on the boundary: what the step
//              leaves there before the network), level 1: s_j c_j, level 2: s_j q_j.
// Backward, with A0, A1, A2 the adjoints of out^m, out^{m-1}, out^{m-2} (complete for out^m):
//   1. g_b = A0_b; dy_b = g_b scale_b [|y_b| < 1] (N = scale h); the network's backward gives
//      the parameter gradient and dx = dy dy/dx; with d = dx / scale = g dh/dx
//      (h = clip(MLP(x)), x = f / scale) the feature gradient is
//      G_k = d_k + [k = k*] sgn(f_k*) (g h - sum_m x_m d_m)   (scale = |f_k*|);
//   2. G is gathered back (a node collects from the boundary nodes whose neighbourhood holds it,
//      in a fixed order): level 0 -> A0 (j not on the boundary) or s_j^2 A2; level 1 -> s_j A1;
//      level 2 -> s_j A2;
//   3. interior adjoint with lambda = A0 on interior nodes and v = a s lambda:
//      A1_j += 2 s_j lambda_j - (K^T v)_j,  A2_j -= s_j^2 lambda_j.
// K^T is gathered from the rows of K (K_ij from node i's local indices and weights), so the
// rows of the domain's boundary nodes, which the forward never forms, are not needed.
#include <cuda_runtime.h>

#include <algorithm>

#include "mlp.h"

namespace semgb {

namespace {

struct Geo {
    int nx, ny, nz;
    int64_t nxp;
    const float *sx, *sy, *sz;  // null: no sponge
};

__device__ __forceinline__ void coords_of(const Geo &g, int64_t q, int &ix, int &iy, int &iz)
{
    const int64_t plane = g.nxp * g.nz;
    iy = (int)(q / plane);
    const int64_t r = q - (int64_t)iy * plane;
    iz = (int)(r / g.nxp);
    ix = (int)(r - (int64_t)iz * g.nxp);
}

__device__ __forceinline__ int64_t index_of(const Geo &g, int ix, int iy, int iz)
{
    return ix + (int64_t)iz * g.nxp + (int64_t)iy * g.nxp * g.nz;
}

__device__ __forceinline__ float sponge_of(const Geo &g, int ix, int iy, int iz)
{
    return g.sx ? (g.sx[ix] * g.sz[iz]) * g.sy[iy] : 1.f;
}

__device__ __forceinline__ bool inside(const Geo &g, int ix, int iy, int iz)
{
    return ix >= 0 && ix < g.nx && iy >= 0 && iy < g.ny && iz >= 0 && iz < g.nz;
}

__device__ __forceinline__ bool on_boundary(const Geo &g, int ix, int iy, int iz)
{
    return ix == 0 || ix == g.nx - 1 || iy == 0 || iy == g.ny - 1 || iz == 0 || iz == g.nz - 1;
}

__global__ void k_bptt_features(const Geo g, const int64_t *nodes, int64_t nb, const float *lm, const float *lm1,
                                const float *lm2, float *x, float *scale, int *kstar)
{
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += (int64_t)gridDim.x * blockDim.x) {
        int ix, iy, iz;
        coords_of(g, nodes[b], ix, iy, iz);
        float f[kMlpIn];
#pragma unroll
        for (int nbh = 0; nbh < 27; nbh++) {
            const int jx = ix + nbh % 3 - 1, jy = iy + (nbh / 3) % 3 - 1, jz = iz + nbh / 9 - 1;
            float f0 = 0.f, f1 = 0.f, f2 = 0.f;
            if (inside(g, jx, jy, jz)) {
                const int64_t qn = index_of(g, jx, jy, jz);
                const float sj = sponge_of(g, jx, jy, jz);
                const float hq = lm2[qn] * sj;  // s q: the history the step keeps
                f0 = on_boundary(g, jx, jy, jz) ? hq * sj : lm[qn];
                f1 = lm1[qn] * sj;
                f2 = hq;
            }
            f[nbh] = f0;
            f[27 + nbh] = f1;
            f[54 + nbh] = f2;
        }
        float m = 0.f;
        int km = 0;
        for (int k = 0; k < kMlpIn; k++)
            if (fabsf(f[k]) > m) { m = fabsf(f[k]); km = k; }
        const float sc = m + 1e-30f, inv = 1.f / sc;
        float *xr = x + b * kMlpIn;
        for (int k = 0; k < kMlpIn; k++) xr[k] = f[k] * inv;
        scale[b] = sc;
        // arg-max feature and its sign; -1 for an all-zero neighbourhood (N is 0 there and has
        // no derivative: its gradient is taken as 0)
        kstar[b] = m > 0.f ? (km | (f[km] < 0.f ? 0x100 : 0)) : -1;
    }
}

// g_b = A0 at the boundary node; the network output's gradient dy_b = g_b scale_b where the
// output is not clipped (the node's value is scale clip(y))
__global__ void k_bptt_dy(const int64_t *nodes, int64_t nb, const float *a0, const float *y, const float *scale,
                          float *g, float *dy)
{
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += (int64_t)gridDim.x * blockDim.x) {
        const float gb = a0[nodes[b]];
        g[b] = gb;
        dy[b] = (y[b] > -1.f && y[b] < 1.f) ? gb * scale[b] : 0.f;
    }
}

// dx (= dy dy/dx) -> feature gradient G, in place: d = dx / scale, plus the scale's share on its
// arg-max feature
__global__ void k_bptt_feature_grad(int64_t nb, const float *x, const float *scale, const int *kstar, const float *g,
                                    const float *y, float *dx)
{
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += (int64_t)gridDim.x * blockDim.x) {
        const float *xr = x + b * kMlpIn;
        float *d = dx + b * kMlpIn;
        if (kstar[b] < 0) {
            for (int k = 0; k < kMlpIn; k++) d[k] = 0.f;
            continue;
        }
        const float inv = 1.f / scale[b];
        float xd = 0.f;
        for (int k = 0; k < kMlpIn; k++) {
            d[k] *= inv;
            xd = fmaf(xr[k], d[k], xd);
        }
        const float h = fminf(fmaxf(y[b], -1.f), 1.f);
        const int ks = kstar[b];
        const float sg = (ks & 0x100) ? -1.f : 1.f;
        d[ks & 0xff] += sg * (g[b] * h - xd);
    }
}

// every node collects the feature gradients of the boundary nodes whose neighbourhood holds it
__global__ void k_bptt_gather(const Geo g, int64_t n_int, const int *sidx, const float *G, float *a0, float *a1,
                              float *a2)
{
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n_int; q += (int64_t)gridDim.x * blockDim.x) {
        int jx, jy, jz;
        coords_of(g, q, jx, jy, jz);
        if (jx >= g.nx) continue;  // padding column
        // only nodes within one node of the boundary can be in a boundary node's neighbourhood
        if (jx > 1 && jx < g.nx - 2 && jy > 1 && jy < g.ny - 2 && jz > 1 && jz < g.nz - 2) continue;
        const float sj = sponge_of(g, jx, jy, jz);
        const bool bj = on_boundary(g, jx, jy, jz);
        float s0 = 0.f, s1 = 0.f, s2 = 0.f;
        for (int o = 0; o < 27; o++) {
            const int dx = o % 3 - 1, dy = (o / 3) % 3 - 1, dz = o / 9 - 1;  // j = b + (dx, dy, dz)
            const int bx = jx - dx, by = jy - dy, bz = jz - dz;
            if (!inside(g, bx, by, bz)) continue;
            const int sb = sidx[index_of(g, bx, by, bz)];
            if (sb < 0) continue;
            const float *Gb = G + (int64_t)sb * kMlpIn;
            s0 += Gb[o];
            s1 += Gb[27 + o];
            s2 += Gb[54 + o];
        }
        if (bj) a2[q] += sj * sj * s0;
        else a0[q] += s0;
        a1[q] += sj * s1;
        a2[q] += sj * s2;
    }
}

// v = a s lambda on interior nodes (lambda = A0), zero elsewhere
__global__ void k_bptt_v(const Geo g, int64_t n_int, const float *a, const float *a0, float *v)
{
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n_int; q += (int64_t)gridDim.x * blockDim.x) {
        int ix, iy, iz;
        coords_of(g, q, ix, iy, iz);
        const bool in = ix > 0 && ix < g.nx - 1 && iy > 0 && iy < g.ny - 1 && iz > 0 && iz < g.nz - 1;
        v[q] = in ? a[q] * sponge_of(g, ix, iy, iz) * a0[q] : 0.f;
    }
}

__global__ void k_bptt_interior(const Geo g, int64_t n_int, const BpttOperator op, const float *v, const float *a0,
                                float *a1, float *a2)
{
    const int O = op.order, W = 2 * O + 1;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n_int; q += (int64_t)gridDim.x * blockDim.x) {
        int jx, jy, jz;
        coords_of(g, q, jx, jy, jz);
        if (jx >= g.nx) continue;
        const int lx = jx % O, ly = jy % O, lz = jz % O;
        float acc = 0.f;
        for (int d = -O; d <= O; d++) {
            // x: i = j - d e_x, K_ij = g0 W(lz) W(ly) T[lx_i][d]
            const int ixx = jx - d;
            if (ixx >= 0 && ixx < g.nx) {
                const float vi = v[q - d];
                if (vi != 0.f) acc = fmaf(op.g[0] * (op.wa[lz] * op.wa[ly]) * op.T[(ixx % O) * W + d + O], vi, acc);
            }
            // z: i = j - d e_z, K_ij = W(lx) g1 W(ly) T[lz_i][d]
            const int izz = jz - d;
            if (izz >= 0 && izz < g.nz) {
                const float vi = v[q - (int64_t)d * g.nxp];
                if (vi != 0.f) acc = fmaf(op.wa[lx] * (op.g[1] * op.wa[ly]) * op.T[(izz % O) * W + d + O], vi, acc);
            }
            // y: i = j - d e_y, K_ij = W(lx) g2 W(lz) T[ly_i][d]
            const int iyy = jy - d;
            if (iyy >= 0 && iyy < g.ny) {
                const float vi = v[q - (int64_t)d * g.nxp * g.nz];
                if (vi != 0.f) acc = fmaf(op.wa[lx] * (op.g[2] * op.wa[lz]) * op.T[(iyy % O) * W + d + O], vi, acc);
            }
        }
        const bool in = jx > 0 && jx < g.nx - 1 && jy > 0 && jy < g.ny - 1 && jz > 0 && jz < g.nz - 1;
        const float sj = sponge_of(g, jx, jy, jz);
        const float lam = in ? a0[q] : 0.f;
        a1[q] += 2.f * sj * lam - acc;
        a2[q] -= sj * sj * lam;
    }
}

// loss sum_r (out_r - ref_r)^2 over the region of interest, its gradient into A0; one block,
// fixed-order reduction
__global__ void k_bptt_loss(const int64_t *roi, int n_roi, const float *out, const float *ref, float *a0, double *loss)
{
    __shared__ double part[1024];
    double acc = 0.0;
    for (int r = threadIdx.x; r < n_roi; r += blockDim.x) {
        const int64_t q = roi[r];
        const float e = out[q] - ref[r];
        a0[q] += 2.f * e;
        acc += (double)e * e;
    }
    part[threadIdx.x] = acc;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) part[threadIdx.x] += part[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) *loss += part[0];
}

constexpr int kThreads = 256;
int blocks_for(int64_t n) { return (int)std::min<int64_t>((n + kThreads - 1) / kThreads, 152 * 8); }

}  // namespace

cudaError_t bptt_features(const BpttFields &f, const float *lm, const float *lm1, const float *lm2, cudaStream_t s)
{
    const Geo g{f.nx, f.ny, f.nz, f.nxp, f.sx, f.sy, f.sz};
    k_bptt_features<<<blocks_for(f.nb), kThreads, 0, s>>>(g, f.nodes, f.nb, lm, lm1, lm2, f.x, f.scale, f.kstar);
    return cudaGetLastError();
}

cudaError_t bptt_dy(const BpttFields &f, cudaStream_t s)
{
    k_bptt_dy<<<blocks_for(f.nb), kThreads, 0, s>>>(f.nodes, f.nb, f.a[0], f.y, f.scale, f.g, f.dy);
    return cudaGetLastError();
}

cudaError_t bptt_scatter(const BpttFields &f, cudaStream_t s)
{
    const Geo g{f.nx, f.ny, f.nz, f.nxp, f.sx, f.sy, f.sz};
    k_bptt_feature_grad<<<blocks_for(f.nb), kThreads, 0, s>>>(f.nb, f.x, f.scale, f.kstar, f.g, f.y, f.dx);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_bptt_gather<<<blocks_for(f.n_int), kThreads, 0, s>>>(g, f.n_int, f.sidx, f.dx, f.a[0], f.a[1], f.a[2]);
    return cudaGetLastError();
}

cudaError_t bptt_interior(const BpttFields &f, const BpttOperator &op, const float *a_mass, cudaStream_t s)
{
    const Geo g{f.nx, f.ny, f.nz, f.nxp, f.sx, f.sy, f.sz};
    k_bptt_v<<<blocks_for(f.n_int), kThreads, 0, s>>>(g, f.n_int, a_mass, f.a[0], f.v);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_bptt_interior<<<blocks_for(f.n_int), kThreads, 0, s>>>(g, f.n_int, op, f.v, f.a[0], f.a[1], f.a[2]);
    return cudaGetLastError();
}

cudaError_t bptt_loss(const BpttFields &f, const float *out, const float *ref, double *loss, cudaStream_t s)
{
    if (f.n_roi > 0) k_bptt_loss<<<1, 1024, 0, s>>>(f.roi, f.n_roi, out, ref, f.a[0], loss);
    return cudaGetLastError();
}

}  // namespace semgb
