// k_update.cu -- node-wise kernels of the SEM step and its set-up (device layout of kernels.h).
//
//  k_source   SEMsolver.cpp:39-43    p^n[node0(e_k)] += dt^2 c_e^2 r_k(t_n), sources in order
//  k_update   SEMsolver.cpp:85-89    p^{n+1} = 2 p^n - p^{n-1} - dt^2 y / M on interior nodes,
//                                    boundary nodes keep p^{n-1} (homogeneous Dirichlet), then the
//                                    sponge on both levels, receiver sampling, y reset; one pass
//  k_connectivity  SEMmesh.cpp:205-231 (on the device, for the element kernel)
//  k_mass     SEMsolver.cpp:33-36,74-80 assembled once: a_i = dt^2 / M_i
#include <cuda_runtime.h>

#include <algorithm>

#include "kernels.h"

namespace semgb {

namespace {

// One block.  Sources on distinct nodes are added by all threads (one addition per node, the
// same bits as any order); otherwise one thread adds them in source order, as the reference's
// loop does, so that sources sharing a node sum in that order.
__global__ void k_source(const SourceArgs a)
{
    const int n = a.ctr[0];
    __syncthreads();  // every thread has read the step before thread 0 advances the counter
    if (n < a.nsamples) {
        if (a.distinct) {
            for (int k = threadIdx.x; k < a.nsrc; k += blockDim.x)
                a.cur[a.node[k]] += a.coef[k] * a.wavelet[(int64_t)k * a.nsamples + n];
        } else if (threadIdx.x == 0) {
            for (int k = 0; k < a.nsrc; k++)
                a.cur[a.node[k]] += a.coef[k] * a.wavelet[(int64_t)k * a.nsamples + n];
        }
    }
    if (threadIdx.x == 0) {
        a.ctr[1] = n;
        a.ctr[0] = n + 1;
    }
}

// REF: the reference's update arithmetic, (2 p^n - p^{n-1}) - ((dt*dt) y) / M, each operation
// rounded (SEMsolver.cpp:85-89), with M in a.mref; otherwise the precomputed a = dt^2/M.
template <bool SPONGE, bool REF>
__global__ void __launch_bounds__(kUpdateThreads) k_update(const UpdateArgs a)
{
    constexpr int V = kUpdateNodesPerThread;
    const int64_t i0 = ((int64_t)blockIdx.x * kUpdateThreads + threadIdx.x) * V;
    if (i0 < a.n_int) {
        // rows are padded to a multiple of 4 nodes: the 4 nodes share one row
        const int64_t nxz = a.nxp * a.nz;
        const int64_t iy = i0 / nxz, r = i0 - iy * nxz, iz = r / a.nxp, ix0 = r - iz * a.nxp;
        const float4 c4 = *reinterpret_cast<const float4 *>(a.cur + i0);
        const float4 q4 = *reinterpret_cast<const float4 *>(a.prev + i0);
        const float4 y4 = *reinterpret_cast<const float4 *>(a.y + i0);
        const float4 a4 = __ldg(reinterpret_cast<const float4 *>((REF ? a.mref : a.a) + i0));
        const float cc[V] = {c4.x, c4.y, c4.z, c4.w}, qq[V] = {q4.x, q4.y, q4.z, q4.w};
        const float yy[V] = {y4.x, y4.y, y4.z, y4.w}, aa[V] = {a4.x, a4.y, a4.z, a4.w};
        const bool zy_in = iz > 0 && iz < a.nz - 1 && iy > 0 && iy < a.ny - 1;
        float syz = 1.f, szv = 1.f;
        if (SPONGE && ix0 < a.nx) { syz = __ldg(a.sy + iy); szv = __ldg(a.sz + iz); }
        float out[V];
#pragma unroll
        for (int t = 0; t < V; t++) {
            const int64_t ix = ix0 + t;
            out[t] = 0.f;  // padding stays zero
            if (ix < a.nx) {
                float s = 1.f;
                if (SPONGE) s = __ldg(a.sx + ix) * syz * szv;  // (sx*sy)*sz
                const float qd = SPONGE ? s * qq[t] : qq[t];
                const bool interior = zy_in && ix > 0 && ix < a.nx - 1;
                float v = qd;
                if (interior) {
                    if constexpr (REF)
                        v = __fsub_rn(__fsub_rn(2.f * cc[t], qd), __fdiv_rn(__fmul_rn(a.dt2f, yy[t]), aa[t]));
                    else
                        v = (2.f * cc[t] - qd) - aa[t] * yy[t];
                }
                out[t] = SPONGE ? s * v : v;
            }
        }
        *reinterpret_cast<float4 *>(a.prev + i0) = make_float4(out[0], out[1], out[2], out[3]);
        *reinterpret_cast<float4 *>(a.y + i0) = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    if (a.nrec > 0) {
        const int r0 = a.rec_off[blockIdx.x], r1 = a.rec_off[blockIdx.x + 1];
        if (r0 < r1) {  // uniform over the block
            __syncthreads();  // this block's new values are visible to the whole block
            const int step = a.ctr[1];
            for (int r = r0 + threadIdx.x; r < r1; r += kUpdateThreads)
                a.traces[(int64_t)step * a.nrec + a.rec_perm[r]] = a.prev[a.rec_node[r]];
        }
    }
}

__global__ void k_connectivity(int32_t *conn, int ex, int ez, int order, int64_t nxp, int64_t nz,
                               int64_t n_elem)
{
    const int o1 = order + 1, npe = o1 * o1 * o1;
    const int64_t total = n_elem * npe;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = q / npe;
        const int loc = (int)(q - e * npe);
        const int64_t ix = e % ex, iz = (e / ex) % ez, iy = e / ((int64_t)ex * ez);
        const int l = loc % o1, n = (loc / o1) % o1, m = loc / (o1 * o1);
        conn[q] = (int32_t)((ix * order + l) + (iz * order + n) * nxp + (iy * order + m) * nxp * nz);
    }
}

// Elements adjacent to node index i along one axis with ne elements: [lo, hi].
__device__ __forceinline__ void adj_range(int i, int order, int ne, int &lo, int &hi)
{
    const int e = i / order;
    if (i - e * order == 0) {
        lo = e > 0 ? e - 1 : 0;
        hi = e < ne ? e : ne - 1;
    } else {
        lo = hi = e;
    }
}

// 1 / c_e^2 per element, in double (the per-node sums below read it up to 8 times)
__global__ void k_inv_c2(const float *vel, int64_t n, double *out)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double c = vel[i];
        out[i] = 1.0 / (c * c);
    }
}

// a_i = dt^2 / M_i with M_i = w_i detJ sum over the adjacent elements of 1/c_e^2 (or, with a
// node model, m_i w_i detJ times the number of adjacent elements), in double.  Grid: x-blocks of
// a row by z by y (grid-stride over z and y), so node indices come without divisions.
__global__ void k_mass(float *a, const double *inv_c2, const float *slow2, int ex, int ey, int ez, int order,
                       int nxp, const double *w, double detJ, double dt2)
{
    const int nx = ex * order + 1, ny = ey * order + 1, nz = ez * order + 1;
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    if (ix >= nxp) return;
    int x0 = 0, x1 = 0;
    if (ix < nx) adj_range(ix, order, ex, x0, x1);
    for (int iy = blockIdx.z; iy < ny; iy += gridDim.z)
        for (int iz = blockIdx.y; iz < nz; iz += gridDim.y) {
            const int64_t q = ix + (int64_t)nxp * (iz + (int64_t)nz * iy);
            if (ix >= nx) {
                a[q] = 0.f;
                continue;
            }
            // local weight of the node: w[i mod o] (element-boundary nodes have w_0 = w_o)
            const double wq = w[ix % order] * w[iz % order] * w[iy % order];
            int z0, z1, y0, y1;
            adj_range(iz, order, ez, z0, z1);
            adj_range(iy, order, ey, y0, y1);
            double m;
            if (slow2) {
                const double cnt = (double)((x1 - x0 + 1) * (z1 - z0 + 1) * (y1 - y0 + 1));
                m = (double)slow2[q] * wq * detJ * cnt;
            } else {
                double sum = 0.0;
                for (int ey_ = y0; ey_ <= y1; ey_++)
                    for (int ez_ = z0; ez_ <= z1; ez_++)
                        for (int ex_ = x0; ex_ <= x1; ex_++)
                            sum += inv_c2[ex_ + (int64_t)ex * (ez_ + (int64_t)ez * ey_)];
                m = wq * detJ * sum;
            }
            a[q] = (float)(dt2 / m);
        }
}

// The reference's assembled mass (SEMsolver.cpp:74-78, SEMQkGLIntegrals.hpp:352): for each
// adjacent element in increasing element order, M += fl(fl(w_a w_b w_c detJ) / fl(c_e c_e)), the
// local weights by the node's local indices in that element, all in float.  Padding nodes get 1.
__global__ void k_mass_ref(float *m, const float *vel, int ex, int ey, int ez, int order, int nxp, const double *w,
                           double detJ)
{
    const int nx = ex * order + 1, ny = ey * order + 1, nz = ez * order + 1;
    const int ix = blockIdx.x * blockDim.x + threadIdx.x;
    if (ix >= nxp) return;
    int x0 = 0, x1 = 0;
    if (ix < nx) adj_range(ix, order, ex, x0, x1);
    for (int iy = blockIdx.z; iy < ny; iy += gridDim.z)
        for (int iz = blockIdx.y; iz < nz; iz += gridDim.y) {
            const int64_t q = ix + (int64_t)nxp * (iz + (int64_t)nz * iy);
            if (ix >= nx) {
                m[q] = 1.f;
                continue;
            }
            int z0, z1, y0, y1;
            adj_range(iz, order, ez, z0, z1);
            adj_range(iy, order, ey, y0, y1);
            float sum = 0.f;
            for (int ey_ = y0; ey_ <= y1; ey_++)
                for (int ez_ = z0; ez_ <= z1; ez_++)
                    for (int ex_ = x0; ex_ <= x1; ex_++) {
                        const float ml = (float)(w[ix - ex_ * order] * w[iz - ez_ * order] * w[iy - ey_ * order] * detJ);
                        const float c = vel[ex_ + (int64_t)ex * (ez_ + (int64_t)ez * ey_)];
                        sum = __fadd_rn(sum, __fdiv_rn(ml, __fmul_rn(c, c)));
                    }
            m[q] = sum;
        }
}

// g_i <- g_i / m_i with m_i the node's squared slowness, recovered from the stored
// a_i = dt^2 / (m_i W_i) and the geometric mass W_i (quadrature weight x detJ x adjacent elements),
// so it holds for element-velocity and node-slowness models alike.
__global__ void k_grad_scale(float *g, const float *a, int ex, int ey, int ez, int order, int64_t nxp,
                             const double *w, double detJ, double dt2)
{
    const int64_t nx = (int64_t)ex * order + 1, ny = (int64_t)ey * order + 1,
                  nz = (int64_t)ez * order + 1, n = nxp * ny * nz;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t iy = q / (nxp * nz), r = q - iy * nxp * nz, iz = r / nxp, ix = r - iz * nxp;
        if (ix >= nx) {
            g[q] = 0.f;
            continue;
        }
        const double wq = w[ix % order] * w[iz % order] * w[iy % order];
        int x0, x1, z0, z1, y0, y1;
        adj_range((int)ix, order, ex, x0, x1);
        adj_range((int)iz, order, ez, z0, z1);
        adj_range((int)iy, order, ey, y0, y1);
        const double W = wq * detJ * (double)((x1 - x0 + 1) * (z1 - z0 + 1) * (y1 - y0 + 1));
        g[q] = (float)((double)g[q] * (double)a[q] * W / dt2);
    }
}

}  // namespace

cudaError_t launch_grad_scale(float *g, const float *a, int ex, int ey, int ez, int order, int64_t nxp,
                              const double *w_dev, double detJ, double dt2, cudaStream_t s)
{
    k_grad_scale<<<152 * 16, 256, 0, s>>>(g, a, ex, ey, ez, order, nxp, w_dev, detJ, dt2);
    return cudaGetLastError();
}

cudaError_t launch_update(const UpdateArgs &a, bool sponge, cudaStream_t s)
{
    if (a.n_int <= 0) return cudaSuccess;
    const int64_t grid = update_grid(a.n_int);
    if (grid > 0x7fffffffLL) return cudaErrorInvalidValue;
    if (a.mref) {
        if (sponge) k_update<true, true><<<(unsigned)grid, kUpdateThreads, 0, s>>>(a);
        else k_update<false, true><<<(unsigned)grid, kUpdateThreads, 0, s>>>(a);
    } else {
        if (sponge) k_update<true, false><<<(unsigned)grid, kUpdateThreads, 0, s>>>(a);
        else k_update<false, false><<<(unsigned)grid, kUpdateThreads, 0, s>>>(a);
    }
    return cudaGetLastError();
}

cudaError_t launch_mass_ref(float *m, const float *vel, int ex, int ey, int ez, int order, int64_t nxp,
                            const double *w_dev, double detJ, cudaStream_t s)
{
    const int64_t ny = (int64_t)ey * order + 1, nz = (int64_t)ez * order + 1;
    const dim3 grid((unsigned)((nxp + 127) / 128), (unsigned)std::min<int64_t>(nz, 65535),
                    (unsigned)std::min<int64_t>(ny, 65535));
    k_mass_ref<<<grid, 128, 0, s>>>(m, vel, ex, ey, ez, order, (int)nxp, w_dev, detJ);
    return cudaGetLastError();
}

cudaError_t launch_source(const SourceArgs &a, cudaStream_t s)
{
    k_source<<<1, a.distinct && a.nsrc > 32 ? 256 : 32, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_connectivity(int32_t *conn, int ex, int ey, int ez, int order, int64_t nxp,
                                cudaStream_t s)
{
    const int64_t nz = (int64_t)ez * order + 1;
    const int64_t ne = (int64_t)ex * ey * ez;
    k_connectivity<<<152 * 16, 256, 0, s>>>(conn, ex, ez, order, nxp, nz, ne);
    return cudaGetLastError();
}

cudaError_t launch_mass(float *a, const float *vel, const float *slow2, int ex, int ey, int ez,
                        int order, int64_t nxp, const double *w_dev, double detJ, double dt2,
                        cudaStream_t s)
{
    double *inv_c2 = nullptr;
    if (!slow2) {
        const int64_t ne = (int64_t)ex * ey * ez;
        cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&inv_c2), ne * sizeof(double), s);
        if (e != cudaSuccess) return e;
        k_inv_c2<<<(unsigned)std::min<int64_t>((ne + 255) / 256, 152 * 16), 256, 0, s>>>(vel, ne, inv_c2);
    }
    const int64_t ny = (int64_t)ey * order + 1, nz = (int64_t)ez * order + 1;
    const dim3 grid((unsigned)((nxp + 127) / 128), (unsigned)std::min<int64_t>(nz, 65535),
                    (unsigned)std::min<int64_t>(ny, 65535));
    k_mass<<<grid, 128, 0, s>>>(a, inv_c2, slow2, ex, ey, ez, order, (int)nxp, w_dev, detJ, dt2);
    cudaError_t e = cudaGetLastError();
    if (inv_c2) {
        const cudaError_t f = cudaFreeAsync(inv_c2, s);
        if (e == cudaSuccess) e = f;
    }
    return e;
}

}  // namespace semgb
