// k_stencil.cu -- fused SEM step on a uniform box (see stencil.h for the operator).
//
// One thread per node.  For each axis the assembled 1-D stiffness row of a node depends only on
// its local index l = i mod o inside the element, so the three axis terms use one table
//     T[l][d + o] = coupling between a node with local index l and the node d places further
// along the same axis (d in [-o, o]; zero outside the node's element or element pair), applied
// in difference form sum_d T[l][d] (p_{i+d} - p_i), which is exactly zero for a constant field.
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "stencil.h"

namespace semgb {

namespace {

constexpr int kStencilThreads = 256;
constexpr int kTMax = 5 * 5 * 11;
__constant__ float c_T[kMaxOrder][kTMax];  // [order-1][l * (2o+1) + d + o]

// Host: T for one order from the GLL tables (double, rounded once).
void build_T(const Gll &g, float *T)
{
    const int o = g.order, o1 = o + 1, W = 2 * o + 1;
    // element 1-D stiffness A(i, j) = sum_q w_q phi_i'(xi_q) phi_j'(xi_q)
    double A[6][6];
    for (int i = 0; i < o1; i++)
        for (int j = 0; j < o1; j++) {
            double s = 0;
            for (int q = 0; q < o1; q++) s += g.w[q] * g.dphi[i * o1 + q] * g.dphi[j * o1 + q];
            A[i][j] = s;
        }
    for (int l = 0; l < o; l++)
        for (int d = -o; d <= o; d++) {
            double v = 0;
            if (l == 0) {
                if (d >= 0) v += A[0][d];          // element to the right (local 0)
                if (d <= 0) v += A[o][o + d];      // element to the left (local o)
            } else if (l + d >= 0 && l + d <= o) {
                v = A[l][l + d];
            }
            T[l * W + d + o] = (float)v;
        }
}

template <int O, bool SPONGE>
__global__ void __launch_bounds__(kStencilThreads) k_stencil_simple(const StencilTables t, const StencilArgs a)
{
    constexpr int W = 2 * O + 1;
    __shared__ float sT[O * W];
    __shared__ float sW[O];
    for (int q = threadIdx.x; q < O * W; q += kStencilThreads) sT[q] = c_T[O - 1][q];
#pragma unroll
    for (int l = 0; l < O; l++)  // static indices keep the parameter struct out of local memory
        if (threadIdx.x == l) sW[l] = t.wa[l];
    __syncthreads();

    const int64_t i = (int64_t)blockIdx.x * kStencilThreads + threadIdx.x;
    if (i < t.n) {
        const int64_t nxz = t.nx * t.nz;
        const int64_t iy = i / nxz, r = i - iy * nxz, iz = r / t.nx, ix = r - iz * t.nx;
        const float pc = a.cur[i];
        const float q = a.prev[i];
        float s = 1.f;
        if (SPONGE) s = __ldg(a.sx + ix) * __ldg(a.sy + iy) * __ldg(a.sz + iz);
        const float qd = SPONGE ? s * q : q;
        float v = qd;
        if (ix > 0 && ix < t.nx - 1 && iz > 0 && iz < t.nz - 1 && iy > 0 && iy < t.ny - 1) {
            const int lx = (int)(ix % O), lz = (int)(iz % O), ly = (int)(iy % O);
            const float *Tx = sT + lx * W, *Tz = sT + lz * W, *Ty = sT + ly * W;
            float ax = 0.f, az = 0.f, ay = 0.f;
#pragma unroll
            for (int d = -O; d <= O; d++) {
                if (d == 0) continue;
                // offsets with a zero coefficient may leave the box: clamp them onto the axis
                const int64_t dx = min(max((int64_t)d, -ix), t.nx - 1 - ix);
                const int64_t dz = min(max((int64_t)d, -iz), t.nz - 1 - iz);
                const int64_t dy = min(max((int64_t)d, -iy), t.ny - 1 - iy);
                ax = fmaf(Tx[d + O], __ldg(a.cur + i + dx) - pc, ax);
                az = fmaf(Tz[d + O], __ldg(a.cur + i + dz * t.nx) - pc, az);
                ay = fmaf(Ty[d + O], __ldg(a.cur + i + dy * nxz) - pc, ay);
            }
            const float wx = sW[lx], wz = sW[lz], wy = sW[ly];
            const float y = (t.g[0] * (wz * wy)) * ax + (t.g[1] * (wx * wy)) * az + (t.g[2] * (wx * wz)) * ay;
            v = (2.f * pc - qd) - __ldg(a.a + i) * y;
        }
        a.prev[i] = SPONGE ? s * v : v;
    }
    if (a.nrec > 0) {
        __shared__ int r_lo, r_hi;
        __syncthreads();
        if (threadIdx.x == 0) {
            const int64_t b0 = (int64_t)blockIdx.x * kStencilThreads;
            int lo = 0, hi = a.nrec;
            while (lo < hi) { int m = (lo + hi) >> 1; if (a.rec_node[m] < b0) lo = m + 1; else hi = m; }
            r_lo = lo;
            hi = a.nrec;
            while (lo < hi) { int m = (lo + hi) >> 1; if (a.rec_node[m] < b0 + kStencilThreads) lo = m + 1; else hi = m; }
            r_hi = lo;
        }
        __syncthreads();
        const int step = a.ctr[1];
        for (int rr = r_lo + threadIdx.x; rr < r_hi; rr += kStencilThreads)
            a.traces[(int64_t)step * a.nrec + a.rec_perm[rr]] = a.prev[a.rec_node[rr]];
    }
}

template <int O>
cudaError_t launch_o(const StencilTables &t, const StencilArgs &a, bool sponge, cudaStream_t s)
{
    const int64_t grid = (t.n + kStencilThreads - 1) / kStencilThreads;
    if (grid > 0x7fffffffLL) return cudaErrorInvalidValue;
    if (sponge) k_stencil_simple<O, true><<<(unsigned)grid, kStencilThreads, 0, s>>>(t, a);
    else k_stencil_simple<O, false><<<(unsigned)grid, kStencilThreads, 0, s>>>(t, a);
    return cudaGetLastError();
}

}  // namespace

int stencil_tables_create(const Box &b, const Gll &g, const Geometry &geo, StencilTables **out)
{
    StencilTables *t = new StencilTables();
    t->order = b.order;
    t->nx = b.nx; t->ny = b.ny; t->nz = b.nz; t->n = b.n_nodes;
    for (int d = 0; d < 3; d++) t->g[d] = (float)geo.g[d];
    for (int l = 0; l < b.order; l++) t->wa[l] = (float)(l == 0 ? g.w[0] + g.w[b.order] : g.w[l]);
    *out = t;
    return 0;
}

void stencil_tables_free(StencilTables *&t)
{
    delete t;
    t = nullptr;
}

cudaError_t stencil_kernel_setup()
{
    static std::vector<int> done_devices;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    for (int d : done_devices)
        if (d == dev) return cudaSuccess;
    std::vector<float> all(kMaxOrder * kTMax, 0.f);
    for (int o = 1; o <= kMaxOrder; o++) {
        Gll g;
        gll_tables(o, g);
        build_T(g, all.data() + (o - 1) * kTMax);
    }
    e = cudaMemcpyToSymbol(c_T, all.data(), all.size() * sizeof(float));
    if (e == cudaSuccess) done_devices.push_back(dev);
    return e;
}

cudaError_t launch_stencil(const StencilTables &t, const StencilArgs &a, bool sponge, cudaStream_t s)
{
    switch (t.order) {
    case 1: return launch_o<1>(t, a, sponge, s);
    case 2: return launch_o<2>(t, a, sponge, s);
    case 3: return launch_o<3>(t, a, sponge, s);
    case 4: return launch_o<4>(t, a, sponge, s);
    case 5: return launch_o<5>(t, a, sponge, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace semgb
