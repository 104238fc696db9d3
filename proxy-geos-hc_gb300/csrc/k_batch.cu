// k_batch.cu -- many shots on one mesh: the SEM step with the shot index innermost.
//
// A batch advances S shots (independent sources, same mesh, model, sponge and receivers).  The
// levels are stored P[node][S] (device layout of the node, S padded to a multiple of 32), so for
// one node the S shot values are contiguous.  Compared with S separate runs of the plain step:
//  - the mesh-side data (dt^2/M, sponge factors, node indices, GLL coefficients) is read or
//    computed once per node for all shots: bytes per shot-node-step fall from 16 to
//    12 + 4/S (read p^n, p^{n-1}, write p^{n+1}, plus the shared dt^2/M);
//  - a warp owns one (x, z) node column for 32 * SPL shots (SPL shots per lane) and marches
//    along y, so every spatial quantity -- node index, local GLL indices, coefficients, mass,
//    sponge factor -- is warp-uniform and paid once per 32 * SPL shot-nodes, and every load or
//    store is one contiguous 128 * SPL-byte vector;
//  - the y-neighbours come from a per-lane register queue of 2o+1 planes (p^n is read from HBM
//    once per node), the x- and z-neighbours from L1/L2 (the warps of a CTA hold consecutive
//    x-columns and all resident warps march through the same few planes).
// The operator is the assembled tensor-product form of stencil.h.
#include <cuda_runtime.h>

#include "batch.h"

namespace semgb {

namespace {

constexpr int kTBMax = kMaxOrder * (2 * kMaxOrder + 1);
__constant__ float cb_T[kMaxOrder][kTBMax];    // same table as the plain stencil
__constant__ float cb_wa[kMaxOrder][kMaxOrder];

__host__ __device__ constexpr int blo(int O, int l) { return l == 0 ? -O : -l; }
__host__ __device__ constexpr int bhi(int O, int l) { return l == 0 ? O : O - l; }

template <int SPL>
struct Sv {
    float v[SPL];
};

template <int SPL>
__device__ __forceinline__ Sv<SPL> ldv(const float *p)
{
    Sv<SPL> r;
    if constexpr (SPL == 2) {
        const float2 t = *reinterpret_cast<const float2 *>(p);
        r.v[0] = t.x; r.v[1] = t.y;
    } else if constexpr (SPL == 4) {
        const float4 t = *reinterpret_cast<const float4 *>(p);
        r.v[0] = t.x; r.v[1] = t.y; r.v[2] = t.z; r.v[3] = t.w;
    } else {
        r.v[0] = *p;
    }
    return r;
}

template <int SPL>
__device__ __forceinline__ void stv(float *p, const Sv<SPL> &a)
{
    if constexpr (SPL == 2) *reinterpret_cast<float2 *>(p) = make_float2(a.v[0], a.v[1]);
    else if constexpr (SPL == 4) *reinterpret_cast<float4 *>(p) = make_float4(a.v[0], a.v[1], a.v[2], a.v[3]);
    else *p = a.v[0];
}

// acc += sum_d T[L][d] (nbr(d) - c) for the compile-time local index L (neighbours through `at`).
template <int O, int L, int SPL, class At>
__device__ __forceinline__ void axis_term(const Sv<SPL> &c, const At &at, Sv<SPL> &acc)
{
#pragma unroll
    for (int d = blo(O, L); d <= bhi(O, L); d++) {
        if (d == 0) continue;
        const Sv<SPL> v = at(d);
        const float t = cb_T[O - 1][L * (2 * O + 1) + d + O];
#pragma unroll
        for (int k = 0; k < SPL; k++) acc.v[k] = fmaf(t, v.v[k] - c.v[k], acc.v[k]);
    }
}

template <int O, int SPL, class At>
__device__ __forceinline__ Sv<SPL> axis(int l, const Sv<SPL> &c, const At &at)
{
    Sv<SPL> acc;
#pragma unroll
    for (int k = 0; k < SPL; k++) acc.v[k] = 0.f;
    switch (l) {  // warp-uniform
    case 0: axis_term<O, 0, SPL>(c, at, acc); break;
    case 1: if constexpr (O > 1) axis_term<O, 1, SPL>(c, at, acc); break;
    case 2: if constexpr (O > 2) axis_term<O, 2, SPL>(c, at, acc); break;
    case 3: if constexpr (O > 3) axis_term<O, 3, SPL>(c, at, acc); break;
    default: if constexpr (O > 4) axis_term<O, 4, SPL>(c, at, acc); break;
    }
    return acc;
}

template <int SPL>
struct Strided {  // neighbour at offset d: base + d * stride (floats)
    const float *base;
    int64_t stride;
    __device__ __forceinline__ Sv<SPL> operator()(int d) const { return ldv<SPL>(base + d * stride); }
};

template <int O, int SPL>
struct Queue {  // neighbour at offset d along y: register queue
    const Sv<SPL> *q;
    __device__ __forceinline__ Sv<SPL> operator()(int d) const { return q[d + O]; }
};

template <int O, int SPL, bool SPONGE>
__global__ void __launch_bounds__(1024) k_batch(const BatchArgs a)
{
    const int warps = blockDim.x >> 5;
    const int lane = threadIdx.x & 31;
    const int64_t col = (int64_t)blockIdx.x * warps + (threadIdx.x >> 5);  // x fastest
    if (col >= a.nx * a.nz) return;
    const int64_t z = col / a.nx, x = col - z * a.nx;
    const int64_t S = a.s_pad;
    const int64_t sx_stride = S, sz_stride = a.nxp * S, sy_stride = a.nxp * a.nz * S;
    const int64_t shot0 = (int64_t)blockIdx.z * 32 * SPL + lane * SPL;  // this lane's first shot
    const int yb = blockIdx.y * a.ychunk;
    const int ye = (int)min(a.ny, (int64_t)yb + a.ychunk);
    const int lx = (int)(x % O), lz = (int)(z % O);
    const bool xz_in = x > 0 && x < a.nx - 1 && z > 0 && z < a.nz - 1;
    const float wx = cb_wa[O - 1][lx], wz = cb_wa[O - 1][lz];
    float sxz = 1.f;
    if (SPONGE) sxz = __ldg(a.sx + x);
    const float szv = SPONGE ? __ldg(a.sz + z) : 1.f;
    const float *cur_col = a.cur + x * sx_stride + z * sz_stride + shot0;
    float *prv_col = a.prev + x * sx_stride + z * sz_stride + shot0;
    const int64_t acol = x + z * a.nxp;

    Sv<SPL> q[2 * O + 1];  // p^n at planes y-O..y+O of this column, this lane's shots
#pragma unroll
    for (int k = 0; k < 2 * O; k++) {
        const int yy = yb - O + k;
        if (yy >= 0 && yy < a.ny) q[k] = ldv<SPL>(cur_col + yy * sy_stride);
        else
#pragma unroll
            for (int j = 0; j < SPL; j++) q[k].v[j] = 0.f;
    }
    for (int y = yb; y < ye; y++) {
        if (y + O < a.ny) q[2 * O] = ldv<SPL>(cur_col + (int64_t)(y + O) * sy_stride);
        else
#pragma unroll
            for (int j = 0; j < SPL; j++) q[2 * O].v[j] = 0.f;
        const Sv<SPL> c = q[O];
        const float *here = cur_col + (int64_t)y * sy_stride;
        const Sv<SPL> qv = ldv<SPL>(prv_col + (int64_t)y * sy_stride);
        const float s = SPONGE ? sxz * __ldg(a.sy + y) * szv : 1.f;  // (sx*sy)*sz
        Sv<SPL> out;
        if (xz_in && y > 0 && y < a.ny - 1) {
            const int ly = y % O;
            const Sv<SPL> ax = axis<O, SPL>(lx, c, Strided<SPL>{here, sx_stride});
            const Sv<SPL> az = axis<O, SPL>(lz, c, Strided<SPL>{here, sz_stride});
            const Sv<SPL> ay = axis<O, SPL>(ly, c, Queue<O, SPL>{q});
            const float wy = cb_wa[O - 1][ly];
            const float gx = a.g[0] * (wz * wy), gz = a.g[1] * (wx * wy), gy = a.g[2] * (wx * wz);
            const float am = __ldg(a.a + acol + (int64_t)y * a.nxp * a.nz);
#pragma unroll
            for (int k = 0; k < SPL; k++) {
                const float qd = SPONGE ? s * qv.v[k] : qv.v[k];
                const float yv = gx * ax.v[k] + gz * az.v[k] + gy * ay.v[k];
                const float v = (2.f * c.v[k] - qd) - am * yv;
                out.v[k] = SPONGE ? s * v : v;
            }
        } else {
#pragma unroll
            for (int k = 0; k < SPL; k++) {
                const float qd = SPONGE ? s * qv.v[k] : qv.v[k];
                out.v[k] = SPONGE ? s * qd : qd;
            }
        }
        stv<SPL>(prv_col + (int64_t)y * sy_stride, out);
#pragma unroll
        for (int k = 0; k < 2 * O; k++) q[k] = q[k + 1];
    }
}

__global__ void k_batch_source(const BatchSourceArgs a)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = a.ctr[0];
    if (s < a.nshot && n < a.nsamples && a.node[s] >= 0)
        a.cur[a.node[s] * a.s_pad + s] += a.coef[s] * a.wavelet[(int64_t)s * a.nsamples + n];
}

// Advances the step counter after the source launch (blocks of k_batch_source all read it).

__global__ void k_batch_tick(int *ctr)
{
    ctr[1] = ctr[0];
    ctr[0] = ctr[0] + 1;
}

__global__ void k_batch_record(const BatchRecordArgs a)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;  // receiver-major, shot fastest
    if (i >= (int64_t)a.nrec * a.nshot) return;
    const int r = (int)(i / a.nshot), s = (int)(i - (int64_t)r * a.nshot);
    const int step = a.ctr[1];
    a.traces[((int64_t)step * a.nrec + r) * a.nshot + s] = a.level[a.rec_node[r] * a.s_pad + s];
}

template <int O, int SPL>
cudaError_t launch_o(const BatchArgs &a, bool sponge, int warps_per_cta, cudaStream_t st)
{
    const int64_t cols = a.nx * a.nz;
    const dim3 grid((unsigned)((cols + warps_per_cta - 1) / warps_per_cta), (unsigned)((a.ny + a.ychunk - 1) / a.ychunk),
                    (unsigned)(a.s_pad / (32 * SPL)));
    if (sponge) k_batch<O, SPL, true><<<grid, 32 * warps_per_cta, 0, st>>>(a);
    else k_batch<O, SPL, false><<<grid, 32 * warps_per_cta, 0, st>>>(a);
    return cudaGetLastError();
}

template <int SPL>
cudaError_t launch_spl(int order, const BatchArgs &a, bool sponge, int w, cudaStream_t st)
{
    switch (order) {
    case 1: return launch_o<1, SPL>(a, sponge, w, st);
    case 2: return launch_o<2, SPL>(a, sponge, w, st);
    case 3: return launch_o<3, SPL>(a, sponge, w, st);
    case 4: return launch_o<4, SPL>(a, sponge, w, st);
    case 5: return launch_o<5, SPL>(a, sponge, w, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

cudaError_t batch_kernel_setup(const float *T_all, const float *wa_all)
{
    cudaError_t e = cudaMemcpyToSymbol(cb_T, T_all, sizeof(float) * kMaxOrder * kTBMax);
    if (e != cudaSuccess) return e;
    return cudaMemcpyToSymbol(cb_wa, wa_all, sizeof(float) * kMaxOrder * kMaxOrder);
}

cudaError_t launch_batch_step(int order, const BatchArgs &a, bool sponge, const BatchTuning &tune, cudaStream_t st)
{
    switch (tune.shots_per_lane) {
    case 1: return launch_spl<1>(order, a, sponge, tune.warps_per_cta, st);
    case 2: return launch_spl<2>(order, a, sponge, tune.warps_per_cta, st);
    case 4: return launch_spl<4>(order, a, sponge, tune.warps_per_cta, st);
    default: return cudaErrorInvalidValue;
    }
}

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

cudaError_t launch_batch_record(const BatchRecordArgs &a, cudaStream_t st)
{
    const int64_t n = (int64_t)a.nrec * a.nshot;
    if (n == 0) return cudaSuccess;
    k_batch_record<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace semgb
