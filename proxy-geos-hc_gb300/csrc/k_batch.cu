// k_batch.cu -- many shots on one mesh: the SEM step with the shot index innermost.
//
// A batch advances S shots (independent sources, same mesh, model, sponge and receivers).  The
// levels are stored P[node][S] (device layout of the node, S padded to a multiple of 32), so the
// S values of one node are contiguous.  Against S runs of the plain step:
//  - the mesh-side data (dt^2/M, sponge factors, coefficients) is read once per node for all
//    shots: 12 + 4/S bytes per shot-node-step instead of 16;
//  - a warp owns one element's x-span (o nodes) in one z-row for 32 shots (one per lane), so every
//    spatial quantity -- node index, local indices, coefficients, mass, sponge factor -- is
//    warp-uniform, and every load or store is one contiguous 128-byte line;
//  - the x-coupling inside the element comes from registers (only the o nodes of the element to
//    the left and one node to the right are loaded); a CTA holds 8 consecutive z-rows of one
//    element span and stages each y-plane of them, with o halo rows on either side, in shared
//    memory (own rows from registers, halo rows prefetched one plane ahead), so the z-coupling
//    reads shared memory; one barrier per plane, double-buffered;
//  - the warp marches along y element by element: o+1 planes of its span in registers and, for
//    the face plane of the next element, the partial y-sum of the element below, so the y-local
//    index is a compile-time constant.
// Per shot the arithmetic is the plain stencil pass's (k_stencil.cu) in the same order: the
// assembled tensor-product operator of stencil.h, difference form, same sponge product.
#include <cuda_runtime.h>

#include "batch.h"

namespace semgb {

namespace {

constexpr int kTBMax = kMaxOrder * (2 * kMaxOrder + 1);
__constant__ float cb_T[kMaxOrder][kTBMax];
__constant__ float cb_wa[kMaxOrder][kMaxOrder];

__host__ __device__ constexpr int blo(int O, int l) { return l == 0 ? -O : -l; }
__host__ __device__ constexpr int bhi(int O, int l) { return l == 0 ? O : O - l; }

template <int O>
__device__ __forceinline__ float Tc(int l, int d) { return cb_T[O - 1][l * (2 * O + 1) + d + O]; }

// z-term of the O nodes of a row for compile-time z-local index LZ: rows z+d from the staged plane
// (row stride O*32 floats, node j at j*32, lane = shot)
template <int O, int LZ>
__device__ __forceinline__ void zterm(const float (&c)[O], const float *rowc, float (&az)[O])
{
#pragma unroll
    for (int j = 0; j < O; j++) az[j] = 0.f;
#pragma unroll
    for (int d = blo(O, LZ); d <= bhi(O, LZ); d++) {
        if (d == 0) continue;
        const float *row = rowc + d * (O * 32);
        const float t = Tc<O>(LZ, d);
#pragma unroll
        for (int j = 0; j < O; j++) az[j] = fmaf(t, row[j * 32] - c[j], az[j]);
    }
}

template <int O>
__device__ __forceinline__ void zterm_rt(int lz, const float (&c)[O], const float *rowc, float (&az)[O])
{
    switch (lz) {
    case 0: zterm<O, 0>(c, rowc, az); break;
    case 1: if constexpr (O > 1) zterm<O, 1>(c, rowc, az); break;
    case 2: if constexpr (O > 2) zterm<O, 2>(c, rowc, az); break;
    case 3: if constexpr (O > 3) zterm<O, 3>(c, rowc, az); break;
    default: if constexpr (O > 4) zterm<O, 4>(c, rowc, az); break;
    }
}

constexpr int ZR = 8;  // z-rows (warps) per CTA

struct ColumnCtx {
    const float *cur0;  // (x0, z, 0) + shot of this warp's row
    float *prv0;
    const float *a0;
    int64_t S, zs, ys, ays;
    int ny, ye, exi, lz;
    bool last, row_ok, zin;
    float szv, wz, g0, g1, g2;
    float *stage;  // shared: [2][ZR + 2O][O][32]
    int srow;      // this warp's row in the stage
    // halo rows this warp loads (at most two): stage row, global base at y = 0 (nullptr: none)
    int hrow[2];
    const float *hsrc[2];
};

template <int O>
__device__ __forceinline__ constexpr int stage_floats() { return (ZR + 2 * O) * O * 32; }

template <int O, bool SPONGE, int K>
__device__ __forceinline__ void plane_step(const BatchArgs &a, const ColumnCtx &k, int y0, const float (&sxv)[O + 1],
                                       const float (&P)[O + 1][O], const float (&pend)[O], float (&hnext)[2][O])
{
    const int y = y0 + K;
    if (y >= k.ye) return;  // uniform over the CTA
    const int lane = threadIdx.x & 31;
    float *buf = k.stage + (y & 1) * stage_floats<O>();
    // stage plane y: own row from registers, halo rows prefetched during the previous plane
    if (k.row_ok) {
#pragma unroll
        for (int j = 0; j < O; j++) buf[(k.srow * O + j) * 32 + lane] = P[K][j];
    }
#pragma unroll
    for (int t = 0; t < 2; t++)
        if (k.hsrc[t]) {
#pragma unroll
            for (int j = 0; j < O; j++) buf[(k.hrow[t] * O + j) * 32 + lane] = hnext[t][j];
        }
    __syncthreads();
    // prefetch the halo of plane y+1
    if (y + 1 < k.ye)
#pragma unroll
        for (int t = 0; t < 2; t++)
            if (k.hsrc[t]) {
#pragma unroll
                for (int j = 0; j < O; j++) hnext[t][j] = __ldg(k.hsrc[t] + (int64_t)(y + 1) * k.ys + j * k.S);
            }
    if (!k.row_ok) return;
    const float syv = SPONGE ? __ldg(a.sy + y) : 1.f;
    const float *here = k.cur0 + (int64_t)y * k.ys;
    float *dst = k.prv0 + (int64_t)y * k.ys;
    float q[O], am[O];
#pragma unroll
    for (int j = 0; j < O; j++) {
        q[j] = dst[j * k.S];
        am[j] = __ldg(k.a0 + (int64_t)y * k.ays + j);
    }
    float qR = 0.f;
    if (k.last) qR = dst[O * k.S];
    const bool yin = k.zin && y > 0 && y < k.ny - 1;
    float out[O];
    if (yin) {
        float L[O];
        if (k.exi > 0) {
#pragma unroll
            for (int j = 0; j < O; j++) L[j] = __ldg(here + (j - O) * k.S);
        } else {
#pragma unroll
            for (int j = 0; j < O; j++) L[j] = 0.f;
        }
        const float R = __ldg(here + O * k.S);
        float az[O];
        zterm_rt<O>(k.lz, P[K], buf + k.srow * O * 32 + lane, az);
        const float wy = cb_wa[O - 1][K];
        const float gxz = k.g0 * (k.wz * wy), gz0 = k.g1 * wy, gy0 = k.g2 * k.wz;
#pragma unroll
        for (int j = 0; j < O; j++) {
            const float c = P[K][j];
            float ax = 0.f;
#pragma unroll
            for (int d = -O; d <= O; d++) {
                if (d == 0 || d < blo(O, j) || d > bhi(O, j)) continue;
                const int m = j + d;
                float v;
                if (m < 0) v = L[m + O];
                else if (m < O) v = P[K][m];
                else v = R;
                ax = fmaf(Tc<O>(j, d), v - c, ax);
            }
            float ay = K == 0 ? pend[j] : 0.f;
#pragma unroll
            for (int d = blo(O, K); d <= bhi(O, K); d++) {
                if (d == 0 || (K == 0 && d < 0)) continue;
                ay = fmaf(Tc<O>(K, d), P[K + d][j] - c, ay);
            }
            const float s = SPONGE ? sxv[j] * syv * k.szv : 1.f;
            const float qd = SPONGE ? s * q[j] : q[j];
            const float wxj = cb_wa[O - 1][j];
            const float yv = gxz * ax + (gz0 * wxj) * az[j] + (gy0 * wxj) * ay;
            float v = (2.f * c - qd) - am[j] * yv;
            if (j == 0 && k.exi == 0) v = qd;  // x = 0 face
            out[j] = SPONGE ? s * v : v;
        }
    } else {
#pragma unroll
        for (int j = 0; j < O; j++) {
            const float s = SPONGE ? sxv[j] * syv * k.szv : 1.f;
            out[j] = SPONGE ? s * (s * q[j]) : q[j];
        }
    }
#pragma unroll
    for (int j = 0; j < O; j++) dst[j * k.S] = out[j];
    if (k.last) {
        const float s = SPONGE ? sxv[O] * syv * k.szv : 1.f;
        dst[O * k.S] = SPONGE ? s * (s * qR) : qR;
    }
}

template <int O, bool SPONGE, int K = 0>
__device__ __forceinline__ void element_planes(const BatchArgs &a, const ColumnCtx &k, int y0, const float (&sxv)[O + 1],
                                        const float (&P)[O + 1][O], const float (&pend)[O], float (&hnext)[2][O])
{
    plane_step<O, SPONGE, K>(a, k, y0, sxv, P, pend, hnext);
    if constexpr (K + 1 < O) element_planes<O, SPONGE, K + 1>(a, k, y0, sxv, P, pend, hnext);
}

template <int O, bool SPONGE>
__global__ void __launch_bounds__(32 * ZR, 2) k_batch(const BatchArgs a, int ex)
{
    __shared__ __align__(16) float stage[2 * stage_floats<O>()];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t nz = a.nz;
    const int zgroups = (int)((nz + ZR - 1) / ZR);
    const int exi = blockIdx.x / zgroups, z0 = (blockIdx.x - exi * zgroups) * ZR;
    const int z = z0 + warp;
    const int x0 = exi * O;
    ColumnCtx k;
    k.S = a.s_pad;
    k.zs = a.nxp * k.S;
    k.ys = a.nxp * nz * k.S;
    k.ays = a.nxp * nz;
    const int64_t shot = (int64_t)blockIdx.z * 32 + lane;
    k.row_ok = z < nz;
    const int zc = k.row_ok ? z : (int)nz - 1;  // clamped for address arithmetic only
    k.cur0 = a.cur + ((int64_t)x0 + (int64_t)zc * a.nxp) * k.S + shot;
    k.prv0 = a.prev + ((int64_t)x0 + (int64_t)zc * a.nxp) * k.S + shot;
    k.a0 = a.a + x0 + (int64_t)zc * a.nxp;
    k.ny = (int)a.ny;
    const int yb = blockIdx.y * a.ychunk;  // a multiple of O
    k.ye = (int)min((int64_t)k.ny, (int64_t)yb + a.ychunk);
    k.exi = exi;
    k.last = exi == ex - 1;
    k.lz = zc % O;
    k.zin = z > 0 && z < nz - 1;
    k.szv = SPONGE ? __ldg(a.sz + zc) : 1.f;
    k.wz = cb_wa[O - 1][k.lz];
    k.g0 = a.g[0];
    k.g1 = a.g[1];
    k.g2 = a.g[2];
    k.stage = stage;
    k.srow = warp + O;
    // halo rows: stage rows 0..O-1 are z0-O..z0-1, rows ZR+O..ZR+2O-1 are z0+ZR..z0+ZR+O-1
#pragma unroll
    for (int t = 0; t < 2; t++) {
        const int hr = warp + t * ZR;  // halo index 0 .. 2O-1
        k.hsrc[t] = nullptr;
        k.hrow[t] = 0;
        if (hr < 2 * O) {
            const int srow = hr < O ? hr : ZR + hr;
            const int zz = z0 - O + srow;
            k.hrow[t] = srow;
            if (zz >= 0 && zz < nz) k.hsrc[t] = a.cur + ((int64_t)x0 + (int64_t)zz * a.nxp) * k.S + shot;
        }
    }
    float sxv[O + 1];
#pragma unroll
    for (int j = 0; j <= O; j++) sxv[j] = SPONGE && (j < O || k.last) ? __ldg(a.sx + x0 + j) : 1.f;
    float hnext[2][O];
#pragma unroll
    for (int t = 0; t < 2; t++)
#pragma unroll
        for (int j = 0; j < O; j++) hnext[t][j] = k.hsrc[t] ? __ldg(k.hsrc[t] + (int64_t)yb * k.ys + j * k.S) : 0.f;
    float P[O + 1][O];
    float pend[O];
    const int e0 = yb / O;
    if (e0 > 0) {
#pragma unroll
        for (int kk = 0; kk <= O; kk++)
#pragma unroll
            for (int j = 0; j < O; j++) P[kk][j] = __ldg(k.cur0 + (int64_t)(yb - O + kk) * k.ys + j * k.S);
#pragma unroll
        for (int j = 0; j < O; j++) {
            float acc = 0.f;
#pragma unroll
            for (int d = -O; d <= -1; d++) acc = fmaf(Tc<O>(0, d), P[O + d][j] - P[O][j], acc);
            pend[j] = acc;
            P[0][j] = P[O][j];
        }
    } else {
#pragma unroll
        for (int j = 0; j < O; j++) {
            pend[j] = 0.f;
            P[0][j] = __ldg(k.cur0 + (int64_t)yb * k.ys + j * k.S);
        }
    }
    for (int y0 = e0 * O; y0 < k.ye; y0 += O) {
#pragma unroll
        for (int kk = 1; kk <= O; kk++)
#pragma unroll
            for (int j = 0; j < O; j++)
                P[kk][j] = y0 + kk < k.ny ? __ldg(k.cur0 + (int64_t)(y0 + kk) * k.ys + j * k.S) : 0.f;
        element_planes<O, SPONGE>(a, k, y0, sxv, P, pend, hnext);
#pragma unroll
        for (int j = 0; j < O; j++) {
            float acc = 0.f;
#pragma unroll
            for (int d = -O; d <= -1; d++) acc = fmaf(Tc<O>(0, d), P[O + d][j] - P[O][j], acc);
            pend[j] = acc;
            P[0][j] = P[O][j];
        }
    }
}

template <int O>
cudaError_t launch_o(const BatchArgs &a0, bool sponge, cudaStream_t st)
{
    BatchArgs a = a0;
    a.ychunk = (a.ychunk + O - 1) / O * O;
    if (a.s_pad % 32) return cudaErrorInvalidValue;
    const int ex = (int)((a.nx - 1) / O);
    const int zgroups = (int)((a.nz + ZR - 1) / ZR);
    const dim3 grid((unsigned)(ex * zgroups), (unsigned)((a.ny + a.ychunk - 1) / a.ychunk), (unsigned)(a.s_pad / 32));
    if (sponge) k_batch<O, true><<<grid, 32 * ZR, 0, st>>>(a, ex);
    else k_batch<O, false><<<grid, 32 * ZR, 0, st>>>(a, ex);
    return cudaGetLastError();
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

}  // namespace

cudaError_t batch_kernel_setup(const float *T_all, const float *wa_all)
{
    cudaError_t e = cudaMemcpyToSymbol(cb_T, T_all, sizeof(float) * kMaxOrder * kTBMax);
    if (e != cudaSuccess) return e;
    return cudaMemcpyToSymbol(cb_wa, wa_all, sizeof(float) * kMaxOrder * kMaxOrder);
}

cudaError_t launch_batch_step(int order, const BatchArgs &a, bool sponge, const BatchTuning &t, cudaStream_t st)
{
    (void)t.warps_per_cta;  // the CTA is fixed at 8 z-rows; the tuner picks the y-chunk
    switch (order) {
    case 1: return launch_o<1>(a, sponge, st);
    case 2: return launch_o<2>(a, sponge, st);
    case 3: return launch_o<3>(a, sponge, st);
    case 4: return launch_o<4>(a, sponge, st);
    case 5: return launch_o<5>(a, sponge, st);
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
