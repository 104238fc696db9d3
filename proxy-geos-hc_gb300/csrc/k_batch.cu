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

// Neighbours of one node along x or z for the compile-time local index L, loaded up front so
// that every load of a plane is in flight at once (offsets blo..bhi, 0 excluded).
template <int O, int L, int SPL>
struct Nbr {
    static constexpr int lo = blo(O, L), hi = bhi(O, L);
    Sv<SPL> v[hi - lo + 1];
    __device__ __forceinline__ void load(const float *c, int64_t stride)
    {
#pragma unroll
        for (int d = lo; d <= hi; d++)
            if (d != 0) v[d - lo] = ldv<SPL>(c + d * stride);
    }
    __device__ __forceinline__ Sv<SPL> operator()(int d) const { return v[d - lo]; }
};

struct ColumnCtx {
    const float *cur_col;  // p^n at (x, 0, z), this lane's first shot
    float *prv_col;
    const float *a_col;    // dt^2/M at (x, 0, z)
    int64_t sx_stride, sz_stride, sy_stride, a_ystride;
    int yb, ye;
    float sx, sz;              // sponge factors of the column
    float gx0, gz0, gy0;       // geometric factors g_d
};

// One interior (x, z) column: x- and z-local indices LX, LZ are compile-time, so every
// neighbour offset and coefficient is an immediate; the y-local index cycles at run time.
template <int O, int SPL, bool SPONGE, int LX, int LZ>
__device__ __forceinline__ void interior_column(const BatchArgs &a, const ColumnCtx &k)
{
    const float wx = cb_wa[O - 1][LX], wz = cb_wa[O - 1][LZ];
    Sv<SPL> q[2 * O + 1];  // p^n at planes y-O..y+O of this column, this lane's shots
#pragma unroll
    for (int j = 0; j < 2 * O; j++) {
        const int yy = k.yb - O + j;
        if (yy >= 0 && yy < a.ny) q[j] = ldv<SPL>(k.cur_col + yy * k.sy_stride);
        else
#pragma unroll
            for (int t = 0; t < SPL; t++) q[j].v[t] = 0.f;
    }
    int ly = k.yb % O;
    for (int y = k.yb; y < k.ye; y++) {
        // every load of this plane first
        const bool top = y + O < a.ny;
        const Sv<SPL> qn = ldv<SPL>(k.cur_col + (int64_t)(top ? y + O : y) * k.sy_stride);
        const float *here = k.cur_col + (int64_t)y * k.sy_stride;
        Nbr<O, LX, SPL> nx;
        nx.load(here, k.sx_stride);
        Nbr<O, LZ, SPL> nz;
        nz.load(here, k.sz_stride);
        const Sv<SPL> qv = ldv<SPL>(k.prv_col + (int64_t)y * k.sy_stride);
        const float am = __ldg(k.a_col + (int64_t)y * k.a_ystride);
        const float s = SPONGE ? k.sx * __ldg(a.sy + y) * k.sz : 1.f;  // (sx*sy)*sz
        if (top) q[2 * O] = qn;
        else
#pragma unroll
            for (int t = 0; t < SPL; t++) q[2 * O].v[t] = 0.f;
        const Sv<SPL> c = q[O];
        Sv<SPL> ax, az;
#pragma unroll
        for (int t = 0; t < SPL; t++) ax.v[t] = az.v[t] = 0.f;
        axis_term<O, LX, SPL>(c, nx, ax);
        axis_term<O, LZ, SPL>(c, nz, az);
        const Sv<SPL> ay = axis<O, SPL>(ly, c, Queue<O, SPL>{q});
        const float wy = cb_wa[O - 1][ly];
        const float gx = k.gx0 * (wz * wy), gz = k.gz0 * (wx * wy), gy = k.gy0 * (wx * wz);
        const bool yin = y > 0 && y < a.ny - 1;
        Sv<SPL> out;
#pragma unroll
        for (int t = 0; t < SPL; t++) {
            const float qd = SPONGE ? s * qv.v[t] : qv.v[t];
            const float yv = gx * ax.v[t] + gz * az.v[t] + gy * ay.v[t];
            const float v = yin ? (2.f * c.v[t] - qd) - am * yv : qd;
            out.v[t] = SPONGE ? s * v : v;
        }
        stv<SPL>(k.prv_col + (int64_t)y * k.sy_stride, out);
#pragma unroll
        for (int j = 0; j < 2 * O; j++) q[j] = q[j + 1];
        ly = ly + 1 == O ? 0 : ly + 1;
    }
}

// Columns on the x or z faces: Dirichlet nodes keep the damped previous level.
template <int SPL, bool SPONGE>
__device__ __forceinline__ void face_column(const BatchArgs &a, const ColumnCtx &k)
{
    for (int y = k.yb; y < k.ye; y++) {
        const Sv<SPL> qv = ldv<SPL>(k.prv_col + (int64_t)y * k.sy_stride);
        const float s = SPONGE ? k.sx * __ldg(a.sy + y) * k.sz : 1.f;
        Sv<SPL> out;
#pragma unroll
        for (int t = 0; t < SPL; t++) out.v[t] = SPONGE ? s * (s * qv.v[t]) : qv.v[t];
        stv<SPL>(k.prv_col + (int64_t)y * k.sy_stride, out);
    }
}

template <int O, int SPL, bool SPONGE, int LX = 0, int LZ = 0>
__device__ __forceinline__ void dispatch_column(int lx, int lz, const BatchArgs &a, const ColumnCtx &k)
{
    if (lx == LX && lz == LZ) {
        interior_column<O, SPL, SPONGE, LX, LZ>(a, k);
        return;
    }
    if constexpr (LZ + 1 < O) dispatch_column<O, SPL, SPONGE, LX, LZ + 1>(lx, lz, a, k);
    else if constexpr (LX + 1 < O) dispatch_column<O, SPL, SPONGE, LX + 1, 0>(lx, lz, a, k);
}

template <int O, int SPL, bool SPONGE>
__global__ void __launch_bounds__(512) k_batch(const BatchArgs a)
{
    const int warps = blockDim.x >> 5;
    const int lane = threadIdx.x & 31;
    const int64_t col = (int64_t)blockIdx.x * warps + (threadIdx.x >> 5);  // x fastest
    if (col >= a.nx * a.nz) return;
    const int64_t z = col / a.nx, x = col - z * a.nx;
    ColumnCtx k;
    const int64_t S = a.s_pad;
    k.sx_stride = S;
    k.sz_stride = a.nxp * S;
    k.sy_stride = a.nxp * a.nz * S;
    k.a_ystride = a.nxp * a.nz;
    const int64_t shot0 = (int64_t)blockIdx.z * 32 * SPL + lane * SPL;  // this lane's first shot
    k.yb = blockIdx.y * a.ychunk;
    k.ye = (int)min(a.ny, (int64_t)k.yb + a.ychunk);
    k.cur_col = a.cur + x * S + z * k.sz_stride + shot0;
    k.prv_col = a.prev + x * S + z * k.sz_stride + shot0;
    k.a_col = a.a + x + z * a.nxp;
    k.sx = SPONGE ? __ldg(a.sx + x) : 1.f;
    k.sz = SPONGE ? __ldg(a.sz + z) : 1.f;
    k.gx0 = a.g[0];
    k.gz0 = a.g[1];
    k.gy0 = a.g[2];
    const bool xz_in = x > 0 && x < a.nx - 1 && z > 0 && z < a.nz - 1;
    if (!xz_in) {
        face_column<SPL, SPONGE>(a, k);
        return;
    }
    dispatch_column<O, SPL, SPONGE>((int)(x % O), (int)(z % O), a, k);
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
