// stencil_body.cuh -- device code of the fused SEM step on a uniform box (k_stencil.cu: the
// kernels over one box; k_group.cu: one launch over the boxes of a group).  The operator, work
// decomposition and pipeline are described in k_stencil.cu.  Included by one translation unit
// each; the constant tables below are that unit's own (upload_stencil_constants fills them).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <type_traits>
#include <vector>

#include "stencil.h"
#include "tma.cuh"

namespace semgb {

namespace {

// Tiling and arithmetic knobs (compile-time; the defaults are the measured best on GB300, other
// values are for sweeps: build.py -D NAME=value builds a separate library).  Both settings of the
// two packing knobs give the same bits: a packed f32x2 instruction rounds each half as the scalar
// instruction does.
#ifndef SEM_STENCIL_LOOKAHEAD
#define SEM_STENCIL_LOOKAHEAD 1  // planes loaded into shared memory ahead of the compute
#endif
#ifndef SEM_STENCIL_NG
#define SEM_STENCIL_NG 2  // row groups per thread where the order allows it
#endif
#ifndef SEM_STENCIL_PACKED
#define SEM_STENCIL_PACKED 1  // the per-node update of node pairs in packed f32x2 arithmetic
#endif
#ifndef SEM_STENCIL_PACKED_AXIS
#define SEM_STENCIL_PACKED_AXIS 1  // even orders, direct form: z- and y-terms on packed node pairs
#endif
#ifndef SEM_STENCIL_RW
#define SEM_STENCIL_RW 2  // rows per warp instruction where the order allows it
#endif
#ifndef SEM_STENCIL_L2PF
#define SEM_STENCIL_L2PF 2  // planes beyond the look-ahead prefetched into L2
#endif
constexpr int kLook = SEM_STENCIL_LOOKAHEAD;  // planes of lookahead
constexpr int kL2Pf = SEM_STENCIL_L2PF;       // further planes prefetched into L2 (0: none)
constexpr uint64_t kWaitLimitNs = 2000000000ull;
constexpr int kTMax = kMaxOrder * (2 * kMaxOrder + 1);
__constant__ float c_T[kMaxOrder][kTMax];  // [order-1][l * (2o+1) + d + o]
__constant__ float2 c_T2[kMaxOrder][kTMax];  // the same coefficients twice, for packed node pairs
__constant__ float c_wa[kMaxOrder][kMaxOrder];  // assembled weights by local index

// Rows per warp instruction of the square order-4 tile (32 x 32 nodes; the default is 64 x 16),
// which a single-shot pass can take where it wastes fewer lanes on the last x- and z-tiles.
constexpr int kSquareRW = 4;

template <int O, int RWS = SEM_STENCIL_RW>
struct Cfg {
    // Orders 1-4 (o divides the warp count: 4 warps, 3 for o = 3): a warp's lanes split into RW
    // sets on rows o apart, and each thread owns NG row groups a further o*RW rows apart, all
    // with the same z-local index (warp-uniform coefficients).  Narrow tiles waste fewer lanes
    // on the last x-tile of a row (801 nodes: 13 tiles of 64 against 7 of 128; 289 nodes at
    // o = 3: 7 of 48 against 4 of 96); the groups share one thread's per-plane bookkeeping
    // (waits, slot selection, coefficient dispatch, sponge).  Order 5: 5 warps, four rows per
    // warp instruction (8 lanes each), one group, tiles of 40 x 20 (801^3 nodes: 242.8
    // Gnode-steps/s, against 234.5 with one row per warp and 8 warps on 160 x 8 tiles and 219.7
    // with row pairs on 80 x 10 tiles).
    static constexpr bool SPLIT = O <= 4;
    static constexpr int NG = SPLIT ? SEM_STENCIL_NG : 1;  // row groups per thread
    static constexpr int WARPS = !SPLIT ? 5 : (O == 3 ? 3 : 8 / NG);
    static constexpr int RW = SPLIT ? RWS : 4;
    static constexpr int LANES = 32 / RW;               // lanes per row
    static constexpr int GR = O * RW;                   // rows between a thread's groups
    static constexpr int TZ = WARPS * RW * NG;          // rows per CTA
    static constexpr int THREADS = 32 * WARPS;
    static constexpr int TX = LANES * O;                // nodes along x per CTA
    static constexpr int HX = O <= 4 ? 4 : 8;           // x halo, a multiple of 4 floats
    static constexpr int TXP = TX + 2 * HX;             // window row length
    static constexpr int TZP = TZ + 2 * O;              // window rows: tile plus z halo
    static constexpr int W = 2 * O + 1;
    static constexpr int R = W + kLook;                 // ring slots
    static constexpr int AUX = kLook + 1;               // aux slots
    static constexpr size_t al(size_t b) { return (b + 127) / 128 * 128; }
    static constexpr int TILE_FLOATS = (int)(al(sizeof(float) * TZ * TX) / 4);
    static constexpr int WIN_FLOATS = (int)(al(sizeof(float) * TZP * TXP) / 4);  // plane with halos
    static constexpr int RING_FLOATS = TILE_FLOATS;     // y-ring: tile rows only
    static constexpr int AUX_FLOATS = 2 * TILE_FLOATS + WIN_FLOATS;  // p^{n-1}, dt^2/M tiles; p^n window
    static constexpr size_t OFF_AUX = (size_t)R * RING_FLOATS * 4;
    static constexpr size_t OFF_BAR = OFF_AUX + (size_t)AUX * AUX_FLOATS * 4;
    static constexpr size_t SMEM = OFF_BAR + 8 * (R + AUX);
    static constexpr uint32_t RING_TX = sizeof(float) * TZ * TX;
    static constexpr uint32_t AUX_TX = sizeof(float) * (2 * TZ * TX + TZP * TXP);
    // CTAs per SM that shared memory allows (228 KB per SM, 1 KB reserved per CTA), at most 6;
    // the register cap follows from it
    static constexpr int BY_SMEM = (int)(233472 / (SMEM + 1024));
    static constexpr int MIN_BLOCKS = BY_SMEM < 1 ? 1 : (BY_SMEM > 6 ? 6 : BY_SMEM);
};

// Offsets d with a non-zero coefficient for local index l: [-o, o] for l == 0 (element face),
// [-l, o-l] otherwise.
__host__ __device__ constexpr int dlo(int O, int l) { return l == 0 ? -O : -l; }
__host__ __device__ constexpr int dhi(int O, int l) { return l == 0 ? O : O - l; }

template <int O>
__device__ __forceinline__ void load_o(const float *p, float (&v)[O])
{
    if constexpr (O == 4) {
        const float4 t = *reinterpret_cast<const float4 *>(p);
        v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
    } else if constexpr (O == 2) {
        const float2 t = *reinterpret_cast<const float2 *>(p);
        v[0] = t.x; v[1] = t.y;
    } else {
#pragma unroll
        for (int j = 0; j < O; j++) v[j] = p[j];
    }
}

// As load_o, for a run of which only the first `lim` values lie inside the row's allocation
// (padding columns included); the others read as zero.
template <int O>
__device__ __forceinline__ void load_o_lim(const float *p, float (&v)[O], int lim)
{
    if (lim >= O) {
        load_o<O>(p, v);
    } else {
#pragma unroll
        for (int j = 0; j < O; j++) v[j] = j < lim ? p[j] : 0.f;
    }
}

// Stores O values at p, of which the first `lim` lie inside the row's allocation (padding
// columns included); one vector store when all do and the width allows it.
template <int O>
__device__ __forceinline__ void store_o_lim(float *p, const float (&v)[O], int lim)
{
    if constexpr (O == 4) {
        if (lim >= 4) { *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]); return; }
    } else if constexpr (O == 2) {
        if (lim >= 2) { *reinterpret_cast<float2 *>(p) = make_float2(v[0], v[1]); return; }
    }
#pragma unroll
    for (int j = 0; j < O; j++)
        if (j < lim) p[j] = v[j];
}

template <int O, int NG>
struct VecG {
    float v[NG][O];
};

// Axis term along a direction whose local index LOC is uniform over the thread's NG groups of O
// nodes: direct form r[g][j] = sum_d T[LOC][d] row_g(d)[j] (diagonal included), difference form
// r[g][j] = sum_{d!=0} T[LOC][d] (row_g(d)[j] - c[g][j]).  row(d) returns the pointer to group
// 0's O values at offset d along the axis; group g's lie g*GS floats further.
template <int O, int NG, int GS, int LOC, bool DIRECT, class RowFn>
__device__ __forceinline__ VecG<O, NG> axis_uniform(const float (&c)[NG][O], const RowFn &row)
{
    VecG<O, NG> r;
    if constexpr (DIRECT && SEM_STENCIL_PACKED_AXIS && O % 2 == 0) {
        // node pairs in packed f32x2 with the coefficient pair from the constant bank: the same
        // products and sums in the same order as the scalar form below, each half rounded alike
        float2 rr[NG][O / 2];
        const float2 td = c_T2[O - 1][LOC * (2 * O + 1) + O];
#pragma unroll
        for (int g = 0; g < NG; g++)
#pragma unroll
            for (int jp = 0; jp < O / 2; jp++) rr[g][jp] = mul2(td, make_float2(c[g][2 * jp], c[g][2 * jp + 1]));
#pragma unroll
        for (int d = dlo(O, LOC); d <= dhi(O, LOC); d++) {
            if (d == 0) continue;
            const float *p = row(d);
            const float2 tt = c_T2[O - 1][LOC * (2 * O + 1) + d + O];
#pragma unroll
            for (int g = 0; g < NG; g++) {
                float v[O];
                load_o<O>(p + g * GS, v);
#pragma unroll
                for (int jp = 0; jp < O / 2; jp++) rr[g][jp] = fma2(tt, make_float2(v[2 * jp], v[2 * jp + 1]), rr[g][jp]);
            }
        }
#pragma unroll
        for (int g = 0; g < NG; g++)
#pragma unroll
            for (int jp = 0; jp < O / 2; jp++) {
                r.v[g][2 * jp] = rr[g][jp].x;
                r.v[g][2 * jp + 1] = rr[g][jp].y;
            }
    } else if constexpr (DIRECT) {
        // the coefficients are constant-bank operands of scalar fmas
#pragma unroll
        for (int g = 0; g < NG; g++)
#pragma unroll
            for (int j = 0; j < O; j++) r.v[g][j] = c_T[O - 1][LOC * (2 * O + 1) + O] * c[g][j];
#pragma unroll
        for (int d = dlo(O, LOC); d <= dhi(O, LOC); d++) {
            if (d == 0) continue;
            const float *p = row(d);
#pragma unroll
            for (int g = 0; g < NG; g++) {
                float v[O];
                load_o<O>(p + g * GS, v);
#pragma unroll
                for (int j = 0; j < O; j++) r.v[g][j] = fmaf(c_T[O - 1][LOC * (2 * O + 1) + d + O], v[j], r.v[g][j]);
            }
        }
    } else {
#pragma unroll
        for (int g = 0; g < NG; g++)
#pragma unroll
            for (int j = 0; j < O; j++) r.v[g][j] = 0.f;
#pragma unroll
        for (int d = dlo(O, LOC); d <= dhi(O, LOC); d++) {
            if (d == 0) continue;
            const float *p = row(d);
            const float t = c_T[O - 1][LOC * (2 * O + 1) + d + O];
#pragma unroll
            for (int g = 0; g < NG; g++) {
                float v[O];
                load_o<O>(p + g * GS, v);
                if constexpr (O % 2 == 0) {
                    // the coefficient is shared by the thread's nodes: pairs of nodes in packed
                    // f32x2 (each half rounds as the scalar sub and fma would)
#pragma unroll
                    for (int j = 0; j < O; j += 2) {
                        const float2 acc = fma2(make_float2(t, t),
                                                sub2(make_float2(v[j], v[j + 1]), make_float2(c[g][j], c[g][j + 1])),
                                                make_float2(r.v[g][j], r.v[g][j + 1]));
                        r.v[g][j] = acc.x;
                        r.v[g][j + 1] = acc.y;
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < O; j++) r.v[g][j] = fmaf(t, v[j] - c[g][j], r.v[g][j]);
                }
            }
        }
    }
    return r;
}

// Axis term of the reference-rounding pass: continues the node's accumulation r (x-term already
// in it) with sum_{d!=0} C[d][j] row_g(d)[j], C the node-class coefficients of this axis
// (cb + LOC*stride points to the [2o+1][o] block of the thread's class), in order of d.
template <int O, int NG, int GS, int LOC, class RowFn>
__device__ __forceinline__ VecG<O, NG> axis_class(VecG<O, NG> r, const float *cb0, int stride, const RowFn &row)
{
    const float *cb = cb0 + LOC * stride;
#pragma unroll
    for (int d = dlo(O, LOC); d <= dhi(O, LOC); d++) {
        if (d == 0) continue;
        const float *p = row(d);
        const float *cd = cb + (d + O) * O;
#pragma unroll
        for (int g = 0; g < NG; g++) {
            float v[O];
            load_o<O>(p + g * GS, v);
            if constexpr (SEM_STENCIL_PACKED_AXIS && O % 2 == 0) {
#pragma unroll
                for (int jp = 0; jp < O / 2; jp++) {
                    const float2 acc = fma2(*reinterpret_cast<const float2 *>(cd + 2 * jp),
                                            make_float2(v[2 * jp], v[2 * jp + 1]),
                                            make_float2(r.v[g][2 * jp], r.v[g][2 * jp + 1]));
                    r.v[g][2 * jp] = acc.x;
                    r.v[g][2 * jp + 1] = acc.y;
                }
            } else {
#pragma unroll
                for (int j = 0; j < O; j++) r.v[g][j] = fmaf(cd[j], v[j], r.v[g][j]);
            }
        }
    }
    return r;
}

template <int O, int NG, int GS, class RowFn>
__device__ __forceinline__ VecG<O, NG> axis_class_dispatch(int loc, const VecG<O, NG> &r, const float *cb0, int stride,
                                                          const RowFn &row)
{
    switch (loc) {
    case 0: return axis_class<O, NG, GS, 0>(r, cb0, stride, row);
    case 1: if constexpr (O > 1) return axis_class<O, NG, GS, 1>(r, cb0, stride, row);
    case 2: if constexpr (O > 2) return axis_class<O, NG, GS, 2>(r, cb0, stride, row);
    case 3: if constexpr (O > 3) return axis_class<O, NG, GS, 3>(r, cb0, stride, row);
    default: if constexpr (O > 4) return axis_class<O, NG, GS, 4>(r, cb0, stride, row);
    }
    return axis_class<O, NG, GS, 0>(r, cb0, stride, row);  // not reached: loc < O
}

template <int O, int NG, int GS, bool DIRECT, class RowFn>
__device__ __forceinline__ VecG<O, NG> axis_dispatch(int loc, const float (&c)[NG][O], const RowFn &row)
{
    switch (loc) {
    case 0: return axis_uniform<O, NG, GS, 0, DIRECT>(c, row);
    case 1: if constexpr (O > 1) return axis_uniform<O, NG, GS, 1, DIRECT>(c, row);
    case 2: if constexpr (O > 2) return axis_uniform<O, NG, GS, 2, DIRECT>(c, row);
    case 3: if constexpr (O > 3) return axis_uniform<O, NG, GS, 3, DIRECT>(c, row);
    default: if constexpr (O > 4) return axis_uniform<O, NG, GS, 4, DIRECT>(c, row);
    }
    return axis_uniform<O, NG, GS, 0, DIRECT>(c, row);  // not reached: loc < O
}

// z-neighbour rows: window rows are contiguous over the tile and its z halo.
struct ZRows {
    const float *base;  // current plane, row of the thread's node, first column of its nodes
    int txp;
    __device__ __forceinline__ const float *operator()(int d) const { return base + d * txp; }
};

// y-neighbour rows: ring slot of plane y+d.  `base` points into the slot of plane y (index
// `slot` of R slots of SF floats); wrapping around the ring selects one of two precomputed
// bases, the offset d*SF being an immediate of the load.
template <int R, int SF>
struct YPlanes {
    const float *base, *base_lo, *base_hi;  // base, base + R*SF, base - R*SF
    int slot;
    __device__ __forceinline__ const float *operator()(int d) const
    {
        if (d > 0) return (slot >= R - d ? base_hi : base) + d * SF;
        return (slot < -d ? base_lo : base) + d * SF;
    }
};

struct NoClassTable {
    int unused;
};
template <int O, bool REF>
using ClassParam = typename std::conditional<REF, ClassTable<O>, NoClassTable>::type;


// REF: the reference-rounding operator -- every coefficient from the node-class table `ct`, one
// accumulation per node over the x-, z- and y-terms (direct form only).
//
// One CTA of the pass: tile (bx, bz) of shot `shot`, y-chunk `chunk`.  The tensor maps describe the
// current level (ring: tile boxes; win: tile plus halos), the stored previous level and dt^2/M.
// GROUP: the CTA may have more threads than the order's configuration uses (a launch that mixes
// orders); the extra threads take part in the barriers only.
template <int O, bool SPONGE, int MODE, bool DIRECT, bool MULTI, bool REF, bool GROUP, int RWS = SEM_STENCIL_RW>
__device__ __forceinline__ void stencil_cta(const CUtensorMap *rmap, const CUtensorMap *wmap, const CUtensorMap *pmap,
                                            const CUtensorMap *amap, const StencilTables &t, const StencilArgs &a,
                                            const ClassParam<O, REF> &ct, const int shot, const int bx, const int bz,
                                            const int chunk)
{
    static_assert(!REF || DIRECT, "the reference-rounding operator is a direct form");
    using C = Cfg<O, RWS>;
    constexpr int TZ = C::TZ, TX = C::TX, HX = C::HX, TXP = C::TXP, R = C::R, AUX = C::AUX;
    extern __shared__ __align__(128) unsigned char smem[];
    float *ring = reinterpret_cast<float *>(smem);
    float *aux = reinterpret_cast<float *>(smem + C::OFF_AUX);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + C::OFF_BAR);  // [R] ring, [AUX] aux

    const bool act = !GROUP || threadIdx.x < (unsigned)C::THREADS;  // a thread of the configuration
    const int tid = act ? (int)threadIdx.x : 0;  // extra threads shadow thread 0 and store nothing
    const int w = tid >> 5, l = tid & 31;
    const int x0 = bx * TX, z0 = bz * TZ;
    const int yb = chunk * t.ychunk;
    const int ys = MULTI ? shot * (int)t.ny : 0;  // plane offset of the shot in the stacked levels
    const int ye = (int)min((int64_t)t.ny, (int64_t)yb + t.ychunk);
    const int nx = (int)t.nx, nz = (int)t.nz, ny = (int)t.ny;

    // ring plane p (p >= yb - O) lives in slot (p - yb + O) % R; aux plane p in (p - yb) % AUX
    auto issue_ring = [=](int p) {
        const int i = (p - yb + O) % R;
        bar_arrive_expect_tx(bars + i, C::RING_TX);
        tma_load_3d(ring + i * C::RING_FLOATS, rmap, x0, z0, ys + p, bars + i);
    };
    auto issue_aux = [=](int p) {
        const int i = (p - yb) % AUX;
        float *b = aux + i * C::AUX_FLOATS;
        bar_arrive_expect_tx(bars + R + i, C::AUX_TX);
        tma_load_3d(b, pmap, x0, z0, ys + p, bars + R + i);
        tma_load_3d(b + C::TILE_FLOATS, amap, x0, z0, p, bars + R + i);  // shared by the shots
        tma_load_3d(b + 2 * C::TILE_FLOATS, wmap, x0 - HX, z0 - O, ys + p, bars + R + i);
    };

    if (threadIdx.x == 0) {
        for (int i = 0; i < R + AUX; i++) bar_init(bars + i, 1);
        fence_barrier_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int p = yb - O; p <= min(yb + O + kLook - 1, ye - 1 + O); p++) issue_ring(p);
        for (int p = yb; p <= min(yb + kLook - 1, ye - 1); p++) issue_aux(p);
    }

    // per-thread constants.  Tile row of the thread's group 0 and its x position: the rows of
    // one warp (and of all groups of a thread) share z mod O; group g lies g*GR rows further.
    constexpr int NG = C::NG, GR = C::GR;
    const int xl = l % C::LANES;
    const int rw = C::RW == 1 && NG == 1 ? w : (w / O) * (O * C::RW * NG) + w % O + (l / C::LANES) * O;
    const int z = z0 + rw;
    const int lz = z % O;
    const int xb = x0 + O * xl;  // first node of the thread
    float sxv[O];
#pragma unroll
    for (int j = 0; j < O; j++) sxv[j] = (SPONGE && xb + j < nx) ? __ldg(a.sx + xb + j) : 1.f;
    bool row_ok[NG], zin[NG];
    bool zin_all = true;
    float sxz[NG][O];  // (sx*sz) of the thread's nodes; the node factor is (sx*sz)*sy
#pragma unroll
    for (int g = 0; g < NG; g++) {
        const int zg = z + g * GR;
        row_ok[g] = act && zg < nz;
        zin[g] = zg > 0 && zg < nz - 1;
        zin_all = zin_all && zin[g];
        const float szv = (SPONGE && row_ok[g]) ? __ldg(a.sz + zg) : 1.f;
#pragma unroll
        for (int j = 0; j < O; j++) sxz[g][j] = sxv[j] * szv;
    }
    const float wz = c_wa[O - 1][lz];
    const int off = (rw + O) * TXP + HX + O * xl;  // offset of the thread's first node in the window
    const int toff = rw * TX + O * xl;             // in-tile offset (aux tiles, y-ring slots)
    // loop-invariant fields of the tables and arguments, read once: the level stores below cannot
    // change them, which the compiler cannot tell through the references
    const float tg0 = t.g[0], tg1 = t.g[1], tg2 = t.g[2];
    const int64_t nxp = t.nxp;
    const float *const a_sy = a.sy;
    float *const a_kp = a.kp;
    float *const a_grad = a.grad;
    int *const a_status = a.status;
    float *const a_prev = a.prev;
    float *dst_col = a_prev + (MULTI ? (int64_t)shot * t.shot_stride : 0) + (int64_t)xb + (int64_t)z * nxp;
    const int64_t plane_stride = nxp * t.nz;
    const int64_t group_stride = (int64_t)GR * nxp;

    bool ok = true;
    for (int p = yb - O; p < yb + O; p++) {
        const int i = p - yb + O;  // < 2O < R: first fill of each of these slots
        ok &= bar_wait(bars + i, 0, kWaitLimitNs);
    }
    if (!ok) atomicExch(a_status, 1);
    bool aborted = __syncthreads_or(!ok) != 0;

    // all nodes of the thread strictly inside the mesh along x and z: no per-node checks on the
    // common path
    const bool xall = xb > 0 && xb + O < nx;
    const bool inner = xall && zin_all;

    int rs = O;         // ring slot of plane y
    int ws = 2 * O;     // ring slot of plane y+O, the one waited for (2O < R), and its phase
    uint32_t wph = 0;
    int as = 0;         // aux slot of plane y and its phase
    uint32_t aph = 0;
    int ly = yb % O;
    for (int y = yb; y < ye && !aborted; y++) {
        if (threadIdx.x == 0 && y + kLook <= ye - 1) {
            issue_ring(y + O + kLook);
            issue_aux(y + kLook);
            if constexpr (kL2Pf > 0) {
                // tiles kL2Pf planes beyond the shared-memory look-ahead, into L2; only boxes that
                // lie inside the tensor (the window's halos are other CTAs' tiles)
                const int pr = y + O + kLook + kL2Pf, pa = y + kLook + kL2Pf;
                if (pr < ny) tma_prefetch_3d(rmap, x0, z0, ys + pr);
                if (pa <= ye - 1) {
                    tma_prefetch_3d(pmap, x0, z0, ys + pa);
                    tma_prefetch_3d(amap, x0, z0, pa);
                }
            }
        }
        // gradient pass: the recorded K p' and the running gradient of the thread's nodes, loaded
        // before the waits so that their latency overlaps the plane's work
        float kpv[NG][O], grv[NG][O];
        if constexpr (MODE == STENCIL_GRADIENT) {
            const int64_t so = (dst_col - a_prev) + (int64_t)y * plane_stride;
#pragma unroll
            for (int g = 0; g < NG; g++) {
                if (row_ok[g]) {
                    load_o_lim<O>(a_kp + so + g * group_stride, kpv[g], (int)nxp - xb);
                    load_o_lim<O>(a_grad + so + g * group_stride, grv[g], (int)nxp - xb);
                } else {
#pragma unroll
                    for (int j = 0; j < O; j++) kpv[g][j] = grv[g][j] = 0.f;
                }
            }
        }
        ok = bar_wait(bars + ws, wph, kWaitLimitNs);
        ok &= bar_wait(bars + R + as, aph, kWaitLimitNs);
        if (!ok) atomicExch(a_status, 1);
        {
            // rows past the mesh read zero-filled shared memory; only their stores are skipped
            const float *cur = aux + as * C::AUX_FLOATS + 2 * C::TILE_FLOATS + off;  // window
            const float *tq = aux + as * C::AUX_FLOATS + toff;
            float c[NG][O], left[NG][O], right[NG], q[NG][O], am[NG][O];
#pragma unroll
            for (int g = 0; g < NG; g++) {
                load_o<O>(cur + g * GR * TXP, c[g]);
                load_o<O>(cur + g * GR * TXP - O, left[g]);
                right[g] = cur[g * GR * TXP + O];
                load_o<O>(tq + g * GR * TX, q[g]);
                load_o<O>(tq + g * GR * TX + C::TILE_FLOATS, am[g]);
            }

            // x: local index j is compile-time
            float ax[NG][O];
            // REF: the class coefficients of the thread's nodes along x, [2o+1][o]
            const float *cx = nullptr;
            if constexpr (REF) cx = &ct.c[0][ly][lz][0][0];
#pragma unroll
            for (int g = 0; g < NG; g++)
#pragma unroll
                for (int j = 0; j < O; j++) {
                    float acc = REF ? cx[O * O + j] * c[g][j]
                                    : (DIRECT ? c_T[O - 1][j * (2 * O + 1) + O] * c[g][j] : 0.f);
                    // constant trip count, so that the loop unrolls together with j and every
                    // index below is a constant (a j-dependent range left it rolled, with the
                    // arrays in memory)
#pragma unroll
                    for (int d = -O; d <= O; d++) {
                        if (d == 0 || d < dlo(O, j) || d > dhi(O, j)) continue;
                        const int m = j + d;  // offset from the thread's first node, in [-O, O]
                        const float v = m < 0 ? left[g][m + O] : (m < O ? c[g][m] : right[g]);
                        acc = fmaf(REF ? cx[(d + O) * O + j] : c_T[O - 1][j * (2 * O + 1) + d + O],
                                   DIRECT ? v : v - c[g][j], acc);
                    }
                    ax[g][j] = acc;
                }
            const float *yb0 = ring + rs * C::RING_FLOATS + toff;
            const YPlanes<R, C::RING_FLOATS> yrows{yb0, yb0 + R * C::RING_FLOATS, yb0 - R * C::RING_FLOATS, rs};
            VecG<O, NG> az, ay;
            if constexpr (REF) {
                // one accumulation per node: x-terms, then z-terms, then y-terms, in order of d
                VecG<O, NG> r;
#pragma unroll
                for (int g = 0; g < NG; g++)
#pragma unroll
                    for (int j = 0; j < O; j++) r.v[g][j] = ax[g][j];
                constexpr int WO = (2 * O + 1) * O;
                r = axis_class_dispatch<O, NG, GR * TXP>(lz, r, &ct.c[1][ly][0][0][0], WO, ZRows{cur, TXP});
                ay = axis_class_dispatch<O, NG, GR * TX>(ly, r, &ct.c[2][0][lz][0][0], O * WO, yrows);
            } else {
                az = axis_dispatch<O, NG, GR * TXP, DIRECT>(lz, c, ZRows{cur, TXP});
                ay = axis_dispatch<O, NG, GR * TX, DIRECT>(ly, c, yrows);
            }

            const bool yin = y > 0 && y < ny - 1;
            const float wy = c_wa[O - 1][ly];
            const float syv = SPONGE ? __ldg(a_sy + y) : 1.f;
            const float gx = tg0 * (wz * wy), gzy = tg1 * wy, gyz = tg2 * wz;
            float *dst = dst_col + (int64_t)y * plane_stride;
            float out[NG][O], kp[NG][O], sv[NG][O], qdv[NG][O];
            if constexpr (SEM_STENCIL_PACKED && O > 1) {
                // node pairs in packed f32x2: the same operations in the same order as the
                // scalar form below, each half rounded as the scalar instruction; an odd order's
                // last node of the run alone
#pragma unroll
                for (int g = 0; g < NG; g++) {
#pragma unroll
                    for (int j = 0; j + 1 < O; j += 2) {
                        const float2 s2 = SPONGE ? mul2(make_float2(sxz[g][j], sxz[g][j + 1]), make_float2(syv, syv))
                                                 : make_float2(1.f, 1.f);
                        const float2 q2 = make_float2(q[g][j], q[g][j + 1]);
                        const float2 qd2 = SPONGE ? mul2(s2, q2) : q2;
                        float2 y2;
                        if constexpr (REF)
                            y2 = make_float2(ay.v[g][j], ay.v[g][j + 1]);
                        else
                            y2 = fma2(make_float2(c_wa[O - 1][j], c_wa[O - 1][j + 1]),
                                      fma2(make_float2(gyz, gyz), make_float2(ay.v[g][j], ay.v[g][j + 1]),
                                           mul2(make_float2(gzy, gzy), make_float2(az.v[g][j], az.v[g][j + 1]))),
                                      mul2(make_float2(gx, gx), make_float2(ax[g][j], ax[g][j + 1])));
                        // (2c - qd) - am*y: 2c is exact, then one fused multiply-add
                        const float2 t2 = sub2(mul2(make_float2(2.f, 2.f), make_float2(c[g][j], c[g][j + 1])), qd2);
                        const float2 o2 = fma2(make_float2(-am[g][j], -am[g][j + 1]), y2, t2);
                        sv[g][j] = s2.x; sv[g][j + 1] = s2.y;
                        qdv[g][j] = qd2.x; qdv[g][j + 1] = qd2.y;
                        out[g][j] = o2.x; out[g][j + 1] = o2.y;
                        if (MODE == STENCIL_RECORD_KP) { kp[g][j] = y2.x; kp[g][j + 1] = y2.y; }
                    }
                    if constexpr (O % 2 == 1) {
                        constexpr int j = O - 1;
                        sv[g][j] = SPONGE ? sxz[g][j] * syv : 1.f;
                        qdv[g][j] = SPONGE ? sv[g][j] * q[g][j] : q[g][j];
                        float yv;
                        if constexpr (REF)
                            yv = ay.v[g][j];
                        else
                            yv = fmaf(c_wa[O - 1][j], fmaf(gyz, ay.v[g][j], gzy * az.v[g][j]), gx * ax[g][j]);
                        out[g][j] = (2.f * c[g][j] - qdv[g][j]) - am[g][j] * yv;
                        if (MODE == STENCIL_RECORD_KP) kp[g][j] = yv;
                    }
                }
            } else {
#pragma unroll
                for (int g = 0; g < NG; g++) {
#pragma unroll
                    for (int j = 0; j < O; j++) {
                        const float wxj = c_wa[O - 1][j];
                        sv[g][j] = SPONGE ? sxz[g][j] * syv : 1.f;
                        qdv[g][j] = SPONGE ? sv[g][j] * q[g][j] : q[g][j];
                        // K.p at the node: g1 Wz Wy A_x + Wx (g2 Wy A_z + g3 Wz A_y)
                        float yv;
                        if constexpr (REF)
                            yv = ay.v[g][j];
                        else
                            yv = fmaf(wxj, fmaf(gyz, ay.v[g][j], gzy * az.v[g][j]), gx * ax[g][j]);
                        out[g][j] = (2.f * c[g][j] - qdv[g][j]) - am[g][j] * yv;
                        if (MODE == STENCIL_RECORD_KP) kp[g][j] = yv;
                    }
                }
            }
            if (!(inner && yin)) {
                // boundary and padding nodes: no update (the stored previous level is kept, then
                // damped), padding columns stay zero
#pragma unroll
                for (int g = 0; g < NG; g++)
#pragma unroll
                    for (int j = 0; j < O; j++) {
                        if (!(xb + j > 0 && xb + j < nx - 1 && zin[g] && yin)) {
                            out[g][j] = qdv[g][j];
                            if (MODE == STENCIL_RECORD_KP) kp[g][j] = 0.f;
                        }
                    }
            }
#pragma unroll
            for (int g = 0; g < NG; g++)
#pragma unroll
                for (int j = 0; j < O; j++) {
                    if (SPONGE) out[g][j] = sv[g][j] * out[g][j];
                    if (!xall && xb + j >= nx) out[g][j] = 0.f;
                }
#pragma unroll
            for (int g = 0; g < NG; g++) {
                if (!row_ok[g]) continue;
                float *dg = dst + g * group_stride;
                if (MODE != STENCIL_PLAIN) {
                    // side buffers: same device layout as the levels (padding columns hold zeros:
                    // K p' is 0 there and the gradient keeps its value)
                    const int64_t so = dg - a_prev;
                    if (MODE == STENCIL_GRADIENT)
#pragma unroll
                        for (int j = 0; j < O; j++) kp[g][j] = fmaf(c[g][j], kpv[g][j], grv[g][j]);
                    store_o_lim<O>((MODE == STENCIL_GRADIENT ? a_grad : a_kp) + so, kp[g], (int)nxp - xb);
                }
                if constexpr (O == 4) {
                    if (xb + 4 <= nxp)
                        *reinterpret_cast<float4 *>(dg) = make_float4(out[g][0], out[g][1], out[g][2], out[g][3]);
                } else if constexpr (O == 2) {
                    if (xb + 2 <= nxp) *reinterpret_cast<float2 *>(dg) = make_float2(out[g][0], out[g][1]);
                } else {
#pragma unroll
                    for (int j = 0; j < O; j++)
                        if (xb + j < nxp) dg[j] = out[g][j];
                }
            }
        }
        aborted = __syncthreads_or(!ok) != 0;
        rs = rs + 1 == R ? 0 : rs + 1;
        if (++ws == R) { ws = 0; wph ^= 1; }
        if (++as == AUX) { as = 0; aph ^= 1; }
        ly = ly + 1 == O ? 0 : ly + 1;
    }

    if (aborted) {
        // leave no copy in flight into this CTA's shared memory: bounded drain of every barrier
        if (threadIdx.x == 0)
            for (int i = 0; i < R + AUX; i++) {
                bar_wait(bars + i, 0, kWaitLimitNs / 8);
                bar_wait(bars + i, 1, kWaitLimitNs / 8);
            }
        return;
    }
    if (a.nrec > 0) {
        const int cta = bx + t.grid[0] * (bz + t.grid[1] * chunk);  // tile and chunk
        const int r0 = a.rec_off[cta], r1 = a.rec_off[cta + 1];
        if (r0 < r1) {  // uniform over the CTA; its new values are visible after the last barrier
            const int step = a.ctr[1];
            const float *lvl = a.prev + (MULTI ? (int64_t)shot * t.shot_stride : 0);
            for (int r = r0 + (int)threadIdx.x; r < r1; r += GROUP ? (int)blockDim.x : C::THREADS) {
                const int j = a.rec_idx[r];
                // traces [step][receiver][shot]
                const int64_t k = (int64_t)step * a.nrec + a.rec_perm[j];
                a.traces[MULTI ? k * t.nshot + shot : k] = lvl[a.rec_node[j]];
            }
        }
    }
}


using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encoder()
{
    static EncodeTiled fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void *p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
    }
    return fn;
}

// Tensor map of a float buffer seen as (d0, d1, d2) row-major (d0 fastest) with box (b0, b1, 1).
bool encode_map_3d(CUtensorMap &m, const float *base, int64_t d0, int64_t d1, int64_t d2, int b0, int b1)
{
    EncodeTiled enc = encoder();
    if (!enc) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)d0, (cuuint64_t)d1, (cuuint64_t)d2};
    const cuuint64_t strides[2] = {(cuuint64_t)d0 * 4, (cuuint64_t)(d0 * d1) * 4};
    const cuuint32_t box[3] = {(cuuint32_t)b0, (cuuint32_t)b1, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return enc(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Fill this translation unit's coefficient tables (orders 1..kMaxOrder).
cudaError_t upload_stencil_constants()
{
    std::vector<float> all(kMaxOrder * kTMax, 0.f), wa(kMaxOrder * kMaxOrder, 0.f);
    for (int o = 1; o <= kMaxOrder; o++) {
        Gll g;
        gll_tables(o, g);
        float *T = all.data() + (o - 1) * kTMax;
        stencil_table(g, T);
        // diagonal entry: minus the sum of the row's float coefficients, rounded once, so that
        // the float row sums to zero up to that rounding (used by the direct form)
        for (int l = 0; l < o; l++) {
            double sum = 0;
            for (int d = -o; d <= o; d++)
                if (d != 0) sum += T[l * (2 * o + 1) + d + o];
            T[l * (2 * o + 1) + o] = (float)-sum;
        }
        for (int l = 0; l < o; l++) wa[(o - 1) * kMaxOrder + l] = (float)(l == 0 ? g.w[0] + g.w[o] : g.w[l]);
    }
    cudaError_t e;
    if ((e = cudaMemcpyToSymbol(c_T, all.data(), all.size() * sizeof(float))) != cudaSuccess) return e;
    std::vector<float2> all2(all.size());
    for (size_t i = 0; i < all.size(); i++) all2[i] = make_float2(all[i], all[i]);
    if ((e = cudaMemcpyToSymbol(c_T2, all2.data(), all2.size() * sizeof(float2))) != cudaSuccess) return e;
    return cudaMemcpyToSymbol(c_wa, wa.data(), wa.size() * sizeof(float));
}

}  // namespace

}  // namespace semgb
