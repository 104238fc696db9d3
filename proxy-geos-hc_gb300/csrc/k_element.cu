// k_element.cu -- element-by-element stiffness product of the SEM step on GB300.
//
// Replaces the element loop of SEMsolver::computeOneStep (SEMsolver.cpp:46-82) and its per-element
// computeMassMatrixAndStiffnessVector (SEMQkGLIntegrals.hpp:206-565).  The reference rebuilds the
// Jacobian, the mass and a dense (o+1)^3-wide stiffness row per node for every element every step
// (O(n_pe^2) per element).  Here the mass is precomputed once (launch_mass) and K_e.p is
// sum-factorised: for each reference direction d, along the 1-D lines ("pencils") of the element,
//     y_d(i) = g_d * W(pencil) * sum_{m != i} S(i, m) * (p_m - p_i)
// with S the element's 1-D stiffness (S(i, m) = sum_l w_l phi_i'(xi_l) phi_m'(xi_l), the product
// of the reference's derivative contraction and its transpose, tabulated once in double), which
// is O(n_pe*(o+1)) per element.  The difference form gives exactly zero on a constant field (the
// float-rounded rows of S do not sum exactly to zero), and as S is symmetric and
// p_m - p_i = -(p_i - p_m) exactly, each pair's difference is formed once.
//
// CTA shape: TE elements x (o+1)^2 pencils, thread = (pencil, element); TE = 32 (one element per
// lane, one pencil per warp) for orders 1-4 and 16 for order 5 (36 pencils would exceed 1024
// threads).  All lanes of a warp work on the same local pencil of different elements, so
// coefficient indices are warp-uniform and shared-memory accesses are unit-stride.  Phases:
//   A  the connectivity rows of the tile two ahead (contiguous in HBM) -> shared by asynchronous
//      copies (cp.async, no register staging), three row buffers in rotation
//   B  gather p through the rows: each thread loads its x-pencil (registers + shared copy)
//   C  x-direction contraction in registers
//   D  z-direction (xi2) pencils from shared, result -> s_y
//   E  y-direction (xi3) pencils from shared, result -> s_w (no barrier after D: both only read s_p)
//   F  y = yx + yz + yy scattered with red.global.add.f32 through the connectivity
#include <cuda_runtime.h>

#include <algorithm>

#include "kernels.h"

namespace semgb {

int coef_table_size(int order) { return 3 * (order + 1) * (order + 1); }

namespace {

// Elements per CTA at orders 1-4 (compile-time knob for sweeps: 32 = one element per lane and
// one pencil per warp; 16 = two pencils per warp, half-size CTAs, twice as many per SM).
#ifndef SEM_ELEMENT_TE
#define SEM_ELEMENT_TE 32
#endif

template <int O, bool REF = false>
struct ElemCfg {
    static constexpr int O1 = O + 1, NP = O1 * O1, NPE = O1 * O1 * O1;
    static constexpr int TE = O <= 4 ? SEM_ELEMENT_TE : 16;  // elements per CTA
    static constexpr int CS = NPE | 1;  // odd row stride: lanes hit distinct banks
    static constexpr int THREADS = TE * NP;
    static constexpr int MINB = (O == 1 ? 8 : O == 2 ? 5 : O == 3 ? 3 : 2) * (O <= 4 ? 32 / SEM_ELEMENT_TE : 1);
    static constexpr int TAB = REF ? 3 * NPE * O1 : 3 * NP;  // coefficient floats in shared memory
    static constexpr int NBUF = 3;      // connectivity row buffers: this tile, the next two
    static constexpr size_t SMEM = sizeof(int) * NBUF * TE * CS + sizeof(float) * NPE * TE * 3 + sizeof(float) * TAB;
};

// Asynchronous global -> shared copies (completion tracked per thread in commit groups).
__device__ __forceinline__ uint32_t sh_addr(const void *p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }
__device__ __forceinline__ void cp_async4(void *dst, const void *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sh_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async16(void *dst, const void *src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sh_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// wait until none of this thread's copies is in flight
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
// wait until at most one group (the most recent) of this thread is still in flight
__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// One direction of the element operator along one pencil: out = base * S p in difference form,
// base = g_d * w_a * w_b of the pencil.
template <int O>
__device__ __forceinline__ void pencil_apply(const ElementArgs &a, const float (&p)[O + 1],
                                             float base, float (&out)[O + 1])
{
    float acc[O + 1];
#pragma unroll
    for (int i = 0; i <= O; i++) acc[i] = 0.f;
#pragma unroll
    for (int i = 0; i <= O; i++)
#pragma unroll
        for (int m = i + 1; m <= O; m++) {
            const float d = p[m] - p[i];
            acc[i] = fmaf(a.S[i][m], d, acc[i]);
            acc[m] = fmaf(-a.S[m][i], d, acc[m]);
        }
#pragma unroll
    for (int i = 0; i <= O; i++) out[i] = base * acc[i];
}

// REF: the reference's rows in its order (SEM_ROUNDING_REFERENCE).  CHECKED: caller-supplied
// connectivity, every index checked against [0, a.n_check) before it is used.
template <int O, bool REF, bool CHECKED = false>
__global__ void __launch_bounds__(ElemCfg<O>::THREADS, ElemCfg<O>::MINB)
    k_element(const ElementArgs a)
{
    using C = ElemCfg<O, REF>;
    constexpr int O1 = C::O1, NP = C::NP, NPE = C::NPE, CS = C::CS, TE = C::TE;
    extern __shared__ __align__(16) unsigned char smem[];
    int *s_conn = reinterpret_cast<int *>(smem);  // [NBUF][TE * CS]: this tile's rows and the next two tiles'
    float *s_p = reinterpret_cast<float *>(s_conn + C::NBUF * TE * CS);
    float *s_y = s_p + NPE * TE;  // z-direction results
    float *s_w = s_y + NPE * TE;  // y-direction results
    float *s_tab = s_w + NPE * TE;

    // "lane" = element of the tile, "warp" = pencil (a hardware warp when TE == 32)
    const int tid = threadIdx.x, lane = tid % TE, warp = tid / TE;
    const int64_t ntiles = (a.n_elem + TE - 1) / TE;
    int64_t t = blockIdx.x;
    if (t >= ntiles) return;

    // connectivity rows of tile u (contiguous in HBM) into buffer b by asynchronous copies, then
    // one commit group (also when u is past the end, so that every thread counts groups alike).
    // Where the shared rows are unpadded (CS == NPE) and the array is 16-byte aligned (a caller's
    // array need not be) the block is copied 16 bytes at a time: a tile's block then starts at a
    // multiple of TE * NPE * 4 bytes, a multiple of 16, and so does its shared buffer.
    auto load_conn = [&](int64_t u, int b) {
        if (u < ntiles) {
            const int64_t e0 = u * TE;
            const int ne = (int)min((int64_t)TE, a.n_elem - e0);
            const int32_t *cg = a.conn + e0 * NPE;
            int *dst = s_conn + b * TE * CS;
            int q0 = 0;
            if constexpr (CS == NPE && (TE * NPE) % 4 == 0) {
                if ((reinterpret_cast<uintptr_t>(a.conn) & 15) == 0) {
                    q0 = ne * NPE / 4 * 4;
                    for (int c = tid; c < q0 / 4; c += C::THREADS) cp_async16(dst + 4 * c, cg + 4 * c);
                }
            }
            for (int q = q0 + tid; q < ne * NPE; q += C::THREADS) {
                const int e = q / NPE;
                cp_async4(dst + e * CS + (q - e * NPE), cg + q);
            }
        }
        cp_async_commit();
    };
    // the thread's x-pencil (local j, k fixed) of tile u through buffer b
    const int jx = warp % O1, kx = warp / O1;
    auto gather = [&](int64_t u, int b, float (&v)[O1]) {
        const bool act = lane < (int)min((int64_t)TE, a.n_elem - u * TE);
        const int *cr = s_conn + b * TE * CS + lane * CS;
#pragma unroll
        for (int i = 0; i < O1; i++) {
            const int g = cr[i + O1 * jx + NP * kx];
            v[i] = act && (!CHECKED || (g >= 0 && g < a.n_check)) ? __ldg(a.p + g) : 0.f;
        }
    };

    // A: coefficient table, the first two tiles' rows, and the first tile's pencil values
    for (int q = tid; q < C::TAB; q += C::THREADS) s_tab[q] = __ldg((REF ? a.rtab : a.tab) + q);
    load_conn(t, 0);
    load_conn(t + gridDim.x, 1);
    cp_async_wait_one();
    __syncthreads();
    float pn[O1];
    gather(t, 0, pn);

    // Persistent loop: while a tile runs its z- and y-directions and its scatter, the next
    // tile's connectivity rows are in shared memory and its pencil values are in flight, and the
    // rows of the tile after it are being copied.  Buffer b holds this tile's rows, bn the
    // next tile's, bf the one after (last read by the previous tile's scatter).  Two barriers
    // per tile: (1) after the pencil values are stored -- every warp has also finished the
    // previous tile's scatter, so bf and the z/y result buffers are free, and the copies of the
    // next tile's rows have landed; (2) after the z- and y-directions.  The pencil values of the
    // next tile are stored after barrier 2 of this one, when no warp reads them any more.  The
    // reference-rounding form reads the pencil values after barrier 1 and keeps a third barrier
    // at the end of the tile, with the copies issued before barrier 1.
    for (int b = 0; t < ntiles; t += gridDim.x, b = b == 2 ? 0 : b + 1) {
        const int64_t tn = t + gridDim.x;
        const int bn = b == 2 ? 0 : b + 1, bf = bn == 2 ? 0 : bn + 1;
        const bool act = lane < (int)min((int64_t)TE, a.n_elem - t * TE);
        // B: this tile's pencil values into shared memory; copies of the rows two tiles ahead
        float px[O1];
#pragma unroll
        for (int i = 0; i < O1; i++) {
            px[i] = pn[i];
            s_p[(i + O1 * jx + NP * kx) * TE + lane] = px[i];
        }
        if constexpr (REF) load_conn(tn + gridDim.x, bf);
        float yx[O1];
        if constexpr (REF) {
            cp_async_wait_one();  // the next tile's rows (all but the copies just issued)
            __syncthreads();
            if (tn < ntiles) gather(tn, bn, pn);
            // C': K_e p at the thread's nodes as the reference forms it (SEMQkGLIntegrals.hpp:
            // 508-513): Y = sum over the row in increasing local index j of R[j] p[j], multiply and
            // add rounded separately.  The row's non-zero entries lie on the node's three lines;
            // in increasing j: the y-line below the node, the z-line below it, the x-line, the
            // z-line above, the y-line above.
#pragma unroll
            for (int i1 = 0; i1 < O1; i1++) {
                const int node = i1 + O1 * jx + NP * kx;
                const float *rx = s_tab + (0 * NPE + node) * O1;
                const float *rz = s_tab + (1 * NPE + node) * O1;
                const float *ry = s_tab + (2 * NPE + node) * O1;
                float acc = 0.f;
                for (int m = 0; m < kx; m++)
                    acc = __fadd_rn(acc, __fmul_rn(ry[m], s_p[(i1 + O1 * jx + NP * m) * TE + lane]));
                for (int m = 0; m < jx; m++)
                    acc = __fadd_rn(acc, __fmul_rn(rz[m], s_p[(i1 + O1 * m + NP * kx) * TE + lane]));
#pragma unroll
                for (int m = 0; m < O1; m++) acc = __fadd_rn(acc, __fmul_rn(rx[m], px[m]));
                for (int m = jx + 1; m < O1; m++)
                    acc = __fadd_rn(acc, __fmul_rn(rz[m], s_p[(i1 + O1 * m + NP * kx) * TE + lane]));
                for (int m = kx + 1; m < O1; m++)
                    acc = __fadd_rn(acc, __fmul_rn(ry[m], s_p[(i1 + O1 * jx + NP * m) * TE + lane]));
                yx[i1] = acc;
            }
        } else {
            // C: x-direction in registers
            pencil_apply<O>(a, px, s_tab[0 * NP + jx + O1 * kx], yx);
            cp_async_wait_all();  // the next tile's rows
            __syncthreads();
            load_conn(tn + gridDim.x, bf);
            if (tn < ntiles) gather(tn, bn, pn);
            // D: z-direction (local index j varies) into s_y, and E: y-direction (local index k
            // varies) into s_w; both only read s_p, so no barrier between them
            {
                const int i = warp % O1, k = warp / O1;
                float pz[O1], yz[O1];
#pragma unroll
                for (int m = 0; m < O1; m++) pz[m] = s_p[(i + O1 * m + NP * k) * TE + lane];
                pencil_apply<O>(a, pz, s_tab[1 * NP + i + O1 * k], yz);
#pragma unroll
                for (int m = 0; m < O1; m++) s_y[(i + O1 * m + NP * k) * TE + lane] = yz[m];
            }
            {
                const int i = warp % O1, j = warp / O1;
                float py[O1], yy[O1];
#pragma unroll
                for (int n = 0; n < O1; n++) py[n] = s_p[(i + O1 * j + NP * n) * TE + lane];
                pencil_apply<O>(a, py, s_tab[2 * NP + i + O1 * j], yy);
#pragma unroll
                for (int n = 0; n < O1; n++) s_w[(i + O1 * j + NP * n) * TE + lane] = yy[n];
            }
            __syncthreads();
        }
        // F: scatter through the connectivity.  The tile's elements are consecutive (one per
        // lane); where the next lane's element shares this element's right x-face (same global
        // nodes), its left-face value is added here with a shuffle and it skips that atomic.
        {
            const int *cr = s_conn + b * TE * CS + lane * CS;
            float v[O1];
#pragma unroll
            for (int i = 0; i < O1; i++) {
                const int node = i + O1 * jx + NP * kx;
                if constexpr (REF) v[i] = act ? yx[i] : 0.f;
                else v[i] = act ? yx[i] + s_y[node * TE + lane] + s_w[node * TE + lane] : 0.f;
            }
            const int g_left = act ? cr[0 + O1 * jx + NP * kx] : -1;
            const int g_right = act ? cr[O + O1 * jx + NP * kx] : -2;
            const float v_next = __shfl_down_sync(0xffffffffu, v[0], 1, TE);
            const int g_next = __shfl_down_sync(0xffffffffu, g_left, 1, TE);
            const int g_prev = __shfl_up_sync(0xffffffffu, g_right, 1, TE);
            const bool merge_next = lane + 1 < TE && g_next == g_right;
            const bool merged_into_prev = lane > 0 && g_prev == g_left;
            if (merge_next) v[O] += v_next;
            if (act) {
#pragma unroll
                for (int i = 0; i < O1; i++) {
                    if (i == 0 && merged_into_prev) continue;
                    const int g = cr[i + O1 * jx + NP * kx];
                    if (CHECKED && !(g >= 0 && g < a.n_check)) continue;
                    atomicAdd(a.y + g, v[i]);  // result unused: compiles to RED
                }
            }
        }
        if constexpr (REF) __syncthreads();  // s_p and this tile's rows are reused by the next iteration
    }
    cp_async_wait_all();  // no copy left in flight into shared memory
}

template <int O, bool REF, bool CHECKED = false>
cudaError_t launch_element_r(const ElementArgs &a, cudaStream_t s)
{
    using C = ElemCfg<O, REF>;
    if (a.n_elem <= 0) return cudaSuccess;
    const int64_t tiles = (a.n_elem + C::TE - 1) / C::TE;
    // persistent CTAs: as many as are resident at once
    int dev = 0, sms = 152, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_element<O, REF, CHECKED>, C::THREADS, C::SMEM) !=
            cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    const int64_t grid = std::min<int64_t>(tiles, (int64_t)sms * per_sm);
    k_element<O, REF, CHECKED><<<(unsigned)grid, C::THREADS, C::SMEM, s>>>(a);
    return cudaGetLastError();
}

template <int O>
cudaError_t launch_element_t(const ElementArgs &a, cudaStream_t s)
{
    if (a.n_check > 0) return a.rtab ? cudaErrorInvalidValue : launch_element_r<O, false, true>(a, s);
    return a.rtab ? launch_element_r<O, true>(a, s) : launch_element_r<O, false>(a, s);
}

template <int O, bool REF, bool CHECKED>
cudaError_t setup_one()
{
    return cudaFuncSetAttribute(k_element<O, REF, CHECKED>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)ElemCfg<O, REF>::SMEM);
}

template <int O>
cudaError_t setup_t()
{
    cudaError_t e = setup_one<O, false, false>();
    if (e == cudaSuccess) e = setup_one<O, true, false>();
    if (e == cudaSuccess) e = setup_one<O, false, true>();
    return e;
}

}  // namespace

cudaError_t element_kernel_setup()
{
    cudaError_t e;
    if ((e = setup_t<1>()) != cudaSuccess) return e;
    if ((e = setup_t<2>()) != cudaSuccess) return e;
    if ((e = setup_t<3>()) != cudaSuccess) return e;
    if ((e = setup_t<4>()) != cudaSuccess) return e;
    return setup_t<5>();
}

cudaError_t launch_element(int order, const ElementArgs &a, cudaStream_t s)
{
    switch (order) {
    case 1: return launch_element_t<1>(a, s);
    case 2: return launch_element_t<2>(a, s);
    case 3: return launch_element_t<3>(a, s);
    case 4: return launch_element_t<4>(a, s);
    case 5: return launch_element_t<5>(a, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace semgb
