// k_mlp.cu -- kernels of the boundary network (mlp.h): BF16 tensor-core forward (mma.sync
// m16n8k16, FP32 accumulators), the training pass (forward on the tensor cores, backward and
// parameter gradients in FP32), Adam, and the boundary-strip gather / correction.
//
// Tile: 128 rows (samples or strip nodes) per CTA, 4 warps of 32 rows.  Shared memory holds the
// BF16 weights as [out][in] rows (the MMA's column-major B operand) and the BF16 inputs and
// hidden activations as row-major [row][in] (the row-major A operand); row strides are padded by
// 8 elements so that the fragment loads of a warp hit 32 different banks.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>
#include <cstddef>

#include "mlp.h"
#include "tma.cuh"

namespace semgb {

namespace {

// Fragment loads of the register-resident inference forward (compile-time knob: 1 = ldmatrix,
// 0 = one 32-bit shared load per fragment register; the same fragments either way, so the same
// bits).  ldmatrix: a quarter of the load instructions, 162 registers, no spill.
#ifndef SEM_MLP_LDSM
#define SEM_MLP_LDSM 1
#endif
// Face kernel staging (compile-time knob: 1 = the next tile's patch loads issued into registers
// before the current tile's network runs, stored to shared memory after it; 0 = load and store
// each tile's patch before its features).  The same values either way.
#ifndef SEM_MLP_FACE_PIPE
#define SEM_MLP_FACE_PIPE 1
#endif

constexpr int H = kMlpHidden;
constexpr int KP1 = kMlpInPad + 8;  // row stride (bf16) of X and W1
constexpr int KP2 = H + 8;          // row stride (bf16) of H1 and W2
constexpr int T = kMlpTile;

__device__ __forceinline__ uint16_t f2bf(float x)
{
    const __nv_bfloat16 b = __float2bfloat16_rn(x);
    return *reinterpret_cast<const uint16_t *>(&b);
}

__device__ __forceinline__ float bf2f(uint16_t u)
{
    __nv_bfloat16 b;
    *reinterpret_cast<uint16_t *>(&b) = u;
    return __bfloat162float(b);
}

// two floats to BF16 (round to nearest even, as f2bf) in one conversion: lo in the low half
__device__ __forceinline__ uint32_t pack_bf2(float lo, float hi)
{
    const __nv_bfloat162 b = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&b);
}

// GELU in the tanh form of Hendrycks & Gimpel (2016), GELU(z) = z/2 (1 + tanh(u)),
// u = sqrt(2/pi) (z + 0.044715 z^3), and its derivative; tanh from the hardware approximation
// (tanh.approx.f32, relative error about 2^-11, below the BF16 rounding of the activations)
__device__ __forceinline__ float tanh_hw(float x)
{
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
constexpr float kGeluC = 0.7978845608028654f;  // sqrt(2/pi)
constexpr float kGeluCA = 0.7978845608028654f * 0.044715f;
// u = z (c + c a z^2): two multiplies and one fma
__device__ __forceinline__ float gelu_u(float z) { return z * fmaf(kGeluCA, z * z, kGeluC); }
__device__ __forceinline__ float gelu(float z)
{
    const float t = tanh_hw(gelu_u(z));
    const float h = 0.5f * z;
    return fmaf(h, t, h);
}
// gelu of two values with packed f32x2 arithmetic: the same operations in the same order as gelu,
// each half rounded as the scalar instruction would round it
__device__ __forceinline__ float2 gelu2(float2 z)
{
    const float2 w = fma2(make_float2(kGeluCA, kGeluCA), mul2(z, z), make_float2(kGeluC, kGeluC));
    const float2 u = mul2(z, w);
    const float2 t = make_float2(tanh_hw(u.x), tanh_hw(u.y));
    const float2 h = mul2(make_float2(0.5f, 0.5f), z);
    return fma2(h, t, h);
}
__device__ __forceinline__ float gelu_d(float z)
{
    // d/dz [z/2 (1 + tanh u)] = (1 + t)/2 + z/2 (1 - t^2) (c + 3 c a z^2)
    const float t = tanh_hw(gelu_u(z));
    return fmaf(0.5f, t, 0.5f) + (0.5f * z) * fmaf(-t, t, 1.f) * fmaf(3.f * kGeluCA, z * z, kGeluC);
}

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2])
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

#if SEM_MLP_LDSM
// 8x8 b16 matrices from shared memory (fragment layout of the mma operands): x4 takes row
// addresses from lanes 0-31 (matrix lane/8), x2 from lanes 0-15.
__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const void *p)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(static_cast<uint32_t>(__cvta_generic_to_shared(p))));
}
__device__ __forceinline__ void ldsm_x2(uint32_t (&r)[2], const void *p)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0, %1}, [%2];"
                 : "=r"(r[0]), "=r"(r[1])
                 : "r"(static_cast<uint32_t>(__cvta_generic_to_shared(p))));
}
#endif

struct NetSmem {
    uint16_t w1[H * KP1];
    uint16_t w2[H * KP2];
    float b1[H], b2[H], w3[H], b3;
};

__device__ void load_net(NetSmem &s, const MlpDev &net)
{
    // 16-byte chunks: W1 rows are 96 bf16 (12 chunks), W2 rows 64 (8 chunks); shared rows are
    // padded to 104 and 72 elements, still 16-byte aligned
    constexpr int C1 = kMlpInPad / 8, C2 = H / 8;
    static_assert((KP1 * 2) % 16 == 0 && (KP2 * 2) % 16 == 0, "16-byte aligned shared rows");
#pragma unroll 4
    for (int i = threadIdx.x; i < H * C1; i += blockDim.x) {
        const int nn = i / C1, j = i - nn * C1;
        *reinterpret_cast<uint4 *>(s.w1 + nn * KP1 + j * 8) = __ldg(reinterpret_cast<const uint4 *>(net.w1) + i);
    }
#pragma unroll 4
    for (int i = threadIdx.x; i < H * C2; i += blockDim.x) {
        const int nn = i / C2, j = i - nn * C2;
        *reinterpret_cast<uint4 *>(s.w2 + nn * KP2 + j * 8) = __ldg(reinterpret_cast<const uint4 *>(net.w2) + i);
    }
    for (int i = threadIdx.x; i < H; i += blockDim.x) {
        s.b1[i] = net.b1[i];
        s.b2[i] = net.b2[i];
        s.w3[i] = net.w3[i];
    }
    if (threadIdx.x == 0) s.b3 = net.b3[0];
}

// Forward of the warp's 32 rows (tile rows wr..wr+31): xs [T][KP1] bf16 in, h1 [T][KP2] bf16
// written, returns y for rows wr + mt*16 + g (+8) in yv[mt][0/1] (valid on every lane of a quad).
// With z1/z2 non-null the pre-activations are kept (FP32 [T][H]).
__device__ void forward_rows(const NetSmem &s, const uint16_t *xs, uint16_t *h1, float *z1, float *z2, int wr,
                             float (&yv)[2][2])
{
    const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
    float acc[2][8][4];
#pragma unroll
    for (int mt = 0; mt < 2; mt++)
#pragma unroll
        for (int nt = 0; nt < 8; nt++)
#pragma unroll
            for (int j = 0; j < 4; j++) acc[mt][nt][j] = 0.f;
#pragma unroll
    for (int ks = 0; ks < kMlpInPad / 16; ks++) {
        const int k0 = ks * 16 + q * 2;
        uint32_t a[2][4];
#pragma unroll
        for (int mt = 0; mt < 2; mt++) {
            const int r = wr + mt * 16 + g;
            a[mt][0] = *reinterpret_cast<const uint32_t *>(xs + r * KP1 + k0);
            a[mt][1] = *reinterpret_cast<const uint32_t *>(xs + (r + 8) * KP1 + k0);
            a[mt][2] = *reinterpret_cast<const uint32_t *>(xs + r * KP1 + k0 + 8);
            a[mt][3] = *reinterpret_cast<const uint32_t *>(xs + (r + 8) * KP1 + k0 + 8);
        }
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
            const int n = nt * 8 + g;
            uint32_t b[2];
            b[0] = *reinterpret_cast<const uint32_t *>(s.w1 + n * KP1 + k0);
            b[1] = *reinterpret_cast<const uint32_t *>(s.w1 + n * KP1 + k0 + 8);
            mma16816(acc[0][nt], a[0], b);
            mma16816(acc[1][nt], a[1], b);
        }
    }
    // layer-1 epilogue: bias, GELU, BF16 into h1 (the warp's own rows)
#pragma unroll
    for (int mt = 0; mt < 2; mt++)
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
            const int c = nt * 8 + q * 2;
#pragma unroll
            for (int hrow = 0; hrow < 2; hrow++) {
                const int r = wr + mt * 16 + g + hrow * 8;
                const float za = acc[mt][nt][hrow * 2] + s.b1[c], zb = acc[mt][nt][hrow * 2 + 1] + s.b1[c + 1];
                if (z1) {
                    z1[r * H + c] = za;
                    z1[r * H + c + 1] = zb;
                }
                *reinterpret_cast<uint32_t *>(h1 + r * KP2 + c) = pack_bf2(gelu(za), gelu(zb));
                acc[mt][nt][hrow * 2] = 0.f;
                acc[mt][nt][hrow * 2 + 1] = 0.f;
            }
        }
    __syncwarp();
#pragma unroll
    for (int ks = 0; ks < H / 16; ks++) {
        const int k0 = ks * 16 + q * 2;
        uint32_t a[2][4];
#pragma unroll
        for (int mt = 0; mt < 2; mt++) {
            const int r = wr + mt * 16 + g;
            a[mt][0] = *reinterpret_cast<const uint32_t *>(h1 + r * KP2 + k0);
            a[mt][1] = *reinterpret_cast<const uint32_t *>(h1 + (r + 8) * KP2 + k0);
            a[mt][2] = *reinterpret_cast<const uint32_t *>(h1 + r * KP2 + k0 + 8);
            a[mt][3] = *reinterpret_cast<const uint32_t *>(h1 + (r + 8) * KP2 + k0 + 8);
        }
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
            const int n = nt * 8 + g;
            uint32_t b[2];
            b[0] = *reinterpret_cast<const uint32_t *>(s.w2 + n * KP2 + k0);
            b[1] = *reinterpret_cast<const uint32_t *>(s.w2 + n * KP2 + k0 + 8);
            mma16816(acc[0][nt], a[0], b);
            mma16816(acc[1][nt], a[1], b);
        }
    }
    // layer-2 epilogue and the output layer: y = b3 + sum_c w3[c] GELU(z2[c])
#pragma unroll
    for (int mt = 0; mt < 2; mt++)
#pragma unroll
        for (int hrow = 0; hrow < 2; hrow++) {
            const int r = wr + mt * 16 + g + hrow * 8;
            float part = 0.f;
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                const int c = nt * 8 + q * 2;
                const float za = acc[mt][nt][hrow * 2] + s.b2[c], zb = acc[mt][nt][hrow * 2 + 1] + s.b2[c + 1];
                if (z2) {
                    z2[r * H + c] = za;
                    z2[r * H + c + 1] = zb;
                }
                part = fmaf(s.w3[c], gelu(za), part);
                part = fmaf(s.w3[c + 1], gelu(zb), part);
            }
            part += __shfl_xor_sync(0xffffffffu, part, 1);
            part += __shfl_xor_sync(0xffffffffu, part, 2);
            yv[mt][hrow] = part + s.b3;
        }
}

// As forward_rows for inference (no saved activations), with the hidden layer kept in registers:
// the m16n8 accumulator fragments of layer-1 columns 16k..16k+15 (n-tiles 2k and 2k+1) are, after
// bias, GELU and BF16 rounding, exactly the m16n8k16 A fragments of layer 2's k-step k, so no
// shared-memory copy of the hidden activations is made.  Same roundings and summation order as
// forward_rows, which the training and the adjoint use: a network must be trained and
// differentiated as it runs, and the training of the learned boundary, a feedback loop over whole
// runs, follows last-bit differences far (biases entered as the first MMA's accumulator, which
// round the pre-activations differently, moved the reflected energy of the network trained with
// the gradient line search from 0.0043 to 0.011-0.045).
__device__ void forward_rows_regs(const NetSmem &s, const uint16_t *xs, int wr, float (&yv)[2][2])
{
    const int lane = threadIdx.x & 31, q = lane & 3;
#if SEM_MLP_LDSM
    // ldmatrix row addresses: A (rows of xs) {rows 0-7, 8-15} x {cols 0-7, 8-15}; B (rows n of
    // W) {cols 0-7, 8-15} of one n-tile
    const int a_row = (lane & 7) + ((lane >> 3) & 1) * 8, a_col = (lane >> 4) * 8;
    const int b_row = lane & 7, b_col = ((lane >> 3) & 1) * 8;
#else
    const int g = lane >> 2;
#endif
    float acc[2][8][4];
#pragma unroll
    for (int mt = 0; mt < 2; mt++)
#pragma unroll
        for (int nt = 0; nt < 8; nt++)
#pragma unroll
            for (int j = 0; j < 4; j++) acc[mt][nt][j] = 0.f;
#pragma unroll
    for (int ks = 0; ks < kMlpInPad / 16; ks++) {
        uint32_t a[2][4];
#if !SEM_MLP_LDSM
        const int k0 = ks * 16 + q * 2;
#endif
#pragma unroll
        for (int mt = 0; mt < 2; mt++) {
#if SEM_MLP_LDSM
            ldsm_x4(a[mt], xs + (wr + mt * 16 + a_row) * KP1 + ks * 16 + a_col);
#else
            const int r = wr + mt * 16 + g;
            a[mt][0] = *reinterpret_cast<const uint32_t *>(xs + r * KP1 + k0);
            a[mt][1] = *reinterpret_cast<const uint32_t *>(xs + (r + 8) * KP1 + k0);
            a[mt][2] = *reinterpret_cast<const uint32_t *>(xs + r * KP1 + k0 + 8);
            a[mt][3] = *reinterpret_cast<const uint32_t *>(xs + (r + 8) * KP1 + k0 + 8);
#endif
        }
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
#if SEM_MLP_LDSM
            uint32_t b[2];
            ldsm_x2(b, s.w1 + (nt * 8 + b_row) * KP1 + ks * 16 + b_col);
#else
            const int n = nt * 8 + g;
            const uint32_t b[2] = {*reinterpret_cast<const uint32_t *>(s.w1 + n * KP1 + k0),
                                   *reinterpret_cast<const uint32_t *>(s.w1 + n * KP1 + k0 + 8)};
#endif
            mma16816(acc[0][nt], a[0], b);
            mma16816(acc[1][nt], a[1], b);
        }
    }
    // layer-1 epilogue into layer-2 A fragments: h[mt][ks] = {row g cols 16ks+2q.., row g+8 the
    // same, row g cols 16ks+8+2q.., row g+8 the same}
    uint32_t h[2][H / 16][4];
#pragma unroll
    for (int mt = 0; mt < 2; mt++)
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
            const int c = nt * 8 + q * 2;
#pragma unroll
            for (int hrow = 0; hrow < 2; hrow++) {
                const float2 z = add2(make_float2(acc[mt][nt][hrow * 2], acc[mt][nt][hrow * 2 + 1]),
                                      *reinterpret_cast<const float2 *>(s.b1 + c));
                const float2 gz = gelu2(z);
                h[mt][nt >> 1][(nt & 1) * 2 + hrow] = pack_bf2(gz.x, gz.y);
                acc[mt][nt][hrow * 2] = 0.f;
                acc[mt][nt][hrow * 2 + 1] = 0.f;
            }
        }
#pragma unroll
    for (int ks = 0; ks < H / 16; ks++) {
#if !SEM_MLP_LDSM
        const int k0 = ks * 16 + q * 2;
#endif
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
#if SEM_MLP_LDSM
            uint32_t b[2];
            ldsm_x2(b, s.w2 + (nt * 8 + b_row) * KP2 + ks * 16 + b_col);
#else
            const int n = nt * 8 + g;
            const uint32_t b[2] = {*reinterpret_cast<const uint32_t *>(s.w2 + n * KP2 + k0),
                                   *reinterpret_cast<const uint32_t *>(s.w2 + n * KP2 + k0 + 8)};
#endif
            mma16816(acc[0][nt], h[0][ks], b);
            mma16816(acc[1][nt], h[1][ks], b);
        }
    }
#pragma unroll
    for (int mt = 0; mt < 2; mt++)
#pragma unroll
        for (int hrow = 0; hrow < 2; hrow++) {
            float part = 0.f;
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                const int c = nt * 8 + q * 2;
                const float2 z = add2(make_float2(acc[mt][nt][hrow * 2], acc[mt][nt][hrow * 2 + 1]),
                                      *reinterpret_cast<const float2 *>(s.b2 + c));
                const float2 gz = gelu2(z);
                part = fmaf(s.w3[c], gz.x, part);
                part = fmaf(s.w3[c + 1], gz.y, part);
            }
            part += __shfl_xor_sync(0xffffffffu, part, 1);
            part += __shfl_xor_sync(0xffffffffu, part, 2);
            yv[mt][hrow] = part + s.b3;
        }
}

// stage rows [row0, row0 + T) of x [n][81] (FP32, scaled by 1/scale[i] when scale is given) as
// BF16 [T][KP1] with zero padding
__device__ void stage_x(uint16_t *xs, const float *x, int64_t row0, int64_t n)
{
    for (int i = threadIdx.x; i < T * kMlpInPad; i += blockDim.x) {
        const int r = i / kMlpInPad, k = i - r * kMlpInPad;
        const int64_t row = row0 + r;
        const float v = (row < n && k < kMlpIn) ? x[row * kMlpIn + k] : 0.f;
        xs[r * KP1 + k] = f2bf(v);
    }
}

__global__ void __launch_bounds__(128) k_mlp_forward(const MlpDev net, const float *x, float *y, int64_t n)
{
    extern __shared__ __align__(16) unsigned char smem[];
    NetSmem &s = *reinterpret_cast<NetSmem *>(smem);
    uint16_t *xs = reinterpret_cast<uint16_t *>(smem + sizeof(NetSmem));
    uint16_t *h1 = xs + T * KP1;
    load_net(s, net);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
    for (int64_t row0 = (int64_t)blockIdx.x * T; row0 < n; row0 += (int64_t)gridDim.x * T) {
        __syncthreads();
        stage_x(xs, x, row0, n);
        __syncthreads();
        float yv[2][2];
        forward_rows(s, xs, h1, nullptr, nullptr, w * 32, yv);
        if (q == 0)
#pragma unroll
            for (int mt = 0; mt < 2; mt++)
#pragma unroll
                for (int hrow = 0; hrow < 2; hrow++) {
                    const int64_t row = row0 + w * 32 + mt * 16 + g + hrow * 8;
                    if (row < n) y[row] = yv[mt][hrow];
                }
    }
}

// Training pass: loss and parameter gradients over all n samples, accumulated per CTA in shared
// memory (each gradient entry owned by one thread) and added to the global buffers once.
struct TrainSmem {
    float z1[T * H];
    float z2[T * H];
    float dy[T];
    float g[kMlpParams];
};

// dy_in non-null: the gradient of the output per row is given (dy_in[row]; no loss), otherwise
// dy = 2 (y - t) / n.  dx_out non-null: the gradient with respect to the (BF16-rounded) inputs,
// dx[row][k] = sum_n dZ1[row][n] W1[n][k] (k < 81), is written too.
__global__ void __launch_bounds__(128) k_mlp_train_pass(const MlpDev net, const float *x, const float *t, int64_t n,
                                                        double *part_loss, float *part, const float *dy_in,
                                                        float *dx_out)
{
    extern __shared__ __align__(16) unsigned char smem[];
    NetSmem &s = *reinterpret_cast<NetSmem *>(smem);
    uint16_t *xs = reinterpret_cast<uint16_t *>(smem + sizeof(NetSmem));
    uint16_t *h1 = xs + T * KP1;
    TrainSmem &ts = *reinterpret_cast<TrainSmem *>(h1 + T * KP2);
    load_net(s, net);
    for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) ts.g[i] = 0.f;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
    const int tid = threadIdx.x;
    const float inv_n = 1.f / (float)n;
    double lsum = 0.0;
    for (int64_t row0 = (int64_t)blockIdx.x * T; row0 < n; row0 += (int64_t)gridDim.x * T) {
        __syncthreads();
        stage_x(xs, x, row0, n);
        __syncthreads();
        float yv[2][2];
        forward_rows(s, xs, h1, ts.z1, ts.z2, w * 32, yv);
        if (q == 0)
#pragma unroll
            for (int mt = 0; mt < 2; mt++)
#pragma unroll
                for (int hrow = 0; hrow < 2; hrow++) {
                    const int r = w * 32 + mt * 16 + g + hrow * 8;
                    const int64_t row = row0 + r;
                    float d = 0.f;
                    if (row < n) {
                        if (dy_in) {
                            d = dy_in[row];
                        } else {
                            const float e = yv[mt][hrow] - t[row];
                            lsum += (double)e * e;
                            d = 2.f * e * inv_n;
                        }
                    }
                    ts.dy[r] = d;
                }
        __syncthreads();
        // row pass (thread = row): output layer, dZ2 = dy w3 GELU'(z2) in place of z2
        {
            const int r = tid;
            const float d = ts.dy[r];
            for (int c = 0; c < H; c++) {
                const float z = ts.z2[r * H + c];
                ts.z2[r * H + c] = d * s.w3[c] * gelu_d(z);
            }
        }
        __syncthreads();
        // column sums: db2[c] (thread c < 64) and db3; dw3 needs GELU(z2), which this pass
        // overwrites, so k_mlp_grad_w3 accumulates it from a second forward
        if (tid < H) {
            float a2 = 0.f;
            for (int r = 0; r < T; r++) a2 += ts.z2[r * H + tid];
            ts.g[kOffB2 + tid] += a2;
        } else if (tid == H) {
            float a = 0.f;
            for (int r = 0; r < T; r++) a += ts.dy[r];
            ts.g[kOffB3] += a;
        }
        // dW2[n][k] = sum_r dZ2[r][n] H1[r][k]: 4096 entries, 32 per thread
        for (int e = tid; e < H * H; e += blockDim.x) {
            const int nn = e / H, k = e - nn * H;
            float a = 0.f;
            for (int r = 0; r < T; r++) a = fmaf(ts.z2[r * H + nn], bf2f(h1[r * KP2 + k]), a);
            ts.g[kOffW2 + e] += a;
        }
        __syncthreads();
        // row pass: dZ1[r][k] = GELU'(z1[r][k]) sum_n dZ2[r][n] W2[n][k], in place of z1
        {
            const int r = tid;
            float dh[H];
#pragma unroll
            for (int k = 0; k < H; k++) dh[k] = 0.f;
            for (int nn = 0; nn < H; nn++) {
                const float dz = ts.z2[r * H + nn];
#pragma unroll
                for (int k = 0; k < H; k++) dh[k] = fmaf(dz, bf2f(s.w2[nn * KP2 + k]), dh[k]);
            }
#pragma unroll
            for (int k = 0; k < H; k++) ts.z1[r * H + k] = dh[k] * gelu_d(ts.z1[r * H + k]);
            if (dx_out && row0 + r < n) {
                // input gradient of the row from its own dZ1 (this thread's row only)
                float *dxr = dx_out + (row0 + r) * kMlpIn;
                for (int k = 0; k < kMlpIn; k++) {
                    float a = 0.f;
                    for (int nn = 0; nn < H; nn++) a = fmaf(ts.z1[r * H + nn], bf2f(s.w1[nn * KP1 + k]), a);
                    dxr[k] = a;
                }
            }
        }
        __syncthreads();
        // db1 and dW1[n][k] = sum_r dZ1[r][n] X[r][k] (k < 81)
        if (tid < H) {
            float a = 0.f;
            for (int r = 0; r < T; r++) a += ts.z1[r * H + tid];
            ts.g[kOffB1 + tid] += a;
        }
        for (int e = tid; e < H * kMlpIn; e += blockDim.x) {
            const int nn = e / kMlpIn, k = e - nn * kMlpIn;
            float a = 0.f;
            for (int r = 0; r < T; r++) a = fmaf(ts.z1[r * H + nn], bf2f(xs[r * KP1 + k]), a);
            ts.g[kOffW1 + e] += a;
        }
        __syncthreads();
    }
    __syncthreads();
    // this CTA's partial sums (the W3 range is written by k_mlp_grad_w3)
    float *pg = part + (int64_t)blockIdx.x * kMlpParams;
    for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x)
        if (i < kOffW3 || i >= kOffW3 + H) pg[i] = ts.g[i];
    // loss: quad leaders hold partial sums; warps added in order
    lsum += __shfl_xor_sync(0xffffffffu, lsum, 4);
    lsum += __shfl_xor_sync(0xffffffffu, lsum, 8);
    lsum += __shfl_xor_sync(0xffffffffu, lsum, 16);
    __shared__ double wl[4];
    if (lane == 0) wl[w] = lsum;
    __syncthreads();
    if (threadIdx.x == 0) part_loss[blockIdx.x] = (((wl[0] + wl[1]) + wl[2]) + wl[3]) / (double)n;
}

// grad[i] += sum over CTAs b (in order) of part[b][i]; *loss += sum of part_loss[b] in order
__global__ void k_mlp_reduce(const float *part, const double *part_loss, int nb, float *grad, double *loss)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kMlpParams) {
        float a = 0.f;
        for (int b = 0; b < nb; b++) a += part[(int64_t)b * kMlpParams + i];
        grad[i] += a;
    }
    if (i == 0) {
        double l = 0.0;
        for (int b = 0; b < nb; b++) l += part_loss[b];
        *loss += l;
    }
}

// dw3[c] = sum_r dy[r] GELU(z2[r][c]) needs the forward activations the training pass
// overwrites; this pass recomputes them (forward only) and accumulates dw3.
__global__ void __launch_bounds__(128) k_mlp_grad_w3(const MlpDev net, const float *x, const float *t, int64_t n,
                                                     float *part, const float *dy_in)
{
    extern __shared__ __align__(16) unsigned char smem[];
    NetSmem &s = *reinterpret_cast<NetSmem *>(smem);
    uint16_t *xs = reinterpret_cast<uint16_t *>(smem + sizeof(NetSmem));
    uint16_t *h1 = xs + T * KP1;
    float *z2 = reinterpret_cast<float *>(h1 + T * KP2);
    float *dy = z2 + T * H;
    float *gw3 = dy + T;
    load_net(s, net);
    for (int i = threadIdx.x; i < H; i += blockDim.x) gw3[i] = 0.f;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
    const float inv_n = 1.f / (float)n;
    for (int64_t row0 = (int64_t)blockIdx.x * T; row0 < n; row0 += (int64_t)gridDim.x * T) {
        __syncthreads();
        stage_x(xs, x, row0, n);
        __syncthreads();
        float yv[2][2];
        forward_rows(s, xs, h1, nullptr, z2, w * 32, yv);
        if (q == 0)
#pragma unroll
            for (int mt = 0; mt < 2; mt++)
#pragma unroll
                for (int hrow = 0; hrow < 2; hrow++) {
                    const int r = w * 32 + mt * 16 + g + hrow * 8;
                    const int64_t row = row0 + r;
                    dy[r] = row < n ? (dy_in ? dy_in[row] : 2.f * (yv[mt][hrow] - t[row]) * inv_n) : 0.f;
                }
        __syncthreads();
        if (threadIdx.x < H) {
            const int c = threadIdx.x;
            float a = 0.f;
            for (int r = 0; r < T; r++) a = fmaf(dy[r], gelu(z2[r * H + c]), a);
            gw3[c] += a;
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < H; i += blockDim.x) part[(int64_t)blockIdx.x * kMlpParams + kOffW3 + i] = gw3[i];
}

__global__ void k_mlp_pack(const float *m, uint16_t *w1, uint16_t *w2, float *b1, float *b2, float *w3, float *b3)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < H * kMlpInPad) {
        const int nn = i / kMlpInPad, k = i - nn * kMlpInPad;
        w1[i] = f2bf(k < kMlpIn ? m[kOffW1 + nn * kMlpIn + k] : 0.f);
    }
    if (i < H * H) w2[i] = f2bf(m[kOffW2 + i]);
    if (i < H) {
        b1[i] = m[kOffB1 + i];
        b2[i] = m[kOffB2 + i];
        w3[i] = m[kOffW3 + i];
    }
    if (i == 0) b3[0] = m[kOffB3];
}

__global__ void k_mlp_adam(float *p, const float *g, float *m, float *v, float lr, float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kMlpParams) return;
    const float gi = g[i];
    const float mi = 0.9f * m[i] + 0.1f * gi;
    const float vi = 0.999f * v[i] + 0.001f * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + 1e-8f);
}

// ---- boundary strip ---------------------------------------------------------------------------

// Four CTAs per SM: the weights, the features and the scales fit 4 x 51 KB of shared memory,
// the hidden layer stays in registers (forward_rows_regs).  Warp w gathers rows 32w..32w+31 of
// the tile and runs the network on the same rows, so after the weights are staged the warps
// only synchronise with themselves.
static_assert(offsetof(NetSmem, b1) % 8 == 0 && offsetof(NetSmem, b2) % 8 == 0, "bias pairs load as float2");
// features start on a 16-byte boundary after the weights (their rows are stored 16 bytes at a time)
constexpr size_t kAbcXsOff = (sizeof(NetSmem) + 15) / 16 * 16;
static_assert((KP1 * sizeof(uint16_t)) % 16 == 0 && kMlpInPad % 8 == 0, "16-byte feature rows");

__global__ void __launch_bounds__(128, 4) k_abc_correction(const MlpDev net, const AbcArgs a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    NetSmem &s = *reinterpret_cast<NetSmem *>(smem);
    uint16_t *xs = reinterpret_cast<uint16_t *>(smem + kAbcXsOff);
    float *scale = reinterpret_cast<float *>(xs + T * KP1);
    load_net(s, net);
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
    const int64_t plane = a.nxp * a.nz;
    for (int64_t row0 = (int64_t)blockIdx.x * T; row0 < a.n; row0 += (int64_t)gridDim.x * T) {
        __syncwarp();  // the warp's rows of xs and scale are free again
        // gather, one thread per node: feature (level l, neighbour (dz, dy, dx)) ->
        // l*27 + (dz+1)*9 + (dy+1)*3 + (dx+1); coordinates decoded once, the 27 loads of a level
        // unrolled so that they are in flight together, sponge factors as 3+3+3 axis values.
        // All 81 loads of a node are issued together and held in registers: the largest
        // magnitude, then the scaled BF16 features (no FP32 copy in shared memory).
        {
            const int r = threadIdx.x;  // 128 threads, one row each
            const int64_t row = row0 + r;
            uint16_t *xr = xs + r * KP1;
            if (row < a.n) {
                const int64_t q0 = a.nodes[row];
                const int64_t iy = q0 / plane, rr = q0 - iy * plane, iz = rr / a.nxp, ix = rr - iz * a.nxp;
                bool okx[3], oky[3], okz[3];
                float fx[3], fy[3], fz[3];
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    okx[d] = ix + d - 1 >= 0 && ix + d - 1 < a.nx;
                    oky[d] = iy + d - 1 >= 0 && iy + d - 1 < a.ny;
                    okz[d] = iz + d - 1 >= 0 && iz + d - 1 < a.nz;
                    fx[d] = (a.sx && okx[d]) ? __ldg(a.sx + ix + d - 1) : 1.f;
                    fy[d] = (a.sx && oky[d]) ? __ldg(a.sy + iy + d - 1) : 1.f;
                    fz[d] = (a.sx && okz[d]) ? __ldg(a.sz + iz + d - 1) : 1.f;
                }
                // the 27 features of level l (level 1 carries its pending sponge factor)
                auto level = [&](int l, float (&v)[27]) {
                    const float *lv = l == 0 ? a.p_new : (l == 1 ? a.p_cur : a.hist);
#pragma unroll
                    for (int nb = 0; nb < 27; nb++) {
                        const int dz = nb / 9, dy = (nb / 3) % 3, dx = nb % 3;
                        const float x = (okx[dx] && oky[dy] && okz[dz])
                                            ? lv[(ix + dx - 1) + (iz + dz - 1) * a.nxp + (iy + dy - 1) * plane]
                                            : 0.f;
                        v[nb] = l == 1 ? x * ((fx[dx] * fz[dz]) * fy[dy]) : x;
                    }
                };
                float v[3][27];
#pragma unroll
                for (int l = 0; l < 3; l++) level(l, v[l]);
                float m = 0.f;
#pragma unroll
                for (int l = 0; l < 3; l++)
#pragma unroll
                    for (int nb = 0; nb < 27; nb++) m = fmaxf(m, fabsf(v[l][nb]));
                const float sc = m + 1e-30f;
                scale[r] = sc;
                const float inv = 1.f / sc;
                // the row as BF16 pairs (feature k in the low half), zero-padded, stored 8
                // features at a time (rows are 16-byte aligned)
                uint32_t pk[kMlpInPad / 2];
#pragma unroll
                for (int k = 0; k < kMlpInPad; k += 2) {
                    if (k < kMlpIn) {
                        const float2 f = mul2(make_float2(v[k / 27][k % 27], k + 1 < kMlpIn ? v[(k + 1) / 27][(k + 1) % 27] : 0.f),
                                              make_float2(inv, inv));
                        pk[k / 2] = pack_bf2(f.x, f.y);
                    } else {
                        pk[k / 2] = 0u;
                    }
                }
#pragma unroll
                for (int c = 0; c < kMlpInPad / 8; c++)
                    reinterpret_cast<uint4 *>(xr)[c] = make_uint4(pk[4 * c], pk[4 * c + 1], pk[4 * c + 2], pk[4 * c + 3]);
            } else {
                scale[r] = 1e-30f;
#pragma unroll
                for (int c = 0; c < kMlpInPad / 8; c++) reinterpret_cast<uint4 *>(xr)[c] = make_uint4(0, 0, 0, 0);
            }
        }
        __syncwarp();
        float yv[2][2];
        forward_rows_regs(s, xs, w * 32, yv);
        if (q == 0)
#pragma unroll
            for (int mt = 0; mt < 2; mt++)
#pragma unroll
                for (int hrow = 0; hrow < 2; hrow++) {
                    const int r = w * 32 + mt * 16 + g + hrow * 8;
                    const int64_t row = row0 + r;
                    // the features are normalised by their largest magnitude: a correction larger
                    // than that is clipped (it bounds what one step of the network can inject)
                    if (row < a.n) {
                        const float v = scale[r] * fminf(fmaxf(yv[mt][hrow], -1.f), 1.f);
                        // absolute: the new value itself, which then never exceeds the largest
                        // magnitude of its own neighbourhood over the three levels
                        a.corr[row] = a.absolute ? v - a.p_new[a.nodes[row]] : v;
                    }
                }
    }
}

constexpr int kPU = kFaceTU + 2, kPV = kFaceTV + 2, kPD = kPU * kPV;  // patch plane with its rim
constexpr int kPL = 3 * kPD;  // one level: depth planes outside (zeros), face, inside
// shared layout after the weights: xs, scale, then the patch [3 levels][3 depths][kPV][kPU],
// each row's output node (-1: none) and the 27 neighbour offsets
constexpr size_t kFaceXsOff = kAbcXsOff;
constexpr size_t kFacePatchOff = kFaceXsOff + sizeof(uint16_t) * T * KP1 + sizeof(float) * T;
constexpr size_t kFaceOutOff = kFacePatchOff + sizeof(float) * 3 * kPL;
constexpr size_t kFaceOffsOff = kFaceOutOff + sizeof(int64_t) * T;
static_assert(kFaceOutOff % 8 == 0, "8-byte aligned output nodes");

__global__ void __launch_bounds__(128, 3) k_abc_face(const MlpDev net, const AbcFaceArgs a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    NetSmem &s = *reinterpret_cast<NetSmem *>(smem);
    uint16_t *xs = reinterpret_cast<uint16_t *>(smem + kFaceXsOff);
    float *scale = reinterpret_cast<float *>(xs + T * KP1);
    float *patch = reinterpret_cast<float *>(smem + kFacePatchOff);
    int64_t *onode = reinterpret_cast<int64_t *>(smem + kFaceOutOff);
    int *offs = reinterpret_cast<int *>(smem + kFaceOffsOff);
    load_net(s, net);
    // the depth plane outside the box stays zero for every tile
    for (int i = threadIdx.x; i < 3 * kPD; i += blockDim.x) patch[(i / kPD) * kPL + i % kPD] = 0.f;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
    const int64_t plane = a.nxp * a.nz;
    // A tile stages the face and inside planes of the three levels with a one-node rim: a thread
    // takes a position (depth, v, u) and loads it from all three levels, sharing the index
    // arithmetic and the node's sponge factor.  x-faces step through the depth fastest (adjacent
    // in memory), the others along u (rows along x).
    constexpr int NPOS = 2 * kPD, KS = (NPOS + T - 1) / T;
    // position i of the patch: depth (1: face, 2: inside), position along v and u
    auto decode = [&](const FaceDesc &f, int i, int &di, int &vv, int &uu) {
        if (f.axis_n == 0) {
            di = i % 2 + 1;
            const int r = i / 2;
            uu = r % kPU; vv = r / kPU;
        } else {
            uu = i % kPU;
            const int r = i / kPU;
            vv = r % kPV; di = r / kPV + 1;
        }
    };
    // node coordinates by axis (selects, not an indexed array: they stay in registers)
    auto coords = [&](const FaceDesc &f, int u0, int v0, int di, int vv, int uu, int &cx, int &cy, int &cz) {
        const int cu = u0 - 1 + uu, cv = v0 - 1 + vv, cn = f.side + (di - 1) * f.inward;
        cx = f.axis_u == 0 ? cu : (f.axis_v == 0 ? cv : cn);
        cy = f.axis_u == 1 ? cu : (f.axis_v == 1 ? cv : cn);
        cz = f.axis_u == 2 ? cu : (f.axis_v == 2 ? cv : cn);
    };
    // p^{n+1} of a boundary node is the stored p^{n-1} twice damped (the step keeps the
    // Dirichlet value): s * (s * p^{n-1}) = s * hist, the same bits, so boundary nodes take
    // level 0 from the history and this kernel can write their new values in place (no tile
    // reads p^{n+1} of a boundary node, so a tile's loads may run ahead of other tiles' writes).
    // s = (sx*sz)*sy, as the step rounds it.
    float v0s[KS], v1s[KS], v2s[KS], sfs[KS];
    bool bnds[KS];
    auto load_patch = [&](int64_t tt) {
        const int4 td = a.tiles[tt];
        const FaceDesc f = a.face[td.x];
#pragma unroll
        for (int k = 0; k < KS; k++) {
            const int i = threadIdx.x + k * T;
            v0s[k] = v1s[k] = v2s[k] = 0.f;
            sfs[k] = 1.f;
            bnds[k] = false;
            if (i < NPOS) {
                int di, vv, uu, cx, cy, cz;
                decode(f, i, di, vv, uu);
                coords(f, td.y, td.z, di, vv, uu, cx, cy, cz);
                if (cx >= 0 && cx < a.nx && cy >= 0 && cy < a.ny && cz >= 0 && cz < a.nz) {
                    const int64_t qn = cx + (int64_t)cz * a.nxp + (int64_t)cy * plane;
                    bnds[k] = cx == 0 || cx == a.nx - 1 || cy == 0 || cy == a.ny - 1 || cz == 0 || cz == a.nz - 1;
                    v2s[k] = a.hist[qn];
                    v1s[k] = a.p_cur[qn];
                    if (!bnds[k]) v0s[k] = a.p_new[qn];
                    if (a.sx) sfs[k] = (__ldg(a.sx + cx) * __ldg(a.sz + cz)) * __ldg(a.sy + cy);
                }
            }
        }
    };
    // returns the tile's descriptor
    auto store_patch = [&](int64_t tt) {
        const int4 td = a.tiles[tt];
        const FaceDesc f = a.face[td.x];
        if (threadIdx.x < 27) {
            // feature neighbour nb = (dz+1)*9 + (dy+1)*3 + (dx+1) -> offset within a level's patch
            const int dx = (int)threadIdx.x % 3 - 1, dy = ((int)threadIdx.x / 3) % 3 - 1, dz = (int)threadIdx.x / 9 - 1;
            auto along = [&](int axis) { return axis == 0 ? dx : (axis == 1 ? dy : dz); };
            offs[threadIdx.x] = along(f.axis_n) * f.inward * kPD + along(f.axis_v) * kPU + along(f.axis_u);
        }
#pragma unroll
        for (int k = 0; k < KS; k++) {
            const int i = threadIdx.x + k * T;
            if (i < NPOS) {
                int di, vv, uu;
                decode(f, i, di, vv, uu);
                const float p0 = bnds[k] ? v2s[k] * sfs[k] : v0s[k];
                const float p1 = v1s[k] * sfs[k];  // p^n is stored without its last sponge factor
                // p^n of the tile's own nodes and their inside neighbours: the next step's
                // p^{n-1} (every node of the two-node shell is one of these for some tile)
                const int us = td.y - 1 + uu, vs = td.z - 1 + vv;
                if (uu >= 1 && uu <= kFaceTU && vv >= 1 && vv <= kFaceTV && us < f.uhi && vs < f.vhi) {
                    int cx, cy, cz;
                    coords(f, td.y, td.z, di, vv, uu, cx, cy, cz);
                    a.hist_next[cx + (int64_t)cz * a.nxp + (int64_t)cy * plane] = p1;
                }
                const int o = di * kPD + vv * kPU + uu;
                patch[o] = p0;
                patch[kPL + o] = p1;
                patch[2 * kPL + o] = v2s[k];
            }
        }
        return td;
    };
    int4 td = make_int4(0, 0, 0, 0);  // the current tile's descriptor
#if SEM_MLP_FACE_PIPE
    if (blockIdx.x < a.ntiles) {
        load_patch(blockIdx.x);
        td = store_patch(blockIdx.x);
    }
#endif
    for (int64_t t = blockIdx.x; t < a.ntiles; t += gridDim.x) {
#if SEM_MLP_FACE_PIPE
        __syncthreads();  // tile t's patch and offsets are staged
#else
        __syncthreads();  // the previous tile's patch, offsets and rows are consumed
        load_patch(t);
        td = store_patch(t);
        __syncthreads();
#endif
        // features of the row's node from the patch (as k_abc_correction gathers them).  The
        // row's node is on the face if it lies within the face's ranges (every such node is a
        // boundary node, so this is the tile's strip position being valid).
        const int r = threadIdx.x;
        const FaceDesc &fc = a.face[td.x];
        const bool valid = td.y + r % kFaceTU < fc.uhi && td.z + r / kFaceTU < fc.vhi;
        const int base = kPD + (r / kFaceTU + 1) * kPU + (r % kFaceTU + 1);
        uint16_t *xr = xs + r * KP1;
        if (valid) {
            // the row's node on the face plane, where the network's output goes
            int cx, cy, cz;
            coords(fc, td.y, td.z, 1, r / kFaceTU + 1, r % kFaceTU + 1, cx, cy, cz);
            onode[r] = cx + (int64_t)cz * a.nxp + (int64_t)cy * plane;
            float v[3][27];
#pragma unroll
            for (int l = 0; l < 3; l++)
#pragma unroll
                for (int nb = 0; nb < 27; nb++) v[l][nb] = patch[l * kPL + base + offs[nb]];
            // the largest magnitude in nine independent chains (the same value in any order)
            float mm[9];
#pragma unroll
            for (int j = 0; j < 9; j++) mm[j] = 0.f;
#pragma unroll
            for (int l = 0; l < 3; l++)
#pragma unroll
                for (int nb = 0; nb < 27; nb++) mm[nb % 9] = fmaxf(mm[nb % 9], fabsf(v[l][nb]));
            const float m = fmaxf(fmaxf(fmaxf(mm[0], mm[1]), fmaxf(mm[2], mm[3])),
                                  fmaxf(fmaxf(mm[4], mm[5]), fmaxf(fmaxf(mm[6], mm[7]), mm[8])));
            const float sc = m + 1e-30f;
            scale[r] = sc;
            const float inv = 1.f / sc;
            uint32_t pk[kMlpInPad / 2];
#pragma unroll
            for (int k = 0; k < kMlpInPad; k += 2) {
                if (k < kMlpIn) {
                    const float2 fv = mul2(make_float2(v[k / 27][k % 27], k + 1 < kMlpIn ? v[(k + 1) / 27][(k + 1) % 27] : 0.f),
                                           make_float2(inv, inv));
                    pk[k / 2] = pack_bf2(fv.x, fv.y);
                } else {
                    pk[k / 2] = 0u;
                }
            }
#pragma unroll
            for (int c = 0; c < kMlpInPad / 8; c++)
                reinterpret_cast<uint4 *>(xr)[c] = make_uint4(pk[4 * c], pk[4 * c + 1], pk[4 * c + 2], pk[4 * c + 3]);
        } else {
            onode[r] = -1;
            scale[r] = 1e-30f;
#pragma unroll
            for (int c = 0; c < kMlpInPad / 8; c++) reinterpret_cast<uint4 *>(xr)[c] = make_uint4(0, 0, 0, 0);
        }
#if SEM_MLP_FACE_PIPE
        // the next tile's loads are in flight while this tile runs the network
        const int64_t tn = t + gridDim.x;
        if (tn < a.ntiles) load_patch(tn);
#endif
        __syncwarp();
        float yv[2][2];
        forward_rows_regs(s, xs, w * 32, yv);
        if (q == 0)
#pragma unroll
            for (int mt = 0; mt < 2; mt++)
#pragma unroll
                for (int hrow = 0; hrow < 2; hrow++) {
                    // rows of this warp: their nodes and scales were written by its own lanes
                    const int rr = w * 32 + mt * 16 + g + hrow * 8;
                    const int64_t o = onode[rr];
                    if (o >= 0) a.p_new[o] = scale[rr] * fminf(fmaxf(yv[mt][hrow], -1.f), 1.f);
                }
#if SEM_MLP_FACE_PIPE
        __syncthreads();  // every warp has read tile t's patch and offsets
        if (tn < a.ntiles) td = store_patch(tn);
#endif
    }
}

__global__ void k_abc_apply(const AbcArgs a, float *p_new)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x)
        p_new[a.nodes[i]] += a.corr[i];
}

// hist <- p^n (actual values) on the history shell
__global__ void k_abc_history(const int64_t *shell, int64_t n, const float *p_cur, const float *sx, const float *sy,
                              const float *sz, int64_t nxp, int64_t nz, float *hist)
{
    const int64_t plane = nxp * nz;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t q0 = shell[i];
        const int64_t iy = q0 / plane, rr = q0 - iy * plane, iz = rr / nxp, ix = rr - iz * nxp;
        hist[q0] = p_cur[q0] * (sx ? (sx[ix] * sz[iz]) * sy[iy] : 1.f);
    }
}

__global__ void k_gather_rows(const float *x, const float *t, const int64_t *idx, int64_t nb, float *bx, float *bt)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nb * kMlpIn;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / kMlpIn, k = i - r * kMlpIn;
        const int64_t src = idx[r];
        bx[i] = x[src * kMlpIn + k];
        if (k == 0) bt[r] = t[src];
    }
}

size_t smem_forward() { return sizeof(NetSmem) + sizeof(uint16_t) * T * (KP1 + KP2); }
size_t smem_train() { return smem_forward() + sizeof(TrainSmem); }
size_t smem_w3() { return smem_forward() + sizeof(float) * (T * H + T + H); }
size_t smem_abc() { return kAbcXsOff + sizeof(uint16_t) * T * KP1 + sizeof(float) * T; }
size_t smem_face() { return kFaceOffsOff + sizeof(int) * 32; }

int grid_for(int64_t n)
{
    const int64_t tiles = (n + T - 1) / T;
    return (int)std::min<int64_t>(tiles, 152 * 4);
}

}  // namespace

cudaError_t mlp_pack(const float *master, uint16_t *w1, uint16_t *w2, float *b1, float *b2, float *w3, float *b3,
                     cudaStream_t s)
{
    k_mlp_pack<<<(H * kMlpInPad + 255) / 256, 256, 0, s>>>(master, w1, w2, b1, b2, w3, b3);
    return cudaGetLastError();
}

cudaError_t mlp_forward(const MlpDev &net, const float *x, float *y, int64_t n, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    const size_t sm = smem_forward();
    cudaError_t e = cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    k_mlp_forward<<<grid_for(n), T, sm, s>>>(net, x, y, n);
    return cudaGetLastError();
}

cudaError_t mlp_loss_grad(const MlpDev &net, const float *x, const float *t, int64_t n, double *loss, float *grad,
                          float *part, double *part_loss, cudaStream_t s, const float *dy_in, float *dx_out)
{
    if (n <= 0) return cudaSuccess;
    const int nb = grid_for(n);
    static_assert(kMlpMaxCTAs >= 152 * 4, "partial-sum rows for every CTA of grid_for");
    size_t sm = smem_train();
    cudaError_t e = cudaFuncSetAttribute(k_mlp_train_pass, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    k_mlp_train_pass<<<nb, T, sm, s>>>(net, x, t, n, part_loss, part, dy_in, dx_out);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    sm = smem_w3();
    if ((e = cudaFuncSetAttribute(k_mlp_grad_w3, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)) != cudaSuccess)
        return e;
    k_mlp_grad_w3<<<nb, T, sm, s>>>(net, x, t, n, part, dy_in);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    k_mlp_reduce<<<(kMlpParams + 255) / 256, 256, 0, s>>>(part, part_loss, nb, grad, loss);
    return cudaGetLastError();
}

cudaError_t mlp_adam(float *master, const float *grad, float *m, float *v, int t, float lr, cudaStream_t s)
{
    const float c1 = 1.f / (1.f - powf(0.9f, (float)t)), c2 = 1.f / (1.f - powf(0.999f, (float)t));
    k_mlp_adam<<<(kMlpParams + 255) / 256, 256, 0, s>>>(master, grad, m, v, lr, c1, c2);
    return cudaGetLastError();
}

cudaError_t mlp_gather_rows(const float *x, const float *t, const int64_t *idx, int64_t nb, float *bx, float *bt,
                            cudaStream_t s)
{
    if (nb > 0)
        k_gather_rows<<<(int)std::min<int64_t>((nb * kMlpIn + 255) / 256, 152 * 16), 256, 0, s>>>(x, t, idx, nb, bx, bt);
    return cudaGetLastError();
}

// Per-device launch set-up of a boundary kernel: its shared-memory limit is raised, and the
// resident CTAs of the device (SMs x CTAs per SM) recorded, once per device.
struct DeviceLaunch {
    int dev;
    int resident;
};

template <class K>
cudaError_t resident_ctas(K kernel, size_t sm, std::vector<DeviceLaunch> &cache, int &resident)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    for (const DeviceLaunch &d : cache)
        if (d.dev == dev) { resident = d.resident; return cudaSuccess; }
    if ((e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)) != cudaSuccess) return e;
    int sms = 152, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, T, sm) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    resident = sms * per_sm;
    cache.push_back({dev, resident});
    return cudaSuccess;
}

cudaError_t abc_correction(const MlpDev &net, const AbcArgs &a, cudaStream_t s)
{
    if (a.n <= 0) return cudaSuccess;
    const size_t sm = smem_abc();
    static std::vector<DeviceLaunch> cache;
    int resident = 0;
    cudaError_t e = resident_ctas(k_abc_correction, sm, cache, resident);
    if (e != cudaSuccess) return e;
    // persistent CTAs, as many as are resident at once: the weights are staged once per CTA
    const int64_t tiles = (a.n + T - 1) / T;
    k_abc_correction<<<(unsigned)std::min<int64_t>(tiles, resident), T, sm, s>>>(net, a);
    return cudaGetLastError();
}

cudaError_t abc_face(const MlpDev &net, const AbcFaceArgs &a, cudaStream_t s)
{
    if (a.ntiles <= 0) return cudaSuccess;
    const size_t sm = smem_face();
    static std::vector<DeviceLaunch> cache;
    int resident = 0;
    cudaError_t e = resident_ctas(k_abc_face, sm, cache, resident);
    if (e != cudaSuccess) return e;
    // persistent CTAs, as many as are resident at once (the weights are staged once per CTA)
    k_abc_face<<<(unsigned)std::min<int64_t>(a.ntiles, resident), T, sm, s>>>(net, a);
    return cudaGetLastError();
}

cudaError_t abc_apply(const AbcArgs &a, float *p_new, float *hist, cudaStream_t s)
{
    (void)hist;
    if (a.n > 0) k_abc_apply<<<(int)std::min<int64_t>((a.n + 255) / 256, 152 * 16), 256, 0, s>>>(a, p_new);
    return cudaGetLastError();
}

cudaError_t abc_history(const int64_t *shell, int64_t n, const float *p_cur, const float *sx, const float *sy,
                        const float *sz, int64_t nxp, int64_t nz, float *hist, cudaStream_t s)
{
    if (n > 0)
        k_abc_history<<<(int)std::min<int64_t>((n + 255) / 256, 152 * 16), 256, 0, s>>>(shell, n, p_cur, sx, sy, sz,
                                                                                         nxp, nz, hist);
    return cudaGetLastError();
}

}  // namespace semgb
