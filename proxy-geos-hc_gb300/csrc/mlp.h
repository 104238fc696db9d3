// mlp.h -- the boundary network of the learned absorbing boundary: 81 inputs (p at three time
// levels on the 3x3x3 node neighbourhood, divided by a per-node scale), two hidden layers of 64
// with GELU, one output.  BF16 weights and activations into FP32 accumulators on the tensor
// cores (mma.sync m16n8k16), FP32 master weights and Adam state for training.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "host_util.h"

namespace semgb {

constexpr int kMlpIn = 81;
constexpr int kMlpInPad = 96;  // K of layer 1 padded to whole 16-wide MMA steps
constexpr int kMlpHidden = 64;
// FP32 master layout: W1[64][81], b1[64], W2[64][64], b2[64], w3[64], b3
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kMlpHidden * kMlpIn;
constexpr int kOffW2 = kOffB1 + kMlpHidden;
constexpr int kOffB2 = kOffW2 + kMlpHidden * kMlpHidden;
constexpr int kOffW3 = kOffB2 + kMlpHidden;
constexpr int kOffB3 = kOffW3 + kMlpHidden;
constexpr int kMlpParams = kOffB3 + 1;
constexpr int kMlpTile = 128;  // rows (nodes or samples) per CTA

// Device copy of the network for the kernels: BF16 W1 as [64][96] (zero-padded K) and W2 as
// [64][64], FP32 biases and output layer.
struct MlpDev {
    const uint16_t *w1;  // [64][96] bf16 bits
    const uint16_t *w2;  // [64][64]
    const float *b1, *b2, *w3, *b3;
};

// Strip of nodes the network corrects, and the levels it reads.
struct AbcArgs {
    const int64_t *nodes;  // device-layout indices of the strip nodes
    int64_t n;
    const float *p_new;    // p^{n+1} (sponge applied)
    const float *p_cur;    // p^n stored without its last sponge factor (actual = s * stored)
    const float *hist;     // p^{n-1} (actual values) on the history shell, device layout [n_int]
    const float *sx, *sy, *sz;  // sponge factors (null: none)
    int64_t nx, nxp, ny, nz;
    float *corr;           // out: correction per strip node
    int absolute;          // 1: the network gives the node's value (scale * y), 0: a correction
};

// Face-tiled correction of the boundary nodes (strip layer 0): the six faces of the box are cut
// into tiles of kFaceTU x kFaceTV nodes (one CTA tile of kMlpTile rows), every boundary node on
// exactly one face.  A tile's three levels on the face plane and the plane inside it, with a
// one-node rim, are staged in shared memory once, and each node's 81 features come from there.
constexpr int kFaceTU = 16, kFaceTV = 8;
static_assert(kFaceTU * kFaceTV == kMlpTile, "one face tile is one network tile");
struct FaceDesc {
    int axis_n, axis_u, axis_v;  // axes (0: x, 1: y, 2: z) normal to the face and along its tiles
    int side;                    // node coordinate of the face along axis_n
    int inward;                  // +1 or -1: the direction into the box along axis_n
    int ulo, uhi, vlo, vhi;      // node ranges of the face along axis_u and axis_v
};
struct AbcFaceArgs {
    FaceDesc face[6];
    const int4 *tiles;     // (face, u0, v0, 0) per tile
    int64_t ntiles;
    float *p_new;          // p^{n+1} (sponge applied); out: the boundary nodes' new values
    const float *p_cur;    // p^n stored without its last sponge factor
    const float *hist;     // p^{n-1} (actual values) on the two-node shell, device layout
    float *hist_next;      // out: p^n (actual values) on the two-node shell, device layout
    const float *sx, *sy, *sz;  // sponge factors (null: none)
    int64_t nx, nxp, ny, nz;
};
// Face-tiled boundary values (the features, network, output and clipping of abc_correction with
// absolute values) written into p_new, and p^n into hist_next on the shell.  p^{n+1} of the
// boundary nodes is taken as s * hist (what the step leaves there), the rest from p_new.
cudaError_t abc_face(const MlpDev &net, const AbcFaceArgs &a, cudaStream_t s);

// ---- adjoint of the time loop with the network on the boundary nodes (k_bptt.cu) ----------
// Work arrays of one backward pass over a box (device layout, nb boundary nodes).
struct BpttFields {
    int nx, ny, nz;
    int64_t nxp, n_int;
    const float *sx, *sy, *sz;  // sponge factors (null: none)
    const int64_t *nodes;       // boundary nodes (device layout), nb of them
    int64_t nb;
    const int *sidx;            // [n_int]: index in `nodes`, -1 elsewhere
    float *x;                   // [nb][81] features divided by the scale
    float *scale;               // [nb]
    int *kstar;                 // [nb] arg-max feature | 0x100 if negative; -1: all zero
    float *y, *g, *dy;          // [nb] network output, adjoint of the node's new value, output gradient
    float *dx;                  // [nb][81] input gradient, then feature gradient
    float *a[3];                // adjoints of out^m, out^{m-1}, out^{m-2}
    float *v;                   // [n_int] work field
    const int64_t *roi;         // region of interest (device layout), n_roi nodes
    int n_roi;
};
// The stiffness operator of the stencil pass: 1-D table T[l][d + o] (direct form, diagonal
// included), assembled weights by local index, g for the x, z and y terms.
struct BpttOperator {
    int order;
    float T[kMaxOrder * (2 * kMaxOrder + 1)];
    float wa[kMaxOrder];
    float g[3];
};
// Features of the boundary nodes from out^m, out^{m-1}, out^{m-2}.
cudaError_t bptt_features(const BpttFields &f, const float *lm, const float *lm1, const float *lm2, cudaStream_t s);
// g and dy from A0 and the network output y.
cudaError_t bptt_dy(const BpttFields &f, cudaStream_t s);
// dx -> feature gradient, gathered into A0, A1, A2.
cudaError_t bptt_scatter(const BpttFields &f, cudaStream_t s);
// Interior leapfrog adjoint (A0 -> A1, A2); a_mass = dt^2 / M.
cudaError_t bptt_interior(const BpttFields &f, const BpttOperator &op, const float *a_mass, cudaStream_t s);
// Loss over the region of interest at one step and its gradient into A0.
cudaError_t bptt_loss(const BpttFields &f, const float *out, const float *ref, double *loss, cudaStream_t s);

// bf16 conversion of the FP32 master weights into the device layout.
cudaError_t mlp_pack(const float *master, uint16_t *w1, uint16_t *w2, float *b1, float *b2, float *w3, float *b3,
                     cudaStream_t s);
// y[i] = net(x[i]) for x [n][81] (FP32, device).
cudaError_t mlp_forward(const MlpDev &net, const float *x, float *y, int64_t n, cudaStream_t s);
// Loss 1/n sum (net(x_i) - t_i)^2 accumulated into *loss (double), gradients with respect to the
// master parameters accumulated into grad (FP32 [kMlpParams]).
// Deterministic: every CTA writes its partial sums to part ([kMlpMaxCTAs][kMlpParams]) and
// part_loss ([kMlpMaxCTAs]), and one pass adds them in CTA order.
constexpr int kMlpMaxCTAs = 152 * 4;
// With dy_in (device, [n]) the output gradient per row is given instead of the squared-error loss
// (t is not read and the loss is not accumulated); with dx_out (device, [n][81]) the gradient with
// respect to the inputs is written too.
cudaError_t mlp_loss_grad(const MlpDev &net, const float *x, const float *t, int64_t n, double *loss, float *grad,
                          float *part, double *part_loss, cudaStream_t s, const float *dy_in = nullptr,
                          float *dx_out = nullptr);
// bx[i] = x[idx[i]], bt[i] = t[idx[i]] for i < nb (minibatch rows).
cudaError_t mlp_gather_rows(const float *x, const float *t, const int64_t *idx, int64_t nb, float *bx, float *bt,
                            cudaStream_t s);
// Adam step on the FP32 master weights (m, v moments; t = step count starting at 1).
cudaError_t mlp_adam(float *master, const float *grad, float *m, float *v, int t, float lr, cudaStream_t s);
// Boundary correction: corr[i] = scale_i * net(features_i / scale_i) for the strip nodes.
cudaError_t abc_correction(const MlpDev &net, const AbcArgs &a, cudaStream_t s);
// p_new[node_i] += corr[i].
cudaError_t abc_apply(const AbcArgs &a, float *p_new, float *hist, cudaStream_t s);
// hist[q] <- p^n (actual: stored value times the node's sponge factor) on the history shell.
cudaError_t abc_history(const int64_t *shell, int64_t n, const float *p_cur, const float *sx, const float *sy,
                        const float *sz, int64_t nxp, int64_t nz, float *hist, cudaStream_t s);

}  // namespace semgb
