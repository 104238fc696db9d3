// stencil.h -- the SEM step as one fused pass over the nodes of a uniform box mesh.
//
// On the reference's mesh (SEMmesh: uniform axis-aligned hexahedra) every element has the same
// diagonal metric, so the assembled stiffness factorises exactly over the three axes:
//     (K p)_i = g1 Wz Wy [A_x p]_i + g2 Wx Wy [A_z p]_i + g3 Wx Wz [A_y p]_i
// with A the assembled 1-D GLL stiffness (element blocks D^T diag(w) D, shared end nodes
// summed) and W the assembled 1-D GLL weight of the node along an axis (w_l inside an element,
// w_0 + w_o on an element face).  This is the same linear operator as the element loop of
// SEMsolver::computeOneStep (SEMsolver.cpp:46-82, SEMQkGLIntegrals.hpp:363-520), evaluated node
// by node: no scatter, no accumulator array, and the leapfrog update, sponge and receiver
// sampling happen in the same pass (SEMsolver.cpp:85-89).
#pragma once
#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

#include "host_util.h"
#include "kernels.h"

namespace semgb {

// Tensor maps of one pressure buffer (3-D tiles of the device layout).
struct LevelMaps {
    CUtensorMap win;    // (tile width + x halo) x (TZ + 2o rows) x 1 plane
    CUtensorMap tile;   // tile width x TZ rows x 1 plane
};

// Node-class coefficients of the reference-rounding pass (layout of reference_class_table:
// [axis][ly][lz][d + o][lx]), handed to the kernel by value as a __grid_constant__ parameter.
template <int O>
struct alignas(16) ClassTable {
    float c[3][O][O][2 * O + 1][O];
};

// Tile shapes of the pass: the default for every order, and for order 4 a square 32 x 32 tile
// that single-shot plain steps may take (the 64 x 16 default wastes more lanes on some boxes)
enum StencilTileShape { kTileDefault = 0, kTileSquare = 1 };

struct StencilTables {
    int order = 0;
    int shape = kTileDefault;  // tile shape the kernels and the tables below are built for
    // SEM_ROUNDING_REFERENCE: the reference's assembled node-class coefficients, host memory
    // owned by the tables (null: the tensor-product operator below)
    float *class_tab = nullptr;
    int64_t nx = 0, nxp = 0, ny = 0, nz = 0;
    float g[3] = {0, 0, 0};   // g_d = |detJ| / J_dd^2 for x (xi1), z (xi2), y (xi3)
    float wa[6] = {0};        // assembled weight by local index: wa[0] = 2 w_0, wa[l] = w_l
    int tile_x = 0, tile_z = 0, halo_x = 0;
    int threads = 0;          // per CTA
    int grid[3] = {0, 0, 0};  // tiles along x, z and y-chunks (launch: x * z * nshot CTAs by chunks)
    int nshot = 1;            // shots stacked along y in the levels (many-shot form)
    int cluster = 1;          // many-shot form: CTAs of consecutive shots of a tile co-scheduled as
                              // one thread-block cluster (divides nshot; 1: plain launch)
    int64_t shot_stride = 0;  // floats per shot field: nxp * nz * ny
    int ychunk = 0;           // planes per CTA
    size_t smem = 0;          // dynamic shared memory per CTA
    LevelMaps lv[2];          // per pressure buffer
    CUtensorMap amap;         // dt^2/M, tile boxes
    const float *bound[3] = {nullptr, nullptr, nullptr};  // buffers the maps describe
    // receivers grouped by the CTA that owns their node: rec_off[cta]..rec_off[cta+1] index
    // rec_idx, which holds positions in the solver's node-sorted receiver arrays
    int *d_rec_off = nullptr;
    int *d_rec_idx = nullptr;
    uint64_t rec_version = 0;
};

struct StencilArgs {
    const float *cur;
    float *prev;               // in: stored previous level; out: new level
    const float *sx, *sy, *sz;
    const int64_t *rec_node;   // node-sorted receivers (device-layout indices)
    const int *rec_perm;
    const int *rec_off;        // per CTA (from StencilTables)
    const int *rec_idx;
    int nrec;
    float *traces;
    const int *ctr;
    int *status;               // set non-zero when a bounded wait gives up
    // adjoint support (device layout, one value per node; unused by the plain step):
    //   STENCIL_RECORD_KP: kp <- (K p^n) on interior nodes, 0 elsewhere
    //   STENCIL_GRADIENT:  grad += p^n * kp (kp recorded by a forward pass)
    float *kp;
    float *grad;
};

enum StencilMode { STENCIL_PLAIN = 0, STENCIL_RECORD_KP = 1, STENCIL_GRADIENT = 2 };

// One member of a group launch (k_group.cu): several boxes of orders 1..kGroupMaxOrder advanced
// by one launch per step.  Lives in device memory; the launch's CTAs cta0.. belong to it.
constexpr int kGroupMaxOrder = 4;
struct GroupMember {  // 128-byte aligned, as its tensor maps
    StencilTables t;    // tensor maps of the member's levels, its tiling with the group's y-chunks
    StencilArgs a[2];   // [k]: pass arguments at group parity k (current level cur0 ^ k)
    SourceArgs src[2];  // [k]: source arguments at group parity k
    int order;
    int cur0;           // index of the member's current level at parity 0
    int cta0;           // the member's first CTA in the launch
};

// Set up the group kernels on the current device (coefficient tables, shared-memory limit).
cudaError_t group_kernel_setup();
// Dynamic shared memory of a group launch whose members have orders up to max_order, and the
// CTAs per SM it allows (threads per CTA: kGroupThreads).
constexpr int kGroupThreads = 128;
size_t group_smem(int max_order);
int group_blocks_per_sm(int max_order);
// One step of every member: sources, then the pass (receivers included).  cta_member[c] is the
// member of CTA c; members[m].cta0 its first CTA.
cudaError_t launch_group_step(const GroupMember *members, int n_members, const int *cta_member, int n_ctas,
                              int max_order, int k, cudaStream_t s);

// Tables and tiling for a box (no device buffers yet).  Returns 0 or a cudaError_t.
// nshot > 1: the many-shot form, levels holding nshot fields one after another (traces
// [step][receiver][shot]); dt^2/M and the sponge are shared.
// shape: kTileDefault, kTileSquare (order 4, one shot; otherwise the default) or -1 to choose
int stencil_tables_create(const Box &b, const Gll &g, const Geometry &geo, int nshot, StencilTables **out,
                          int shape = -1);
// tile of a shape: nodes along x and z, x halo, threads per CTA
void stencil_tile_dims(int order, int shape, int &tx, int &tz, int &hx, int &threads);
// Describe the solver's two pressure buffers and its dt^2/M buffer with tensor maps.
int stencil_bind(StencilTables &t, const float *p0, const float *p1, const float *a);
// Group node-sorted receivers (device-layout indices) by owning CTA (device CSR in t).
cudaError_t stencil_set_receivers(StencilTables &t, const int64_t *sorted_nodes, int nrec, uint64_t version);
// Switch the pass to the reference-rounding operator with node-class table `tab` (layout of
// reference_class_table, copied), or back to the tensor-product operator (tab null).
int stencil_set_class_table(StencilTables &t, const float *tab);
void stencil_tables_free(StencilTables *&t);
cudaError_t stencil_kernel_setup();
// cur_index: which of the bound pressure buffers is the current level.
// direct: operator form sum_d T_d p_{i+d} with the diagonal T_0 = -sum_{d!=0} T_d (fewer
// instructions); otherwise the difference form sum_{d!=0} T_d (p_{i+d} - p_i), exactly zero on a
// constant field.
cudaError_t launch_stencil(const StencilTables &t, const StencilArgs &a, int cur_index, bool sponge,
                           cudaStream_t s, int mode = STENCIL_PLAIN, bool direct = true);

}  // namespace semgb
