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
#include <cuda_runtime.h>

#include "host_util.h"
#include "kernels.h"

namespace semgb {

struct StencilTables {
    int order = 0;
    int64_t nx = 0, ny = 0, nz = 0, n = 0;
    float g[3] = {0, 0, 0};   // g_d = |detJ| / J_dd^2 for x (xi1), z (xi2), y (xi3)
    float wa[6] = {0};        // assembled weight by local index: wa[0] = 2 w_0, wa[l] = w_l
};

struct StencilArgs {
    const float *cur;
    float *prev;               // in: stored previous level; out: new level
    const float *a;            // dt^2 / M
    const float *sx, *sy, *sz;
    const int64_t *rec_node;
    const int *rec_perm;
    int nrec;
    float *traces;
    const int *ctr;
};

int stencil_tables_create(const Box &b, const Gll &g, const Geometry &geo, StencilTables **out);
void stencil_tables_free(StencilTables *&t);
cudaError_t stencil_kernel_setup();
cudaError_t launch_stencil(const StencilTables &t, const StencilArgs &a, bool sponge, cudaStream_t s);

}  // namespace semgb
