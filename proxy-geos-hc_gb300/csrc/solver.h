// solver.h -- the solver handle (struct sem_solver) and the internal step interface shared by
// the C-ABI translation units (api.cu: plain solver; adjoint_api.cu: checkpointed adjoint).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "abi.h"
#include "stencil.h"

struct sem_solver {
    sem_mesh *mesh = nullptr;
    float dt = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int kernel = SEM_KERNEL_AUTO;
    int form = SEM_FORM_DIRECT;  // operator form of the stencil pass
    int rounding = SEM_ROUNDING_DEFAULT;  // SEM_ROUNDING_REFERENCE: the reference's rounded rows
    int64_t n_int = 0;               // nodes of the device layout
    float *d_p[2] = {nullptr, nullptr};
    int cur = 0;                 // index of the current level
    float *d_y = nullptr;        // element path accumulator
    float *d_a = nullptr;        // dt^2 / M
    uint64_t a_version = 0;
    float *d_tab = nullptr;      // element coefficient table
    float *d_rtab = nullptr;     // SEM_ROUNDING_REFERENCE: the reference's element rows (element path)
    float *d_mref = nullptr;     // SEM_ROUNDING_REFERENCE: the reference's float mass (element path)
    uint64_t mref_version = 0;
    double *d_w = nullptr;       // GLL weights (double) for the mass kernel
    semgb::StencilTables *stencil = nullptr;
    int tile_shape = -1;  // stencil tile shape: -1 chosen per box, or a semgb::StencilTileShape
    // sponge
    bool sponge = false;
    float *d_sx = nullptr, *d_sy = nullptr, *d_sz = nullptr;
    // sources
    int nsrc = 0, nsamples = 0;
    bool src_distinct = true;  // no two sources on one node
    int64_t *d_src_node = nullptr;
    float *d_src_coef = nullptr;
    float *d_wavelet = nullptr;
    std::vector<int64_t> src_node;
    std::vector<float> src_coef;
    // receivers
    int nrec = 0;
    int64_t *d_rec_node = nullptr;  // sorted by node
    int *d_rec_perm = nullptr;      // sorted position -> caller's receiver index
    std::vector<int64_t> rec_sorted;
    uint64_t rec_version = 1;
    float *d_traces = nullptr;      // [trace_cap][nrec]
    int64_t trace_cap = 0;
    int64_t traces_checked = 0;
    int *d_ctr = nullptr;           // [0] next step, [1] step in flight
    int *d_status = nullptr;        // non-zero after a bounded device wait gave up
    int *d_upd_rec_off = nullptr;   // receivers grouped by update-kernel block
    uint64_t upd_rec_version = 0;
    int64_t steps_done = 0;
    // graphs: [parity] two steps starting at level `parity`
    cudaGraphExec_t graph2[2] = {nullptr, nullptr};
    uint64_t graph_gen = 0;  // bumped whenever captured launch parameters may have changed
};

// Side buffers of one stencil pass (modes of k_stencil.cu: record K p, or accumulate a gradient).
struct StepExtra {
    int mode = semgb::STENCIL_PLAIN;
    float *kp = nullptr;
    float *grad = nullptr;
};

// Device resources for stepping n_new more steps (mass, stencil tables, receiver CSR, trace
// storage).  Returns a SEM_* status.
int solver_prepare(sem_solver *s, int64_t n_new);
// One step from level c (source, stiffness + update, receivers) enqueued on the solver stream.
cudaError_t solver_enqueue_step(sem_solver *s, int c, cudaEvent_t *ev = nullptr, const StepExtra *extra = nullptr);
void solver_invalidate_graphs(sem_solver *s);
// Sources by device-layout node with explicit coefficients: p^n[node_k] += coef_k * wavelet_k[n].
int solver_set_raw_sources(sem_solver *s, int n_src, const int64_t *nodes, const float *coef, const float *wavelet,
                           int n_samples);
// A field between the device layout (rows of nxp floats) and a host array in the reference
// layout (rows of nx floats), `rows` rows, through two pinned staging buffers: the copy engine
// gathers (scatters) one chunk of rows while the host moves the previous one, so the caller's
// pageable array is not crossed row by row.  Ordered on and synchronous with stream s.
cudaError_t field_to_host(float *dst, const float *src, int64_t nx, int64_t nxp, int64_t rows, cudaStream_t s);
cudaError_t field_from_host(float *dst, const float *src, int64_t nx, int64_t nxp, int64_t rows, cudaStream_t s);
