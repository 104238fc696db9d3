/*
 * semgb.h -- C ABI of the GB300-native spectral-element (SEM) acoustic time step.
 *
 * This is the drop-in boundary for the reference's SEM solver path (numpex/proxy-geos-hc,
 * src/sem): mesh and model setup, the per-step compute, source and receiver I/O.  Each entry
 * point names the reference interface it replaces.
 *
 * Conventions
 *  - Every function returns an int status (SEM_OK or a SEM_ERR_* code); sem_last_error_string()
 *    gives a thread-local message for the last failure on the calling thread.  No C++ exception
 *    crosses this boundary.
 *  - The library owns all device memory.  Buffers passed in or out are host memory owned by the
 *    caller unless a name says "device".  Functions that return data synchronise the solver's
 *    stream first; sem_solver_step only enqueues work.  Whole fields (pressure levels, squared
 *    slowness, gradients) cross through the library's pinned staging buffers, so the caller's
 *    arrays may be ordinary pageable memory; the first such copy on each device pins 32 MB of
 *    host memory for that device, kept until the process exits.
 *  - A handle is used by one host thread at a time; separate solvers may run on separate streams.
 *  - Node numbering is the reference's: node = ix + iz*nx + iy*nx*nz with nx = ex*order+1 etc.
 *    (SEMmesh.cpp:142-231); element e = ix + iz*ex + iy*ex*ez; coordinates are (x, y, z).
 *  - Sizes and node indices are 64-bit.
 */
#ifndef SEMGB_H_
#define SEMGB_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    SEM_OK = 0,
    SEM_ERR_ARG = 1,       /* invalid argument (null pointer, size, order, index out of range) */
    SEM_ERR_CUDA = 2,      /* a CUDA call failed (message has the CUDA error string) */
    SEM_ERR_OOM = 3,       /* device or host allocation failed */
    SEM_ERR_TIMEOUT = 4,   /* a bounded device wait gave up */
    SEM_ERR_UNSTABLE = 5,  /* non-finite values detected in the wavefield or traces */
    SEM_ERR_STATE = 6      /* call not valid in the handle's current state */
};

/* Step kernels (sem_solver_set_kernel). */
enum {
    SEM_KERNEL_AUTO = 0,     /* fastest available for the mesh (currently SEM_KERNEL_STENCIL) */
    SEM_KERNEL_ELEMENT = 1,  /* element gather / sum-factorised K.p / atomic scatter + update */
    SEM_KERNEL_STENCIL = 2   /* tensor-product assembled operator, one fused pass per step */
};

/* Operator forms of the stencil pass (sem_solver_set_operator_form).  Both evaluate the same
   assembled stiffness rows in FP32.  DIRECT sums T_d p_{i+d} over the row, its diagonal being
   minus the sum of the row's float coefficients -- the form of the reference's element products,
   with FP32 drift no larger than the reference's -- in fewer instructions.  DIFFERENCE sums
   T_d (p_{i+d} - p_i) over the off-diagonal terms: exactly zero on a constant field and less
   FP32 drift against an FP64 run (16^3 Q2 elements, 300 steps: 3.1e-7 against 7.4e-6 relative
   L2 in the traces), ~5 % slower. */
enum { SEM_FORM_DIRECT = 0, SEM_FORM_DIFFERENCE = 1 };

/* Rounding of the stiffness operator (sem_solver_set_rounding).
   DEFAULT: the operator as the build forms it (tensor-product coefficients for the stencil pass,
   the element's 1-D stiffness in difference form for the element pass).
   REFERENCE: the reference's own float-rounded element rows (sem_box_refround_rows), so that
   the FP32 result follows the reference's rather than drifting from it by the two codes' FP32
   errors: the stencil pass steps with their assembled node-class coefficients
   (sem_box_refround_class_table), one accumulation per node; the element pass applies the rows
   pencil by pencil.  On the 40^3 Q2 1500-step workload the two stay within 1.2e-6 (traces) and
   6.5e-6 (final pressure) relative L2 of the compiled reference, against 2.1e-4 and 4.1e-3 in
   DEFAULT. */
enum { SEM_ROUNDING_DEFAULT = 0, SEM_ROUNDING_REFERENCE = 1 };

/* Tile shape of the stencil pass (sem_solver_set_tile_shape): the nodes along x and z that one
   CTA steps.  DEFAULT: 16o x 8 for o = 1, 2 and 4 (64 x 16 at order 4), 48 x 24 at o = 3, 40 x 20
   at o = 5.  SQUARE: 32 x 32 at order 4 (other orders: the default), for the plain step of one
   shot in the default rounding (the reference rounding, the adjoint's passes and batches keep
   the default; a group's one launch runs each member on its own shape).  AUTO: the shape whose busiest CTA slot marches the
   fewest planes per lane on a node, from the box's node counts (on GB300, 345^3 and 401^3 nodes
   take the square tile: 0.130 against 0.145 ms and 336 against 322 Gnode-steps/s; 481^3 and
   801^3 keep the default).  Every shape gives the same bits. */
enum { SEM_TILE_AUTO = -1, SEM_TILE_DEFAULT = 0, SEM_TILE_SQUARE = 1 };

/* Pressure levels for sem_solver_get_pressure / sem_solver_set_pressure. */
enum { SEM_LEVEL_CURRENT = 0, SEM_LEVEL_PREVIOUS = 1 };

typedef struct sem_mesh sem_mesh;
typedef struct sem_solver sem_solver;

const char *sem_last_error_string(void);
int sem_version(void); /* major*10000 + minor*100 + patch */

/* Self-test of the bounded device waits the kernels use: one CTA waits on an mbarrier phase that
 * nothing completes (no arrival, no copy in flight), so the wait ends at its limit
 * (limit_seconds in (0, 2]); returns SEM_ERR_TIMEOUT with the time waited, and the context stays
 * usable.  Returns SEM_OK only if the wait completed, which would be a defect. */
int sem_selftest_bounded_wait(double limit_seconds, double *waited_seconds);

/* ------------------------------------------------------------------------------------------
 * Host-only utilities (no GPU needed).
 * ------------------------------------------------------------------------------------------ */

/* GLL points xi[order+1], weights w[order+1] (8-decimal values as tabulated by the reference)
 * and derivative table dphi[(order+1)^2], dphi[j*(order+1)+i] = phi_j'(xi_i); order 1..5.
 * Replaces SEMQkGLBasisFunctions::gaussLobattoQuadraturePoints/Weights and
 * getDerivativeBasisFunction1D (SEMQkGLBasisFunctions.hpp:36-117, 310-324). */
int sem_gll_tables(int order, double *xi, double *w, double *dphi);

/* Ricker wavelet samples out[i] = r(i*dt), order 0, 1 or 2.
 * Replaces SolverUtils::computeSourceTerm / evaluateRicker (utils.hpp:11-57). */
int sem_ricker(int nsamples, float dt, float f0, int order, float *out);

/* Node, element and interior-node counts of an ex*ey*ez box of the given order.
 * Replaces SEMmesh::getNumberOfNodes/Elements/InteriorNodes (SEMmesh.cpp:28-54). */
int sem_box_counts(int ex, int ey, int ez, int order, int64_t *n_nodes, int64_t *n_elem,
                   int64_t *n_interior);

/* Element-to-node map rows for elements [e0, e0+count): conn[(e-e0)*(order+1)^3 + local].
 * Replaces SEMmesh::globalNodesList (SEMmesh.cpp:205-231). */
int sem_box_connectivity(int ex, int ey, int ez, int order, int64_t e0, int64_t count,
                         int64_t *conn);

/* Element containing (x,y,z); an axis outside the box maps to element 0 on that axis.
 * Replaces SEMmesh::getElementNumberFromPoints (SEMmesh.cpp:266-285). */
int sem_box_element_from_point(int ex, int ey, int ez, float lx, float ly, float lz, float x,
                               float y, float z, int64_t *element);

/* Nearest GLL node to (x,y,z) (per axis, ties to the lower index, clamped to the box).
 * The reference has no receivers; this is the build's snapping rule for receiver positions. */
int sem_box_nearest_node(int ex, int ey, int ez, float lx, float ly, float lz, int order,
                         float x, float y, float z, int64_t *node);

/* Sponge factors per axis, sx[nx], sy[ny], sz[nz]: for a node at distance d (in elements) from
 * the nearer face of its axis, s = exp(-sigma*((thickness-d)/thickness)^2) when d < thickness,
 * else 1; the node factor is (sx[ix]*sy[iy])*sz[iz].  The reference SEM has no sponge; this is
 * the Gaussian taper of its FD proxy (FDTDinit.hpp:319-396) scaled to `thickness` elements. */
int sem_box_sponge_profile(int ex, int ey, int ez, float lx, float ly, float lz, int order,
                           int thickness, float sigma, float *sx, float *sy, float *sz);

/* The reference's element stiffness rows on one element of the box, rounded as the reference
 * rounds them: computeB's metric in double stored as float, each entry of gradPhiGradPhi's row
 * accumulated in float from double products in its loop order (SEMQkGLIntegrals.hpp:265-513).
 * The box's elements are axis-aligned, so the row of node i has its non-zero entries on the three
 * coordinate lines through i.  rows[3*(order+1)^3*(order+1)]: rows[(a*npe + i)*(order+1) + m] is
 * the entry of node i (local numbering) toward the node of local index m along axis a (0: x,
 * 1: z, 2: y); the x entry at i's own index holds the whole diagonal, the z and y ones zero.
 * These are the rows SEM_ROUNDING_REFERENCE steps with. */
int sem_box_refround_rows(int ex, int ey, int ez, float lx, float ly, float lz, int order, float *rows);

/* Node-class coefficients of the operator the reference assembles from those rows: for a node
 * with local indices (lx, lz, ly) in 0..order-1, the coefficient of the node d places along axis
 * a, summed exactly over the elements holding both nodes and rounded once; the diagonal is the x
 * entry at d = 0.  tab[3*order*order*(2*order+1)*order], index (((a*o + ly)*o + lz)*(2o+1) + d +
 * o)*o + lx.  The stencil pass steps with this table under SEM_ROUNDING_REFERENCE. */
int sem_box_refround_class_table(int ex, int ey, int ez, float lx, float ly, float lz, int order,
                                 float *tab);

/* ------------------------------------------------------------------------------------------
 * Mesh and model (device).
 * ------------------------------------------------------------------------------------------ */

/* Structured box of ex*ey*ez hexahedra of order 1..5 over [0,lx]x[0,ly]x[0,lz].  The element
 * velocity starts at 1500 m/s as in SEMmesh::getModel.
 * Replaces SEMmesh::SEMmesh (SEMmesh.cpp:3-26) plus the mesh half of
 * SEMsolver::computeFEInit / initFEarrays (SEMsolver.cpp:12-17, 144-174). */
int sem_mesh_create_box(int ex, int ey, int ez, float lx, float ly, float lz, int order,
                        sem_mesh **out);
int sem_mesh_destroy(sem_mesh *mesh);

/* n_nodes, n_elem, nodes per element, interior nodes. */
int sem_mesh_info(const sem_mesh *mesh, int64_t *n_nodes, int64_t *n_elem, int *nodes_per_elem,
                  int64_t *n_interior);

/* Copy the device-resident element-to-node map back (int32, [n_elem][(order+1)^3]) for
 * bit-exact checks against SEMmesh::globalNodesList (SEMmesh.cpp:205-231). */
int sem_mesh_get_connectivity(sem_mesh *mesh, int32_t *conn);

/* Per-element velocity c_e (n_elem floats): replaces SEMmesh::getModel (SEMmesh.cpp:288-312).
 * The nodal mass is M_i = sum over elements e touching i of w_i^3 |detJ| / c_e^2
 * (SEMsolver.cpp:74-80). */
int sem_model_set_element_velocity(sem_mesh *mesh, const float *velocity);

/* Per-node squared slowness m_i (n_nodes floats): M_i = m_i * sum_e w_i^3 |detJ|.  Used by the
 * gradient with respect to m; replaces the element model for subsequent solver steps. */
int sem_model_set_node_slowness2(sem_mesh *mesh, const float *m);

/* ------------------------------------------------------------------------------------------
 * Solver.
 * ------------------------------------------------------------------------------------------ */

/* Solver over `mesh` with time step dt; both pressure levels start at zero.
 * Replaces SEMsolver::computeFEInit (SEMsolver.cpp:12-17) and SEMproxy::init_arrays
 * (SEMproxy.cpp:84-90).  The mesh must outlive the solver. */
int sem_solver_create(sem_mesh *mesh, float dt, sem_solver **out);
int sem_solver_destroy(sem_solver *s);

/* Run on a caller-provided cudaStream_t (NULL: the solver's own stream). */
int sem_solver_set_stream(sem_solver *s, void *cuda_stream);

/* Choose the step kernel (SEM_KERNEL_*). */
int sem_solver_set_kernel(sem_solver *s, int kernel);

/* Operator form of the stencil kernel (SEM_FORM_*; default SEM_FORM_DIRECT).  The element kernel
   always uses the difference form.  Extension: the reference has one form. */
int sem_solver_set_operator_form(sem_solver *s, int form);

/* Rounding of the stiffness operator (SEM_ROUNDING_*; default SEM_ROUNDING_DEFAULT).  The
   reference's rows are built for the mesh's exact element size; they are the reference's own
   bit for bit where its float node coordinates are exact (orders 1 and 2 with integer element
   sizes).  SEM_ROUNDING_REFERENCE ignores the operator form.  Extension: parity mode. */
int sem_solver_set_rounding(sem_solver *s, int rounding);

/* Tile shape of the stencil pass (SEM_TILE_*; default SEM_TILE_AUTO).  Extension. */
int sem_solver_set_tile_shape(sem_solver *s, int shape);

/* The shape the solver's stencil tables were built with (SEM_TILE_DEFAULT or SEM_TILE_SQUARE);
   SEM_TILE_AUTO before the first stencil step builds them. */
int sem_solver_get_tile_shape(const sem_solver *s, int *shape);

/* Sponge of `thickness` elements with boundary damping sigma (0 thickness: none), or explicit
 * per-axis factors (see sem_box_sponge_profile).  Applied after each step to both levels. */
int sem_solver_set_sponge(sem_solver *s, int thickness, float sigma);
int sem_solver_set_sponge_profile(sem_solver *s, const float *sx, const float *sy,
                                  const float *sz);

/* Point sources on local node 0 of the given elements, wavelet[n_src][n_samples]; the step n
 * adds dt^2 c_e^2 wavelet[k][n] to the current level at that node (SEMsolver.cpp:39-43,
 * SEMproxy.cpp:93-119).  _points locates elements from coordinates like
 * sem_box_element_from_point. */
int sem_solver_set_sources(sem_solver *s, int n_src, const int64_t *elements,
                           const float *wavelet, int n_samples);
int sem_solver_set_source_points(sem_solver *s, int n_src, const float *xyz,
                                 const float *wavelet, int n_samples);

/* Receivers: sample the new pressure level at these nodes after every step.  The reference
 * only prints the source node every 100 steps (SEMsolver.cpp:127-142).  _points snaps
 * positions with sem_box_nearest_node. */
int sem_solver_set_receiver_nodes(sem_solver *s, int n_rec, const int64_t *nodes);
int sem_solver_set_receivers(sem_solver *s, int n_rec, const float *xyz);

/* Enqueue n_steps of SEMsolver::computeOneStep followed by the level swap of SEMproxy::run
 * (SEMsolver.cpp:21-125, SEMproxy.cpp:45-55), plus sponge and receiver sampling.  The time
 * loop is replayed from a captured CUDA graph. */
int sem_solver_step(sem_solver *s, int n_steps);

/* Streaming form of the same loop with host buffers: copies this chunk's wavelet samples
 * (host [n_steps][n_src], replacing the stored wavelet for these steps) to the device, runs
 * n_steps, and copies the chunk's receiver samples back (host [n_steps][n_rec]).  Either buffer
 * may be NULL.  Mirrors SEMproxy::run's per-step computeOneStep + outputPnValues. */
int sem_solver_step_host(sem_solver *s, int n_steps, const float *wavelet_samples,
                         float *traces_out);

/* Steps completed so far. */
int sem_solver_steps_done(const sem_solver *s, int64_t *n);

/* Receiver traces [n_steps_done][n_rec] (host), receiver order as given. */
int sem_solver_get_traces(sem_solver *s, float *out);

/* Read or overwrite one pressure level (n_nodes floats, reference node numbering).
 * SEM_LEVEL_PREVIOUS is the sponge-damped previous level that the next step uses, as the
 * reference holds it after its sponge pass; the device keeps it without the last sponge factor
 * and applies that factor when the level is read, so writing it divides the factor out (exact
 * to within one rounding). */
int sem_solver_get_pressure(sem_solver *s, int level, float *out);
int sem_solver_set_pressure(sem_solver *s, int level, const float *in);

/* Zero both levels, the traces and the step counter. */
int sem_solver_reset(sem_solver *s);

/* Wait for the solver's stream; returns SEM_ERR_UNSTABLE if any trace sample is non-finite. */
int sem_solver_synchronize(sem_solver *s);

/* Average device time per launch (ms) of the step's kernels over n_steps un-captured steps,
 * measured with CUDA events on the solver's stream: ms[0] source, ms[1] stiffness
 * (element kernel, or the fused stencil pass), ms[2] update (0 for the fused stencil pass).
 * Advances the solver by n_steps. */
int sem_solver_time_kernels(sem_solver *s, int n_steps, float *ms);

/* ------------------------------------------------------------------------------------------
 * Many shots on one mesh (batched form).  The reference runs one source per process
 * (SEMdata.hpp:13, SEMproxy.cpp:93-119); a batch advances n_shots independent shots that share
 * the mesh, the velocity model, the sponge and the receiver set.  The shots' fields lie one
 * after another and one stencil pass steps them all, the CTAs of every shot of a tile running
 * together so that the mesh-side data (dt^2/M, sponge) is read from memory once per tile for
 * the batch; each shot gets the same bits as a plain solver run of it in the default operator
 * form (SEM_FORM_DIRECT, the only form of the batch).  Same conventions as sem_solver_*.
 * ------------------------------------------------------------------------------------------ */

typedef struct sem_batch sem_batch;

int sem_batch_create(sem_mesh *mesh, float dt, int n_shots, sem_batch **out);
int sem_batch_destroy(sem_batch *b);
int sem_batch_set_stream(sem_batch *b, void *cuda_stream);
int sem_batch_set_sponge(sem_batch *b, int thickness, float sigma);
int sem_batch_set_sponge_profile(sem_batch *b, const float *sx, const float *sy, const float *sz);
/* One source per shot on local node 0 of elements[shot] (-1: no source for that shot), wavelet
 * [n_shots][n_samples]; as sem_solver_set_sources per shot. */
int sem_batch_set_sources(sem_batch *b, const int64_t *elements, const float *wavelet, int n_samples);
int sem_batch_set_source_points(sem_batch *b, const float *xyz, const float *wavelet, int n_samples);
/* One receiver set for all shots; traces are [steps][n_rec][n_shots]. */
int sem_batch_set_receiver_nodes(sem_batch *b, int n_rec, const int64_t *nodes);
int sem_batch_set_receivers(sem_batch *b, int n_rec, const float *xyz);
/* Enqueue n_steps for every shot (time loop replayed from a captured CUDA graph). */
int sem_batch_step(sem_batch *b, int n_steps);
int sem_batch_synchronize(sem_batch *b);
int sem_batch_get_traces(sem_batch *b, float *out);
int sem_batch_get_pressure(sem_batch *b, int shot, int level, float *out);
/* Time n_steps (CUDA events on the batch's stream); advances the batch. */
int sem_batch_time_step(sem_batch *b, int n_steps, float *ms_per_step);
/* Time the candidate launch shapes on the current state, keep the fastest, restore the state:
 * shots per thread-block cluster (the CTAs of that many consecutive shots of a tile start
 * together and share the mass tiles through L2; 1, 2, 4 or 8, dividing the shot count) by planes
 * per CTA along y.  warps_per_cta reports the pass's fixed CTA width.  Any output pointer may be
 * NULL. */
int sem_batch_autotune(sem_batch *b, int *shots_per_cluster, int *warps_per_cta, int *ychunk);

/* ------------------------------------------------------------------------------------------
 * Groups of independent problems of uneven size (different meshes, orders, models, dt).  The
 * reference runs one problem per process (SEMproxy.cpp:41-64); a group advances several
 * solvers together, replaying one CUDA graph per two steps.  Two launch forms:
 *   SEM_GROUP_ONE_LAUNCH (default): each step is one source launch and one stencil-pass launch
 *     whose CTAs cover every member's tiles, so small members fill the SMs that large ones
 *     leave idle within the launch.  Needs every member on the stencil pass with order <= 4,
 *     the direct form and the default rounding; otherwise the group uses the branches.
 *   SEM_GROUP_BRANCHES: each member's own launches as a parallel branch of the graph.
 * Members keep their own state and I/O (sem_solver_get_traces etc.) and give the same bits as
 * when stepped alone; they may be stepped alone between group steps.  A solver belongs to at
 * most one group at a time; the group must be destroyed before its members.
 * ------------------------------------------------------------------------------------------ */

typedef struct sem_group sem_group;
enum { SEM_GROUP_ONE_LAUNCH = 0, SEM_GROUP_BRANCHES = 1 };

int sem_group_create(int n_solvers, sem_solver *const *solvers, sem_group **out);
int sem_group_destroy(sem_group *g);
/* Requested launch form (SEM_GROUP_*), from the next step on. */
int sem_group_set_launch(sem_group *g, int form);
/* Launch form of the last step (before any step: the requested one). */
int sem_group_get_launch(sem_group *g, int *form);
/* Every member advances n_steps (enqueued; ordered after earlier work on the members' streams
 * and before later calls on them). */
int sem_group_step(sem_group *g, int n_steps);
/* Wait for the group; then sem_solver_synchronize on every member (status and finite traces). */
int sem_group_synchronize(sem_group *g);
/* Time n_steps of the whole group (CUDA events on the group stream); advances the members. */
int sem_group_time_step(sem_group *g, int n_steps, float *ms_per_step);

/* ------------------------------------------------------------------------------------------
 * Adjoint-state gradient.  The reference has no inversion path; this computes, for one shot,
 *     L = 1/2 sum_n sum_r (d_r^n - obs_r^n)^2
 * over the traces d of n_steps plain steps (SEMsolver.cpp:21-125 with the sponge and receivers
 * of sem_solver_*) and its gradient dL/dm with respect to the per-node squared slowness m
 * (mass M_i = m_i W_i; the mesh model may be element velocities or node slownesses).  The
 * forward levels are checkpointed every `checkpoint_every` steps on the device; the backward
 * sweep recomputes each segment and runs the adjoint steps (the same stencil pass, residuals
 * injected at the interior receiver nodes).  Source coefficients dt^2 c_e^2 are held fixed.
 * Device memory: (2 n_segments + checkpoint_every + 1) levels.
 * ------------------------------------------------------------------------------------------ */

typedef struct sem_adjoint sem_adjoint;

int sem_adjoint_create(sem_mesh *mesh, float dt, int n_steps, int checkpoint_every, sem_adjoint **out);
int sem_adjoint_destroy(sem_adjoint *a);
int sem_adjoint_set_sponge(sem_adjoint *a, int thickness, float sigma);
int sem_adjoint_set_sponge_profile(sem_adjoint *a, const float *sx, const float *sy, const float *sz);
/* As sem_solver_set_sources / sem_solver_set_source_points / sem_solver_set_receiver*. */
int sem_adjoint_set_sources(sem_adjoint *a, int n_src, const int64_t *elements, const float *wavelet, int n_samples);
int sem_adjoint_set_source_points(sem_adjoint *a, int n_src, const float *xyz, const float *wavelet, int n_samples);
int sem_adjoint_set_receiver_nodes(sem_adjoint *a, int n_rec, const int64_t *nodes);
int sem_adjoint_set_receivers(sem_adjoint *a, int n_rec, const float *xyz);
/* Forward run from rest with checkpoints; traces [n_steps][n_rec] (NULL: not copied out). */
int sem_adjoint_forward(sem_adjoint *a, float *traces);
/* Backward sweep for the residual d - obs ([n_steps][n_rec]); grad [n_nodes] (reference node
 * numbering) = dL/dm for L = 1/2 |residual|^2; NULL grad keeps it on the device. */
int sem_adjoint_backward(sem_adjoint *a, const float *residual, float *grad);
/* Residual from the last forward run and `observed` ([n_steps][n_rec]); loss and grad as above. */
int sem_adjoint_gradient(sem_adjoint *a, const float *observed, double *loss, float *grad);
/* Receivers of the adjoint run (for adjoint tests): after sem_adjoint_backward, traces
 * [n_steps][n_rec] of the adjoint field, row j holding step n = n_steps-1-j. */
int sem_adjoint_set_adjoint_receiver_nodes(sem_adjoint *a, int n_rec, const int64_t *nodes);
int sem_adjoint_get_adjoint_traces(sem_adjoint *a, float *out);

/* ------------------------------------------------------------------------------------------
 * Allocation-free step.  This entry point has no counterpart in the reference.
 * ------------------------------------------------------------------------------------------ */

/* One element-path step (K.p by the element kernel, then the leapfrog update) on buffers the
 * caller owns, for callers that cannot allocate device memory while they step -- a host code
 * that gives all device memory to its own pool manager, or one whose time loop runs where
 * allocation is not allowed.  The call allocates nothing: the K.p accumulator and a small
 * coefficient table live in a fixed array of 4,194,304 floats (16 MiB) in the library's device
 * image, so the mesh may have at most 4,194,176 nodes; larger meshes are rejected with
 * SEM_ERR_ARG.  All buffers are device memory in the reference node numbering:
 *   conn    int32 [n_elem][(order+1)^3] element-to-node map (as sem_mesh_get_connectivity gives);
 *           entries must lie in [0, n_nodes): one outside is skipped (read as 0, not scattered)
 *   p_cur   current level; sponge-damped in place when sponge factors are given
 *   p_prev  previous level (already damped); replaced by the new level
 *   coef    dt^2 / M_i per node
 *   sx, sy, sz  per-axis sponge factors (sem_box_sponge_profile), or all three NULL
 * Sources are the caller's: add them to p_cur before the call.  Work is enqueued on `stream`
 * (a cudaStream_t; NULL is the legacy default stream).  The first call on a device looks up
 * the array's device address (cudaGetSymbolAddress) and caches it, and loads the device code
 * of the kernels the step launches; under CUDA's lazy module loading that is when the driver
 * places the library's code and the 16 MiB array in device memory.  So make that first call
 * before the caller's pool manager reserves device memory, and before any stream capture; later
 * calls leave the device's free memory unchanged.  The cached address does not survive
 * cudaDeviceReset (nor does any other handle of this library).  Every call uses the same array,
 * which keeps the last call's contents (the call clears what it needs): calls whose work
 * overlaps on the GPU race on it. */
int sem_element_step_noalloc(int ex, int ey, int ez, float lx, float ly, float lz, int order,
                             const int32_t *conn, float *p_cur, float *p_prev, const float *coef,
                             const float *sx, const float *sy, const float *sz, void *stream);

/* ------------------------------------------------------------------------------------------
 * Learned absorbing boundary.  The reference has none (its only sponge is the FD proxy's,
 * FDTDinit.hpp:319-396).  A small network corrects, after every step, the new level on the
 * boundary nodes (layer_elems 0: the network gives the new face values, which the Dirichlet
 * update would hold fixed) or on the interior nodes within `layer_elems` elements of a face
 * (a correction added to the new level) -- the "strip" --
 * from p^{n+1}, p^n and
 * p^{n-1} on each node's 3x3x3 neighbourhood: 81 features divided by their largest magnitude,
 * two hidden layers of 64 with GELU, one output clipped to [-1, 1] and multiplied back by that
 * magnitude.  BF16 weights
 * and activations, FP32 accumulation on the tensor cores; FP32 master weights for training.
 * Parameter layout (sem_mlp_n_params floats): W1[64][81], b1[64], W2[64][64], b2[64], w3[64], b3.
 * ------------------------------------------------------------------------------------------ */

typedef struct sem_mlp sem_mlp;
typedef struct sem_abc sem_abc;

int sem_mlp_create(uint64_t seed, sem_mlp **out);
int sem_mlp_destroy(sem_mlp *net);
int sem_mlp_n_params(void);
int sem_mlp_set_params(sem_mlp *net, const float *params);
int sem_mlp_get_params(sem_mlp *net, float *params);
/* y[i] = net(x[i]), x [n][81] (host). */
int sem_mlp_forward(sem_mlp *net, int64_t n, const float *x, float *y);
/* Mean squared error over n samples and its gradient with respect to the parameters (host
 * arrays); the rounding to BF16 is passed through as the identity. */
int sem_mlp_loss_grad(sem_mlp *net, int64_t n, const float *x, const float *t, double *loss, float *grad);
/* Adam (beta 0.9 / 0.999) on minibatches of `batch` samples for `epochs` passes over the
 * samples (shuffled with `seed`); losses[epoch] = mean minibatch loss (may be NULL). */
int sem_mlp_train(sem_mlp *net, int64_t n, const float *x, const float *t, int epochs, int batch, float lr,
                  uint64_t seed, double *losses);
/* One Adam step of the network's parameters with a given gradient (host, parameter count). */
int sem_mlp_adam_step(sem_mlp *net, const float *grad, float lr);

/* Attach `net` to a solver (stencil pass) for the strip of `layer_elems` elements. */
int sem_abc_create(sem_solver *s, sem_mlp *net, int layer_elems, sem_abc **out);
int sem_abc_destroy(sem_abc *a);
/* Strip nodes and history nodes (strip plus its inner neighbour layer). */
int sem_abc_info(const sem_abc *a, int64_t *n_nodes, int64_t *n_history);
int sem_abc_nodes(const sem_abc *a, int64_t *nodes); /* reference numbering, [n_nodes] */
/* n_steps solver steps, each followed by the correction (enqueued on the solver's stream). */
int sem_abc_step(sem_abc *a, int n_steps);
/* The correction alone, for the step that just ran (as sem_abc_step applies it). */
int sem_abc_correct(sem_abc *a);
/* Zero the p^{n-1} history, or set it from a full level (n_nodes floats, actual values). */
int sem_abc_reset(sem_abc *a);
int sem_abc_set_history(sem_abc *a, const float *p_prev);
/* The network inputs of every strip node for the step that just ran: x [n_nodes][81] already
 * divided by scale [n_nodes] (may be NULL), as the correction kernel forms them. */
int sem_abc_features(sem_abc *a, float *x, float *scale);
/* Training through the adjoint of the whole time loop (network on the boundary nodes, layer 0).
 * Runs n_steps corrected steps from rest (the solver and the history are reset first) and
 * returns loss = sum over steps m = 1..n_steps and region nodes r of (p^m_r - ref[m-1][r])^2
 * (roi_nodes: reference numbering; ref: host [n_steps][n_roi]).  With grad non-NULL (host,
 * the network's parameter count) the gradient of the loss with respect to the network's
 * parameters is computed by the adjoint of every step, newest first: the network's own backward
 * kernels at the boundary nodes (through the division by the neighbourhood's largest magnitude
 * and the clipping) and the adjoint leapfrog of the stencil pass, from the recorded levels.
 * Sources must lie at least two nodes inside the box.  The solver is left after the n_steps.
 * Every level is recorded: (n_steps + 2) x (the mesh's device-layout node count) floats of
 * device memory, plus a few fields, for the duration of the call (meant for training regions;
 * SEM_ERR_OOM when it does not fit). */
int sem_abc_bptt(sem_abc *a, int n_steps, int n_roi, const int64_t *roi_nodes, const float *ref, double *loss,
                 float *grad);

/* ------------------------------------------------------------------------------------------
 * Output formats.  One container for traces and snapshots: 8-byte magic, little-endian uint64
 * header length, UTF-8 JSON header, zero padding to a 64-byte boundary, little-endian float32
 * samples.  Traces ("SEMTRC01") are stored trace-major (SEG-Y's order: each receiver's whole
 * series in turn) with dt, receiver and source coordinates and optional caller JSON; the
 * in-memory arrays stay [n_steps][n_rec] as sem_solver_get_traces gives them.  Snapshots
 * ("SEMSNP01") hold one x-z plane of a pressure level, rows of x for increasing z, with the node
 * coordinates; they replace the ASCII slice of SEMmesh::saveSnapShot (SEMmesh.cpp:624-654).
 * ------------------------------------------------------------------------------------------ */

int sem_traces_write(const char *path, int n_steps, int n_rec, const float *traces, float dt,
                     const float *rec_xyz, int n_src, const float *src_xyz, const char *extra_json);
int sem_traces_read_info(const char *path, int *n_steps, int *n_rec, float *dt);
int sem_traces_read(const char *path, float *traces);
/* Plane y = y_index (-1: ny/2 - 1, the reference's plane) of a level of the solver. */
int sem_solver_write_snapshot(sem_solver *s, int level, int y_index, const char *path);
int sem_snapshot_read_info(const char *path, int *nx, int *nz, int *y_index);
int sem_snapshot_read(const char *path, float *plane);

#ifdef __cplusplus
}
#endif
#endif /* SEMGB_H_ */
