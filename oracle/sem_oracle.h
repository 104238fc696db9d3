/*
 * sem_oracle.h -- CPU restatement of the reference spectral-element (SEM) acoustic step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: tests/, __graft_entry__.smoke() and
 * the CPU-baseline leg of bench.py load it to produce expected values or a CPU timing.  The
 * product (libsemgb) never links, loads or calls it.
 *
 * The arithmetic follows the reference operation by operation (same float/double types, same
 * evaluation order), so that, compiled with -ffp-contract=off, the float variant reproduces the
 * compiled reference bit for bit when it is given the reference's GLL tables.  Each function
 * names the reference lines it restates (paths inside numpex/proxy-geos-hc).
 */
#ifndef SEM_ORACLE_H_
#define SEM_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- mesh indexing (structured hex box; reference axis order: x fastest, then z, then y) ---- */

/* Node/element/interior counts.  SEMmesh.cpp:28-54 (int there; int64 here). */
void or_box_counts(int ex, int ey, int ez, int order,
                   int64_t *n_nodes, int64_t *n_elem, int64_t *n_interior);

/* Element-to-global-node map, row-major [n_elem][(order+1)^3].  SEMmesh.cpp:205-231. */
void or_connectivity(int ex, int ey, int ez, int order, int32_t *conn);

/* Interior node list (every face Dirichlet).  SEMmesh.cpp:314-344. */
void or_interior_nodes(int ex, int ey, int ez, int order, int32_t *list);

/* Element containing (x,y,z) by per-axis linear scan; 0 on an axis when outside.
 * SEMmesh.cpp:266-285. */
int64_t or_element_from_point(int ex, int ey, int ez, float lx, float ly, float lz,
                              float x, float y, float z);

/* Global node nearest to (x,y,z): per axis, the GLL node (exact double coordinates) closest to
 * the coordinate, ties to the lower index; coordinates outside the box clamp to its faces.
 * (The reference has no receivers; this is the build's snapping rule.) */
int64_t or_nearest_node(int ex, int ey, int ez, float lx, float ly, float lz, int order,
                        float x, float y, float z);

/* Per-element GLL node coordinates (float), arrays [n_elem][(order+1)^3] for the x, z and y
 * axes.  getCoordInOneDirection takes the element size as an int (SEMmesh.cpp:81-139), which
 * this restates.  SEMmesh.cpp:168-202. */
void or_element_coords(int ex, int ey, int ez, float lx, float ly, float lz, int order,
                       float *X, float *Z, float *Y);

/* ---- GLL tables (own derivation; compared against the reference's literals in tests) ----
 * xi[o+1], w[o+1] (rounded to 8 decimals exactly as the reference's table),
 * dphi[(o+1)*(o+1)] with dphi[j*(o+1)+i] = phi_j'(xi_i).
 * SEMQkGLBasisFunctions.hpp:36-117 (points, weights), :178-324 (derivatives). */
int or_gll_tables(int order, double *xi, double *w, double *dphi);

/* ---- Ricker source ---- utils.hpp:11-57 */
float or_ricker(float t, float f0, int order);
void or_source_term(int n, float dt, float f0, int order, float *out);

/* ---- sponge profile: the build's definition (the reference SEM has no sponge; this follows the
 * Gaussian taper of the FD proxy, FDTDinit.hpp:319-396, scaled to `thickness` elements).
 * For a node at physical coordinate c along an axis of length L split into n elements of
 * size h:  d = min(c, L - c) / h  (in elements);  s = exp(-sigma * ((thickness - d)/thickness)^2)
 * when d < thickness, else 1.  Node coordinates use the exact GLL points.
 * Outputs one factor per node index along each axis: sx[nx], sy[ny], sz[nz] (float and double).
 * The per-node factor is (sx[ix] * sy[iy]) * sz[iz]. */
void or_sponge_profile(int ex, int ey, int ez, float lx, float ly, float lz, int order,
                       int thickness, float sigma,
                       float *sx, float *sy, float *sz,
                       double *sxd, double *syd, double *szd);

/* ---- time stepping ---- */
typedef struct or_config {
    int ex, ey, ez, order;
    float lx, ly, lz;
    float dt;
    int nsteps;           /* steps to run */
    int step0;            /* time-sample index of the first step (wavelet index) */
    const double *xi, *w, *dphi;   /* GLL tables (reference's own or or_gll_tables) */
    const float *vel;     /* per-element velocity, n_elem entries */
    int nsrc;
    const int64_t *src_elem;   /* source element per source; source sits on local node 0 */
    const float *wavelet;      /* [nsrc][nsamples] */
    int nsamples;
    const void *sx, *sy, *sz;  /* sponge factors per axis (REAL typed) or NULL for none */
    int nrec;
    const int64_t *rec_node;   /* receiver node indices */
    int nthreads;              /* 1: element order of the reference; >1: 8-colour OpenMP loop */
} or_config;

/* Run cfg->nsteps steps of SEMsolver::computeOneStep (SEMsolver.cpp:21-125) followed by the
 * build's sponge on both levels and receiver sampling of the new level, then the level swap of
 * SEMproxy::run (SEMproxy.cpp:45-55).  p_cur/p_prev are in/out (n_nodes each): on return p_cur
 * holds the newest level.  traces is [nsteps][nrec] (may be NULL when nrec == 0).
 * _f32: the reference's float arithmetic; _f64: the same scheme in double.
 * Returns 0, or a negative value on bad arguments. */
int or_run_f32(const or_config *cfg, float *p_cur, float *p_prev, float *traces);
int or_run_f64(const or_config *cfg, double *p_cur, double *p_prev, double *traces);

/* One element's local mass vector and stiffness product (SEMQkGLIntegrals.hpp:547-565, V2),
 * for element-level parity checks.  p_local, M_local, Y are (order+1)^3. */
void or_element_apply_f32(const or_config *cfg, int64_t e, const float *p_local,
                          float *M_local, float *Y);

#ifdef __cplusplus
}
#endif
#endif
