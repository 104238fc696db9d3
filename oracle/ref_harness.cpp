// ref_harness.cpp -- drives the reference's own SEM classes (compiled from the reference's
// sources where they lie) behind a C interface, so that tests can pin the oracle restatement
// and generate golden fixtures.  TEST INFRASTRUCTURE ONLY: built by oracle/build_ref.sh into
// oracle/_ref/ and never linked into the product.
//
// The harness calls SEMsolver::computeFEInit / computeOneStep exactly as SEMproxy does
// (SEMproxy.cpp:25-55) and adds, after every step, what the reference lacks: the build's sponge
// on both pressure levels and receiver sampling of the new level.  The per-element velocity
// model and the run constants are supplied by the caller (the reference hard-codes them:
// SEMmesh.cpp:288-312, SEMdata.hpp:13-22).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>
#include <algorithm>

// The solver keeps its model and FE arrays private (SEMsolver.hpp:55-92); the harness needs to
// set the model and read the tables, so the class is compiled into this unit with public access.
#define private public
#include "SEMsolver.cpp"
#undef private
#include "utils.hpp"

#include "sem_oracle.h"

namespace {
struct Quiet {  // the reference prints progress on std::cout; keep test output readable
    std::streambuf *old;
    std::ostringstream sink;
    Quiet() : old(std::cout.rdbuf(sink.rdbuf())) {}
    ~Quiet() { std::cout.rdbuf(old); }
};
}  // namespace

extern "C" {

int semref_order(void) { return SEMinfo::myOrderNumber; }

int semref_tables(double *xi, double *w, double *dphi)
{
    const int o = SEMinfo::myOrderNumber, o1 = o + 1;
    SEMQkGLBasisFunctions basis;
    vectorDouble q(o1), ww(o1);
    arrayDouble d(o1, o1);
    basis.gaussLobattoQuadraturePoints(o, q);
    basis.gaussLobattoQuadratureWeights(o, ww);
    basis.getDerivativeBasisFunction1D(o, q, d);
    for (int i = 0; i < o1; i++) { xi[i] = q[i]; w[i] = ww[i]; }
    for (int j = 0; j < o1; j++)
        for (int i = 0; i < o1; i++) dphi[j * o1 + i] = d(j, i);
    return 0;
}

void semref_source_term(int n, float dt, float f0, int order, float *out)
{
    SolverUtils u;
    std::vector<float> s = u.computeSourceTerm(n, dt, f0, order);
    for (int i = 0; i < n; i++) out[i] = s[i];
}

int semref_mesh(int ex, int ey, int ez, float lx, float ly, float lz,
                int64_t *counts /* nodes, elements, interior */, int32_t *conn, int32_t *interior,
                float *X, float *Z, float *Y)
{
    Quiet q;
    const int o = SEMinfo::myOrderNumber;
    SEMmesh mesh(ex, ey, ez, lx, ly, lz, o);
    const int N = mesh.getNumberOfNodes(), NE = mesh.getNumberOfElements();
    const int npe = mesh.getNumberOfPointsPerElement(), NI = mesh.getNumberOfInteriorNodes();
    if (counts) { counts[0] = N; counts[1] = NE; counts[2] = NI; }
    if (conn) {
        arrayInt c(NE, npe);
        mesh.globalNodesList(NE, c);
        for (int e = 0; e < NE; e++)
            for (int i = 0; i < npe; i++) conn[(int64_t)e * npe + i] = c(e, i);
    }
    if (interior) {
        vectorInt l(NI);
        mesh.getListOfInteriorNodes(NI, l);
        for (int i = 0; i < NI; i++) interior[i] = l[i];
    }
    if (X && Y && Z) {
        arrayReal cx(NE, npe), cy(NE, npe), cz(NE, npe);
        mesh.nodesCoordinates(cx, cz, cy);
        for (int e = 0; e < NE; e++)
            for (int i = 0; i < npe; i++) {
                X[(int64_t)e * npe + i] = cx(e, i);
                Y[(int64_t)e * npe + i] = cy(e, i);
                Z[(int64_t)e * npe + i] = cz(e, i);
            }
    }
    return 0;
}

int64_t semref_element_from_point(int ex, int ey, int ez, float lx, float ly, float lz,
                                  float x, float y, float z)
{
    Quiet q;
    SEMmesh mesh(ex, ey, ez, lx, ly, lz, SEMinfo::myOrderNumber);
    return mesh.getElementNumberFromPoints(x, y, z);
}

static SEMinfo make_info(SEMmesh &mesh, int nrhs, float dt, int nsamples)
{
    SEMinfo info{.numberOfNodes = mesh.getNumberOfNodes(),
                 .numberOfElements = mesh.getNumberOfElements(),
                 .numberOfPointsPerElement = mesh.getNumberOfPointsPerElement(),
                 .numberOfInteriorNodes = mesh.getNumberOfInteriorNodes(),
                 .numberOfBoundaryNodes = mesh.getNumberOfBoundaryNodes(),
                 .numberOfBoundaryFaces = mesh.getNumberOfBoundaryFaces(),
                 .myNumberOfRHS = nrhs,
                 .myTimeStep = dt,
                 .myNumSamples = nsamples};
    return info;
}

int semref_element_apply(const or_config *c, int64_t e, const float *p_local, float *M_local,
                         float *Yout)
{
    if (c->order != SEMinfo::myOrderNumber) return -10;
    Quiet q;
    SEMmesh mesh(c->ex, c->ey, c->ez, c->lx, c->ly, c->lz, c->order);
    SEMinfo info = make_info(mesh, 1, c->dt, 1);
    SEMsolver solver;
    solver.computeFEInit(info, mesh);
    const int npe = info.numberOfPointsPerElement;
    float pl[ROW], Ml[ROW], Y[ROW];
    for (int i = 0; i < npe; i++) pl[i] = p_local[i];
    solver.myQkIntegrals.computeMassMatrixAndStiffnessVector(
        (int)e, c->order, npe, solver.globalNodesCoordsX, solver.globalNodesCoordsY,
        solver.globalNodesCoordsZ, solver.weights, solver.derivativeBasisFunction1D, Ml, pl, Y);
    for (int i = 0; i < npe; i++) { M_local[i] = Ml[i]; Yout[i] = Y[i]; }
    return 0;
}

int semref_run(const or_config *c, float *p_cur, float *p_prev, float *traces)
{
    if (c->order != SEMinfo::myOrderNumber) return -10;
    Quiet q;
    SEMmesh mesh(c->ex, c->ey, c->ez, c->lx, c->ly, c->lz, c->order);
    const int nsamp = std::max(c->nsamples, c->step0 + c->nsteps);
    SEMinfo info = make_info(mesh, c->nsrc, c->dt, nsamp);
    SEMsolver solver;
    solver.computeFEInit(info, mesh);
    const int N = info.numberOfNodes, NE = info.numberOfElements;
    const int npe = info.numberOfPointsPerElement;
    if (c->vel)
        for (int e = 0; e < NE; e++) solver.model[e] = c->vel[e];

    arrayReal rhs(std::max(c->nsrc, 1), nsamp);
    vectorInt rhsElement(std::max(c->nsrc, 1));
    for (int k = 0; k < c->nsrc; k++) {
        rhsElement[k] = (int)c->src_elem[k];
        for (int n = 0; n < c->nsamples; n++) rhs(k, n) = c->wavelet[(int64_t)k * c->nsamples + n];
    }
    arrayReal pn(N, 2);
    int i1 = 0, i2 = 1;  // SEMproxy.hpp:58-59
    for (int I = 0; I < N; I++) { pn(I, i2) = p_cur[I]; pn(I, i1) = p_prev[I]; }

    const int nx = c->ex * c->order + 1, nz = c->ez * c->order + 1;
    const float *sx = (const float *)c->sx, *sy = (const float *)c->sy, *sz = (const float *)c->sz;
    for (int s = 0; s < c->nsteps; s++) {
        solver.computeOneStep(c->step0 + s, c->order, npe, i1, i2, info, rhs, pn, rhsElement);
        if (sx && sy && sz) {
            for (int I = 0; I < N; I++) {
                int iy = I / (nx * nz), r = I - iy * nx * nz, iz = r / nx, ix = r - iz * nx;
                float f = sx[ix] * sy[iy] * sz[iz];
                pn(I, i1) = f * pn(I, i1);
                pn(I, i2) = f * pn(I, i2);
            }
        }
        for (int r = 0; r < c->nrec; r++) traces[(int64_t)s * c->nrec + r] = pn((int)c->rec_node[r], i1);
        std::swap(i1, i2);  // SEMproxy.cpp:53
    }
    for (int I = 0; I < N; I++) { p_cur[I] = pn(I, i2); p_prev[I] = pn(I, i1); }
    (void)npe;
    return 0;
}

}  // extern "C"
