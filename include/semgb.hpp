// semgb.hpp -- C++ face of libsemgb shaped like the reference's SEM solver classes.
//
// Header-only, on top of the C ABI in semgb.h.  C++ exceptions are thrown here, on the caller's
// side of the boundary; nothing crosses the C ABI but status codes.
//
//   semgb::Mesh         SEMmesh (SEMmesh.hpp:23-116): a structured box of GLL hexahedra
//   semgb::Solver       RAII over sem_solver: device-resident levels, sources, receivers
//   semgb::SEMsolverGB  SEMsolver (SEMsolver.hpp:18-92): computeFEInit / computeOneStep /
//                       outputPnValues with the reference's argument lists, for callers written
//                       against SEMsolver (SEMproxy.cpp:25-64)
#ifndef SEMGB_HPP_
#define SEMGB_HPP_

#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "semgb.h"

namespace semgb {

class Error : public std::runtime_error {
public:
    Error(int code, const std::string &what) : std::runtime_error(what), code_(code) {}
    int code() const { return code_; }

private:
    int code_;
};

inline void check(int rc, const char *where)
{
    if (rc != SEM_OK) throw Error(rc, std::string(where) + ": " + sem_last_error_string());
}

class Mesh {
public:
    Mesh(int ex, int ey, int ez, float lx, float ly, float lz, int order)
        : ex_(ex), ey_(ey), ez_(ez), order_(order), lx_(lx), ly_(ly), lz_(lz)
    {
        check(sem_mesh_create_box(ex, ey, ez, lx, ly, lz, order, &h_), "sem_mesh_create_box");
        check(sem_mesh_info(h_, &n_nodes_, &n_elem_, &npe_, &n_interior_), "sem_mesh_info");
    }
    ~Mesh() { sem_mesh_destroy(h_); }
    Mesh(const Mesh &) = delete;
    Mesh &operator=(const Mesh &) = delete;

    sem_mesh *handle() const { return h_; }
    int64_t numberOfNodes() const { return n_nodes_; }                 // SEMmesh::getNumberOfNodes
    int64_t numberOfElements() const { return n_elem_; }               // SEMmesh::getNumberOfElements
    int numberOfPointsPerElement() const { return npe_; }              // ...getNumberOfPointsPerElement
    int64_t numberOfInteriorNodes() const { return n_interior_; }      // ...getNumberOfInteriorNodes
    int order() const { return order_; }

    // SEMmesh::getElementNumberFromPoints (SEMmesh.cpp:266-285)
    int64_t elementFromPoint(float x, float y, float z) const
    {
        int64_t e = 0;
        check(sem_box_element_from_point(ex_, ey_, ez_, lx_, ly_, lz_, x, y, z, &e), "element_from_point");
        return e;
    }
    // SEMmesh::globalNodesList (SEMmesh.cpp:205-231), from the device copy
    std::vector<int32_t> connectivity() const
    {
        std::vector<int32_t> c((size_t)n_elem_ * npe_);
        check(sem_mesh_get_connectivity(h_, c.data()), "sem_mesh_get_connectivity");
        return c;
    }
    // SEMmesh::getModel (SEMmesh.cpp:288-312): per-element velocity
    void setVelocity(const std::vector<float> &c)
    {
        if ((int64_t)c.size() != n_elem_) throw Error(SEM_ERR_ARG, "velocity size != number of elements");
        check(sem_model_set_element_velocity(h_, c.data()), "sem_model_set_element_velocity");
    }

private:
    sem_mesh *h_ = nullptr;
    int ex_, ey_, ez_, order_;
    float lx_, ly_, lz_;
    int64_t n_nodes_ = 0, n_elem_ = 0, n_interior_ = 0;
    int npe_ = 0;
};

class Solver {
public:
    Solver(Mesh &mesh, float dt) : mesh_(&mesh) { check(sem_solver_create(mesh.handle(), dt, &h_), "sem_solver_create"); }
    ~Solver() { sem_solver_destroy(h_); }
    Solver(const Solver &) = delete;
    Solver &operator=(const Solver &) = delete;

    sem_solver *handle() const { return h_; }
    void setKernel(int k) { check(sem_solver_set_kernel(h_, k), "sem_solver_set_kernel"); }
    void setOperatorForm(int f) { check(sem_solver_set_operator_form(h_, f), "sem_solver_set_operator_form"); }
    void setRounding(int r) { check(sem_solver_set_rounding(h_, r), "sem_solver_set_rounding"); }
    void setTileShape(int shape) { check(sem_solver_set_tile_shape(h_, shape), "sem_solver_set_tile_shape"); }
    int tileShape() const
    {
        int shape = SEM_TILE_AUTO;
        check(sem_solver_get_tile_shape(h_, &shape), "sem_solver_get_tile_shape");
        return shape;
    }
    void setSponge(int thickness, float sigma) { check(sem_solver_set_sponge(h_, thickness, sigma), "sem_solver_set_sponge"); }
    void setSources(const std::vector<int64_t> &elements, const std::vector<float> &wavelet, int nsamples)
    {
        check(sem_solver_set_sources(h_, (int)elements.size(), elements.data(), wavelet.data(), nsamples),
              "sem_solver_set_sources");
    }
    void setReceiverNodes(const std::vector<int64_t> &nodes)
    {
        check(sem_solver_set_receiver_nodes(h_, (int)nodes.size(), nodes.data()), "sem_solver_set_receiver_nodes");
        nrec_ = (int)nodes.size();
    }
    void step(int n) { check(sem_solver_step(h_, n), "sem_solver_step"); }
    void synchronize() { check(sem_solver_synchronize(h_), "sem_solver_synchronize"); }
    int64_t stepsDone() const
    {
        int64_t n = 0;
        check(sem_solver_steps_done(h_, &n), "sem_solver_steps_done");
        return n;
    }
    std::vector<float> pressure(int level) const
    {
        std::vector<float> p((size_t)mesh_->numberOfNodes());
        check(sem_solver_get_pressure(h_, level, p.data()), "sem_solver_get_pressure");
        return p;
    }
    void setPressure(int level, const std::vector<float> &p) { check(sem_solver_set_pressure(h_, level, p.data()), "sem_solver_set_pressure"); }
    std::vector<float> traces() const
    {
        std::vector<float> t((size_t)stepsDone() * nrec_);
        if (!t.empty()) check(sem_solver_get_traces(h_, t.data()), "sem_solver_get_traces");
        return t;
    }

private:
    Mesh *mesh_;
    sem_solver *h_ = nullptr;
    int nrec_ = 0;
};

// SEMsolver-shaped adapter (SEMsolver.hpp:18-92).  Info is the caller's SEMinfo (fields
// myTimeStep, myNumberOfRHS, myNumSamples, myElementSource are read); Array2D/Vector are the
// caller's containers with operator()(row, col) / operator[] (dataType.hpp:14-80).
//
// The pressure levels live on the GPU.  computeOneStep advances them there: the host
// pnGlobal container is read on the first call (the initial state) and written back only by
// syncPressure() or, for the printed node, by outputPnValues -- copying two full levels every
// step would cost more than the step.
class SEMsolverGB {
public:
    // SEMsolver::computeFEInit(SEMinfo&, SEMmesh) (SEMsolver.cpp:12-17): the box, its order and
    // the element velocities (SEMmesh::getModel gives 1500 m/s everywhere).
    template <class Info>
    void computeFEInit(Info &info, int ex, int ey, int ez, float lx, float ly, float lz, int order,
                       const std::vector<float> *velocity = nullptr)
    {
        mesh_.reset(new Mesh(ex, ey, ez, lx, ly, lz, order));
        if (velocity) mesh_->setVelocity(*velocity);
        solver_.reset(new Solver(*mesh_, info.myTimeStep));
        primed_ = false;
        conn_ = mesh_->connectivity();
        npe_ = mesh_->numberOfPointsPerElement();
    }

    // SEMsolver::computeOneStep (SEMsolver.cpp:21-125) with the reference's arguments.  The
    // sources come from RHSTerm / rhsElement (uploaded on the first call); i1/i2 select which
    // host column holds the previous / current level on that first call.
    template <class Info, class Array2D, class VectorInt>
    void computeOneStep(int timeSample, int order, int nPointsPerElement, int i1, int i2, Info &info,
                        const Array2D &RHSTerm, const Array2D &pnGlobal, const VectorInt &rhsElement)
    {
        (void)order;
        (void)nPointsPerElement;
        if (!primed_) {
            const int64_t n = mesh_->numberOfNodes();
            std::vector<float> cur((size_t)n), prev((size_t)n);
            for (int64_t i = 0; i < n; i++) {
                cur[i] = pnGlobal((int)i, i2);
                prev[i] = pnGlobal((int)i, i1);
            }
            solver_->setPressure(SEM_LEVEL_CURRENT, cur);
            solver_->setPressure(SEM_LEVEL_PREVIOUS, prev);
            // the device counts steps from this first call: store the wavelet from timeSample on
            const int ns = info.myNumSamples > timeSample ? info.myNumSamples - timeSample : 0;
            std::vector<int64_t> el(info.myNumberOfRHS);
            std::vector<float> wav((size_t)info.myNumberOfRHS * ns);
            for (int k = 0; k < info.myNumberOfRHS; k++) {
                el[k] = rhsElement[k];
                for (int s = 0; s < ns; s++) wav[(size_t)k * ns + s] = RHSTerm(k, timeSample + s);
            }
            solver_->setSources(el, wav, ns);
            primed_ = true;
        }
        solver_->step(1);
    }

    // SEMsolver::outputPnValues (SEMsolver.cpp:127-142): every 100 steps, print p^{n+1} at
    // local node 0 of the source element.
    template <class Array2D>
    void outputPnValues(int indexTimeStep, int &i1, int &myElementSource, const Array2D &pnGlobal)
    {
        (void)i1;
        (void)pnGlobal;
        if (indexTimeStep % 100 == 0) {
            const std::vector<float> p = solver_->pressure(SEM_LEVEL_CURRENT);
            const int node = conn_[(size_t)myElementSource * npe_];
            std::printf("TimeStep=%d;  pnGlobal @ elementSource location %d after computeOneStep = %g\n",
                        indexTimeStep, myElementSource, (double)p[node]);
        }
    }

    // Copy both device levels into the caller's container (column i2 = newest level after the
    // caller's swap, as SEMproxy::run leaves them).
    template <class Array2D>
    void syncPressure(Array2D &pnGlobal, int i1, int i2) const
    {
        const std::vector<float> cur = solver_->pressure(SEM_LEVEL_CURRENT);
        const std::vector<float> prev = solver_->pressure(SEM_LEVEL_PREVIOUS);
        for (size_t i = 0; i < cur.size(); i++) {
            pnGlobal((int)i, i2) = cur[i];
            pnGlobal((int)i, i1) = prev[i];
        }
    }

    Mesh &mesh() { return *mesh_; }
    Solver &solver() { return *solver_; }

private:
    struct MeshHolder {
        Mesh *p = nullptr;
        ~MeshHolder() { delete p; }
        void reset(Mesh *m) { delete p; p = m; }
        Mesh &operator*() const { return *p; }
        Mesh *operator->() const { return p; }
    };
    struct SolverHolder {
        Solver *p = nullptr;
        ~SolverHolder() { delete p; }
        void reset(Solver *s) { delete p; p = s; }
        Solver &operator*() const { return *p; }
        Solver *operator->() const { return p; }
    };
    // declaration order matters: the solver must be destroyed before its mesh
    MeshHolder mesh_;
    SolverHolder solver_;
    std::vector<int32_t> conn_;
    int npe_ = 0;
    bool primed_ = false;
};

}  // namespace semgb

#endif  // SEMGB_HPP_
