// sem_proxy.cpp -- the reference's SEM driver (main.cpp + SEMproxy.cpp) written against the
// SEMsolver-shaped C++ face of libsemgb (include/semgb.hpp).
//
//   sem_proxy [ex] [lx] [steps]     defaults: 100 elements per axis, 2000 m, 9 steps
//
// As in SEMproxy: a cube of ex^3 elements of order 2, one Ricker source (first-derivative form,
// f0 = 10 Hz, dt = 1 ms) in the element containing (1001, 1001, 1001), both pressure levels
// zero at start, the source-node value printed every 100 steps, kernel time reported.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "semgb.hpp"

namespace {

struct Info {  // the fields of SEMinfo (SEMdata.hpp:3-30) the solver reads
    int myNumberOfRHS = 1;
    float myTimeStep = 0.001f;
    float f0 = 10.f;
    int sourceOrder = 1;
    int myNumSamples = 9;
    int myElementSource = 0;
};

struct Array2D {  // dataType.hpp:42-55 shape: operator()(row, col)
    int cols;
    std::vector<float> v;
    Array2D(int r, int c) : cols(c), v((size_t)r * c, 0.f) {}
    float &operator()(int r, int c) { return v[(size_t)r * cols + c]; }
    float operator()(int r, int c) const { return v[(size_t)r * cols + c]; }
};

}  // namespace

int main(int argc, char **argv)
{
    const int ex = argc > 1 ? std::atoi(argv[1]) : 100;
    const float lx = argc > 2 ? (float)std::atof(argv[2]) : 2000.f;
    Info info;
    if (argc > 3) info.myNumSamples = std::atoi(argv[3]);
    const int order = 2;
    try {
        semgb::SEMsolverGB solver;
        solver.computeFEInit(info, ex, ex, ex, lx, lx, lx, order);
        semgb::Mesh &mesh = solver.mesh();
        // SEMproxy::init_source (SEMproxy.cpp:93-119)
        Array2D rhs(1, info.myNumSamples);
        std::vector<float> w(info.myNumSamples);
        semgb::check(sem_ricker(info.myNumSamples, info.myTimeStep, info.f0, info.sourceOrder, w.data()), "sem_ricker");
        for (int j = 0; j < info.myNumSamples; j++) rhs(0, j) = w[j];
        std::vector<int> rhsElement{(int)mesh.elementFromPoint(1001.f, 1001.f, 1001.f)};
        info.myElementSource = rhsElement[0];
        std::printf("nodes %lld, elements %lld, source element %d\n", (long long)mesh.numberOfNodes(),
                    (long long)mesh.numberOfElements(), info.myElementSource);
        Array2D pnGlobal((int)mesh.numberOfNodes(), 2);
        int i1 = 0, i2 = 1;
        // SEMproxy::run (SEMproxy.cpp:41-64)
        double kernel_s = 0;
        for (int n = 0; n < info.myNumSamples; n++) {
            const auto t0 = std::chrono::steady_clock::now();
            solver.computeOneStep(n, order, mesh.numberOfPointsPerElement(), i1, i2, info, rhs, pnGlobal, rhsElement);
            solver.solver().synchronize();
            kernel_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            solver.outputPnValues(n, i1, info.myElementSource, pnGlobal);
            std::swap(i1, i2);
        }
        std::printf("---- Elapsed Kernel Time : %g seconds.\n", kernel_s);
    } catch (const semgb::Error &e) {
        std::fprintf(stderr, "sem_proxy: %s\n", e.what());
        return 1;
    }
    return 0;
}
