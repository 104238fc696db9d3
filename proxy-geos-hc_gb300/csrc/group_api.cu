// group_api.cu -- many independent problems of uneven size advanced together (sem_group_*).
//
// Each member is an ordinary solver (its own mesh, order, model, dt, sources and receivers).
// The group captures one CUDA graph per two steps with one branch per member: the group stream
// forks into the members' streams, each branch holds that member's two steps (source, stencil
// pass with update and receivers), and the branches join back.  A launch of the graph hands all
// members' kernels to the GPU at once, so small problems fill the SMs that large ones leave idle
// and the host issues one launch per two steps for the whole group.  Branches are captured
// largest member first.
#include <cuda_runtime.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "abi.h"
#include "solver.h"

struct sem_group {
    std::vector<sem_solver *> members;  // capture order: largest first
    cudaStream_t stream = nullptr;
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> join;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};  // [0]: levels as at capture, [1]: after an odd step
    std::vector<uint64_t> gen;                      // members' graph generations at capture
    int flip = 0;                                   // parity of the members' levels against the capture
};

namespace {

void drop_graphs(sem_group *g)
{
    for (auto &x : g->graph)
        if (x) { cudaGraphExecDestroy(x); x = nullptr; }
    g->gen.clear();
    g->flip = 0;
}

bool stale(const sem_group *g)
{
    if (g->gen.size() != g->members.size()) return true;
    for (size_t i = 0; i < g->members.size(); i++)
        if (g->members[i]->graph_gen != g->gen[i]) return true;
    return false;
}

// Fork the members from the group stream, enqueue `steps` steps on each, join them back.
cudaError_t enqueue_all(sem_group *g, int steps)
{
    cudaError_t e = cudaEventRecord(g->fork, g->stream);
    if (e != cudaSuccess) return e;
    for (size_t i = 0; i < g->members.size(); i++) {
        sem_solver *s = g->members[i];
        if ((e = cudaStreamWaitEvent(s->stream, g->fork, 0)) != cudaSuccess) return e;
        int c = s->cur;
        for (int k = 0; k < steps; k++, c ^= 1)
            if ((e = solver_enqueue_step(s, c)) != cudaSuccess) return e;
        if ((e = cudaEventRecord(g->join[i], s->stream)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(g->stream, g->join[i], 0)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

int capture(sem_group *g, int which)
{
    cudaGraph_t graph = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e1 = enqueue_all(g, 2);
    cudaError_t e2 = cudaStreamEndCapture(g->stream, &graph);
    if (e1 != cudaSuccess || e2 != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return sem_fail(SEM_ERR_CUDA, std::string("group graph capture: ") +
                                          cudaGetErrorString(e1 != cudaSuccess ? e1 : e2));
    }
    cudaError_t e3 = cudaGraphInstantiate(&g->graph[which], graph, 0);
    cudaGraphDestroy(graph);
    if (e3 != cudaSuccess) return sem_fail(SEM_ERR_CUDA, cudaGetErrorString(e3));
    return SEM_OK;
}

}  // namespace

extern "C" {

int sem_group_destroy(sem_group *g)
{
    if (!g) return SEM_OK;
    if (g->stream) cudaStreamSynchronize(g->stream);
    drop_graphs(g);
    for (auto e : g->join) cudaEventDestroy(e);
    if (g->fork) cudaEventDestroy(g->fork);
    if (g->stream) cudaStreamDestroy(g->stream);
    delete g;
    return SEM_OK;
}

int sem_group_create(int n, sem_solver *const *solvers, sem_group **out)
{
    GUARD_BEGIN
    if (!out || n < 1 || !solvers) return sem_fail(SEM_ERR_ARG, "need at least one solver");
    *out = nullptr;
    for (int i = 0; i < n; i++) {
        if (!solvers[i]) return sem_fail(SEM_ERR_ARG, "NULL solver in group");
        for (int j = 0; j < i; j++)
            if (solvers[j] == solvers[i]) return sem_fail(SEM_ERR_ARG, "a solver appears twice in the group");
    }
    sem_group *g = new sem_group();
    g->members.assign(solvers, solvers + n);
    std::stable_sort(g->members.begin(), g->members.end(),
                     [](const sem_solver *a, const sem_solver *b) { return a->n_int > b->n_int; });
    cudaError_t e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->fork, cudaEventDisableTiming);
    g->join.assign(n, nullptr);
    for (int i = 0; i < n && e == cudaSuccess; i++) e = cudaEventCreateWithFlags(&g->join[i], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        sem_group_destroy(g);
        return sem_fail(SEM_ERR_CUDA, cudaGetErrorString(e));
    }
    *out = g;
    return SEM_OK;
    GUARD_END
}

int sem_group_step(sem_group *g, int n_steps)
{
    GUARD_BEGIN
    if (!g || n_steps < 0) return sem_fail(SEM_ERR_ARG, "bad arguments");
    if (n_steps == 0) return SEM_OK;
    for (sem_solver *s : g->members) {
        if (s->kernel == SEM_KERNEL_ELEMENT) return sem_fail(SEM_ERR_STATE, "group members use the stencil pass");
        int rc = solver_prepare(s, n_steps);
        if (rc) return rc;
    }
    if (stale(g)) {
        drop_graphs(g);
        g->gen.resize(g->members.size());
        for (size_t i = 0; i < g->members.size(); i++) g->gen[i] = g->members[i]->graph_gen;
    }
    // order against work already on the members' own streams (set-up, earlier solo steps)
    for (size_t i = 0; i < g->members.size(); i++) {
        CUDA_TRY(cudaEventRecord(g->join[i], g->members[i]->stream));
        CUDA_TRY(cudaStreamWaitEvent(g->stream, g->join[i], 0));
    }
    int done = 0;
    while (n_steps - done >= 2) {
        if (!g->graph[g->flip]) {
            int rc = capture(g, g->flip);
            if (rc) return rc;
        }
        CUDA_TRY(cudaGraphLaunch(g->graph[g->flip], g->stream));
        done += 2;
    }
    if (done < n_steps) {
        CUDA_TRY(enqueue_all(g, 1));
        for (sem_solver *s : g->members) s->cur ^= 1;
        g->flip ^= 1;
    }
    // and the members' later calls (reads, solo steps) after this work
    CUDA_TRY(cudaEventRecord(g->fork, g->stream));
    for (sem_solver *s : g->members) {
        CUDA_TRY(cudaStreamWaitEvent(s->stream, g->fork, 0));
        s->steps_done += n_steps;
    }
    return SEM_OK;
    GUARD_END
}

int sem_group_synchronize(sem_group *g)
{
    GUARD_BEGIN
    if (!g) return sem_fail(SEM_ERR_ARG, "NULL group");
    CUDA_TRY(cudaStreamSynchronize(g->stream));
    for (sem_solver *s : g->members) {
        int rc = sem_solver_synchronize(s);
        if (rc) return rc;
    }
    return SEM_OK;
    GUARD_END
}

int sem_group_time_step(sem_group *g, int n_steps, float *ms_per_step)
{
    GUARD_BEGIN
    if (!g || !ms_per_step || n_steps < 1) return sem_fail(SEM_ERR_ARG, "bad arguments");
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    // resources first, so that the timed region holds only the graph launches
    int rc = SEM_OK;
    for (sem_solver *s : g->members)
        if (rc == SEM_OK) rc = solver_prepare(s, n_steps);
    if (rc == SEM_OK) {
        cudaEventRecord(e0, g->stream);
        rc = sem_group_step(g, n_steps);
        cudaEventRecord(e1, g->stream);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        *ms_per_step = ms / n_steps;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
    GUARD_END
}

}  // extern "C"
