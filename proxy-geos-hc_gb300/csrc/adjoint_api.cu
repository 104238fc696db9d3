// adjoint_api.cu -- gradient of the trace misfit
//     L = 1/2 sum_n sum_r (d_r^n - obs_r^n)^2
// with respect to the per-node squared slowness m (M_i = m_i W_i, W_i the geometric mass), by the
// adjoint-state method with checkpointed forward recompute (sem_adjoint_*).
//
// Forward step n of the plain solver (levels p^n, q^n; sponge s; interior mask J; a = dt^2/M):
//     p'      = p^n + b^n                                    sources   (SEMsolver.cpp:39-43)
//     p^{n+1} = s (J (2 p' - q^n - a K p') + (1 - J) q^n)    update    (SEMsolver.cpp:85-89)
//     q^{n+1} = s p',   d^n = R p^{n+1}                      sponge on both levels, receivers
// K is symmetric and a, s, J are diagonal, so with chi = s a J lambda (lambda = dL/dp) the
// adjoint recursion is the same step run backward in time:
//     chi^n = s (2 chi^{n+1} - s chi^{n+2} - a K chi^{n+1}) + s a R^T res^{n-1}    (interior nodes)
// i.e. the plain stencil pass applied to chi, with the residuals injected at the interior
// receiver nodes as sources of coefficient s_r a_r (boundary values of chi stay zero), and
//     dL/dm_i = (1/m_i) sum_n chi^{n+1}_i (K p'^n)_i .
// The forward levels are checkpointed every k steps; in the backward sweep each segment is
// recomputed from its checkpoint with K p'^n recorded per step (stencil mode RECORD_KP), then the
// segment's adjoint steps run newest first with the gradient accumulated inside the same pass
// (mode GRADIENT).  The source coefficients dt^2 c_e^2 (SEMsolver.cpp:41-42) are held fixed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "abi.h"
#include "solver.h"

using namespace semgb;

struct sem_adjoint {
    sem_mesh *mesh = nullptr;
    float dt = 0;
    int nsteps = 0, every = 0, nseg = 0;
    sem_solver *fwd = nullptr;  // forward run (checkpoints, recompute)
    sem_solver *adj = nullptr;  // adjoint run (residual sources), on the forward run's stream
    float *d_ckpt = nullptr;    // [nseg][2][n_int]: current and stored previous level at n = seg*every
    float *d_kp = nullptr;      // [every][n_int]: K p' of the steps of one segment
    float *d_grad = nullptr;    // [n_int]
    int *d_seg = nullptr;       // segment the backward sweep is on (read by its graphs)
    // one backward segment of `every` steps (restore, recompute, adjoint) replayed as a CUDA
    // graph, per (forward, adjoint) level parity at its start; valid while both solvers'
    // captured parameters are (gen)
    cudaGraphExec_t seg_graph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    uint64_t seg_gen[2] = {0, 0};
    int64_t n_int = 0;
    bool have_forward = false;
    int nrec = 0;
    std::vector<int64_t> rec;   // receiver nodes, device layout, caller order
    bool sponge = false;
    std::vector<float> sx, sy, sz;
};

namespace {

__global__ void k_set_int(int *p, int v) { *p = v; }

__global__ void k_dec_int(int *p) { *p -= 1; }

// Levels of the forward run at the start of segment *seg (its checkpoint) and the step counter
__global__ void k_restore_segment(const float *ckpt, const int *seg, int64_t lv, int every, float *cur, float *prev,
                                  int *ctr)
{
    const int sg = *seg;
    const float *ck = ckpt + (size_t)sg * 2 * lv;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < lv / 4; i += (int64_t)gridDim.x * blockDim.x) {
        reinterpret_cast<float4 *>(cur)[i] = reinterpret_cast<const float4 *>(ck)[i];
        reinterpret_cast<float4 *>(prev)[i] = reinterpret_cast<const float4 *>(ck + lv)[i];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ctr[0] = sg * every;
        ctr[1] = sg * every - 1;
    }
}

void destroy_seg_graphs(sem_adjoint *a)
{
    for (auto &row : a->seg_graph)
        for (auto &g : row)
            if (g) { cudaGraphExecDestroy(g); g = nullptr; }
}

// One backward segment of `len` steps, the segment index read from the device: restore its
// checkpoint, recompute it recording K p', run its adjoint steps newest first with the gradient,
// then step the segment index down.
cudaError_t enqueue_segment(sem_adjoint *a, int len)
{
    sem_solver *f = a->fwd, *g = a->adj;
    const size_t lv = (size_t)a->n_int;
    cudaError_t e;
    k_restore_segment<<<152 * 8, 256, 0, f->stream>>>(a->d_ckpt, a->d_seg, a->n_int, a->every, f->d_p[f->cur],
                                                        f->d_p[1 - f->cur], f->d_ctr);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    for (int n = 0; n < len; n++) {
        StepExtra x;
        x.mode = STENCIL_RECORD_KP;
        x.kp = a->d_kp + (size_t)n * lv;
        if ((e = solver_enqueue_step(f, f->cur, nullptr, &x)) != cudaSuccess) return e;
        f->cur ^= 1;
    }
    for (int n = len - 1; n >= 0; n--) {
        StepExtra x;
        x.mode = STENCIL_GRADIENT;
        x.kp = a->d_kp + (size_t)n * lv;
        x.grad = a->d_grad;
        if ((e = solver_enqueue_step(g, g->cur, nullptr, &x)) != cudaSuccess) return e;
        g->cur ^= 1;
    }
    k_dec_int<<<1, 1, 0, f->stream>>>(a->d_seg);
    return cudaGetLastError();
}

int check_ready(const sem_adjoint *a)
{
    if (!a) return sem_fail(SEM_ERR_ARG, "NULL adjoint handle");
    return SEM_OK;
}

}  // namespace

extern "C" {

int sem_adjoint_destroy(sem_adjoint *a)
{
    if (!a) return SEM_OK;
    if (a->fwd) cudaStreamSynchronize(a->fwd->stream);
    destroy_seg_graphs(a);
    dfree(a->d_seg);
    if (a->adj) sem_solver_destroy(a->adj);
    if (a->fwd) sem_solver_destroy(a->fwd);
    dfree(a->d_ckpt);
    dfree(a->d_kp);
    dfree(a->d_grad);
    delete a;
    return SEM_OK;
}

int sem_adjoint_create(sem_mesh *m, float dt, int n_steps, int checkpoint_every, sem_adjoint **out)
{
    GUARD_BEGIN
    if (!m || !out) return sem_fail(SEM_ERR_ARG, "NULL argument");
    *out = nullptr;
    if (!(dt > 0) || n_steps < 1 || checkpoint_every < 1)
        return sem_fail(SEM_ERR_ARG, "dt > 0, n_steps >= 1 and checkpoint_every >= 1 required");
    sem_adjoint *a = new sem_adjoint();
    a->mesh = m;
    a->dt = dt;
    a->nsteps = n_steps;
    a->every = std::min(checkpoint_every, n_steps);
    a->nseg = (n_steps + a->every - 1) / a->every;
    a->n_int = m->box.n_int;
    int rc = sem_solver_create(m, dt, &a->fwd);
    if (rc == SEM_OK) rc = sem_solver_create(m, dt, &a->adj);
    if (rc == SEM_OK) rc = sem_solver_set_kernel(a->fwd, SEM_KERNEL_STENCIL);
    if (rc == SEM_OK) rc = sem_solver_set_kernel(a->adj, SEM_KERNEL_STENCIL);
    if (rc == SEM_OK) rc = sem_solver_set_stream(a->adj, a->fwd->stream);
    if (rc == SEM_OK) {
        // the recording and gradient passes are built for the default tile shape
        a->fwd->tile_shape = semgb::kTileDefault;
        a->adj->tile_shape = semgb::kTileDefault;
    }
    if (rc != SEM_OK) {
        sem_adjoint_destroy(a);
        return rc;
    }
    cudaError_t e;
    if ((e = dalloc(&a->d_ckpt, (size_t)a->nseg * 2 * a->n_int)) != cudaSuccess ||
        (e = dalloc(&a->d_kp, (size_t)a->every * a->n_int)) != cudaSuccess ||
        (e = dalloc(&a->d_grad, (size_t)a->n_int)) != cudaSuccess || (e = dalloc(&a->d_seg, 1)) != cudaSuccess) {
        sem_adjoint_destroy(a);
        return sem_fail(SEM_ERR_OOM, std::string("checkpoint storage: ") + cudaGetErrorString(e));
    }
    *out = a;
    return SEM_OK;
    GUARD_END
}

int sem_adjoint_set_sponge_profile(sem_adjoint *a, const float *sx, const float *sy, const float *sz)
{
    GUARD_BEGIN
    int rc = check_ready(a);
    if (rc) return rc;
    if ((rc = sem_solver_set_sponge_profile(a->fwd, sx, sy, sz)) != SEM_OK) return rc;
    if ((rc = sem_solver_set_sponge_profile(a->adj, sx, sy, sz)) != SEM_OK) return rc;
    const Box &b = a->mesh->box;
    a->sponge = sx && sy && sz;
    if (a->sponge) {
        a->sx.assign(sx, sx + b.nx);
        a->sy.assign(sy, sy + b.ny);
        a->sz.assign(sz, sz + b.nz);
    }
    a->have_forward = false;
    return SEM_OK;
    GUARD_END
}

int sem_adjoint_set_sponge(sem_adjoint *a, int thickness, float sigma)
{
    GUARD_BEGIN
    int rc = check_ready(a);
    if (rc) return rc;
    if (thickness < 0 || !(sigma >= 0)) return sem_fail(SEM_ERR_ARG, "bad sponge parameters");
    if (thickness == 0) return sem_adjoint_set_sponge_profile(a, nullptr, nullptr, nullptr);
    std::vector<float> x, y, z;
    box_sponge_profile(a->mesh->box, a->mesh->gll, thickness, sigma, x, y, z);
    return sem_adjoint_set_sponge_profile(a, x.data(), y.data(), z.data());
    GUARD_END
}

int sem_adjoint_set_sources(sem_adjoint *a, int n_src, const int64_t *elements, const float *wavelet, int n_samples)
{
    int rc = check_ready(a);
    if (rc) return rc;
    a->have_forward = false;
    return sem_solver_set_sources(a->fwd, n_src, elements, wavelet, n_samples);
}

int sem_adjoint_set_source_points(sem_adjoint *a, int n_src, const float *xyz, const float *wavelet, int n_samples)
{
    int rc = check_ready(a);
    if (rc) return rc;
    a->have_forward = false;
    return sem_solver_set_source_points(a->fwd, n_src, xyz, wavelet, n_samples);
}

int sem_adjoint_set_receiver_nodes(sem_adjoint *a, int n_rec, const int64_t *nodes)
{
    GUARD_BEGIN
    int rc = check_ready(a);
    if (rc) return rc;
    if ((rc = sem_solver_set_receiver_nodes(a->fwd, n_rec, nodes)) != SEM_OK) return rc;
    a->nrec = n_rec;
    a->rec.resize(n_rec);
    for (int r = 0; r < n_rec; r++) a->rec[r] = to_internal(a->mesh->box, nodes[r]);
    a->have_forward = false;
    return SEM_OK;
    GUARD_END
}

int sem_adjoint_set_receivers(sem_adjoint *a, int n_rec, const float *xyz)
{
    GUARD_BEGIN
    int rc = check_ready(a);
    if (rc) return rc;
    if (n_rec < 0 || (n_rec > 0 && !xyz)) return sem_fail(SEM_ERR_ARG, "bad receiver array");
    std::vector<int64_t> nodes(n_rec);
    for (int r = 0; r < n_rec; r++)
        nodes[r] = box_nearest_node(a->mesh->box, a->mesh->gll, xyz[3 * r], xyz[3 * r + 1], xyz[3 * r + 2]);
    return sem_adjoint_set_receiver_nodes(a, n_rec, nodes.data());
    GUARD_END
}

int sem_adjoint_set_adjoint_receiver_nodes(sem_adjoint *a, int n_rec, const int64_t *nodes)
{
    int rc = check_ready(a);
    if (rc) return rc;
    return sem_solver_set_receiver_nodes(a->adj, n_rec, nodes);
}

int sem_adjoint_forward(sem_adjoint *a, float *traces)
{
    GUARD_BEGIN
    int rc = check_ready(a);
    if (rc) return rc;
    sem_solver *f = a->fwd;
    if ((rc = sem_solver_reset(f)) != SEM_OK) return rc;
    if ((rc = solver_prepare(f, a->nsteps)) != SEM_OK) return rc;
    const size_t lv = (size_t)a->n_int;
    for (int seg = 0; seg < a->nseg; seg++) {
        float *ck = a->d_ckpt + (size_t)seg * 2 * lv;
        CUDA_TRY(cudaMemcpyAsync(ck, f->d_p[f->cur], lv * 4, cudaMemcpyDeviceToDevice, f->stream));
        CUDA_TRY(cudaMemcpyAsync(ck + lv, f->d_p[1 - f->cur], lv * 4, cudaMemcpyDeviceToDevice, f->stream));
        const int n = std::min(a->every, a->nsteps - seg * a->every);
        if ((rc = sem_solver_step(f, n)) != SEM_OK) return rc;
    }
    if ((rc = sem_solver_synchronize(f)) != SEM_OK) return rc;
    a->have_forward = true;
    if (traces && a->nrec > 0) return sem_solver_get_traces(f, traces);
    return SEM_OK;
    GUARD_END
}

int sem_adjoint_backward(sem_adjoint *a, const float *residual, float *grad)
{
    GUARD_BEGIN
    int rc = check_ready(a);
    if (rc) return rc;
    if (!a->have_forward) return sem_fail(SEM_ERR_STATE, "sem_adjoint_forward must run first");
    if (a->nrec > 0 && !residual) return sem_fail(SEM_ERR_ARG, "NULL residual");
    sem_solver *f = a->fwd, *g = a->adj;
    const Box &b = a->mesh->box;
    const int N = a->nsteps;
    const size_t lv = (size_t)a->n_int;
    // adjoint sources: residuals at the interior receiver nodes, newest step first, coefficient s a
    std::vector<int64_t> nodes;
    std::vector<float> coef, wav;
    CUDA_TRY(cudaStreamSynchronize(f->stream));
    for (int r = 0; r < a->nrec; r++) {
        const int64_t q = a->rec[r];
        const int64_t iy = q / (b.nxp * b.nz), rr = q - iy * b.nxp * b.nz, iz = rr / b.nxp, ix = rr - iz * b.nxp;
        if (ix == 0 || ix == b.nx - 1 || iy == 0 || iy == b.ny - 1 || iz == 0 || iz == b.nz - 1) continue;
        float av = 0.f;
        CUDA_TRY(cudaMemcpy(&av, f->d_a + q, 4, cudaMemcpyDeviceToHost));
        const float s = a->sponge ? a->sx[ix] * a->sy[iy] * a->sz[iz] : 1.f;
        nodes.push_back(q);
        coef.push_back(s * av);
        for (int j = 0; j < N; j++) wav.push_back(residual[(size_t)(N - 1 - j) * a->nrec + r]);
    }
    if ((rc = solver_set_raw_sources(g, (int)nodes.size(), nodes.data(), coef.data(), wav.data(), N)) != SEM_OK)
        return rc;
    if ((rc = sem_solver_reset(g)) != SEM_OK) return rc;
    if ((rc = solver_prepare(g, N)) != SEM_OK) return rc;
    if ((rc = solver_prepare(f, 0)) != SEM_OK) return rc;
    CUDA_TRY(cudaMemsetAsync(a->d_grad, 0, lv * 4, f->stream));
    if (a->seg_gen[0] != f->graph_gen || a->seg_gen[1] != g->graph_gen) {
        destroy_seg_graphs(a);
        a->seg_gen[0] = f->graph_gen;
        a->seg_gen[1] = g->graph_gen;
    }
    k_set_int<<<1, 1, 0, f->stream>>>(a->d_seg, a->nseg - 1);
    CUDA_TRY(cudaGetLastError());
    // the newest segment (possibly shorter) directly, then whole segments from graphs
    CUDA_TRY(enqueue_segment(a, N - (a->nseg - 1) * a->every));
    for (int seg = a->nseg - 2; seg >= 0; seg--) {
        cudaGraphExec_t &ge = a->seg_graph[f->cur][g->cur];
        if (!ge) {
            cudaGraph_t gr = nullptr;
            CUDA_TRY(cudaStreamBeginCapture(f->stream, cudaStreamCaptureModeThreadLocal));
            const int fc = f->cur, gc = g->cur;
            const cudaError_t e1 = enqueue_segment(a, a->every);
            const cudaError_t e2 = cudaStreamEndCapture(f->stream, &gr);
            // the capture ran nothing: the parities advance with the replays below
            f->cur = fc;
            g->cur = gc;
            if (e1 != cudaSuccess || e2 != cudaSuccess) {
                if (gr) cudaGraphDestroy(gr);
                return sem_fail(SEM_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e1 != cudaSuccess ? e1 : e2));
            }
            const cudaError_t e3 = cudaGraphInstantiate(&ge, gr, 0);
            cudaGraphDestroy(gr);
            if (e3 != cudaSuccess) return sem_fail(SEM_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e3));
        }
        CUDA_TRY(cudaGraphLaunch(ge, f->stream));
        if (a->every % 2) {
            f->cur ^= 1;
            g->cur ^= 1;
        }
    }
    g->steps_done = N;
    // the forward run ends on its first segment; its checkpoints and traces stay valid
    CUDA_TRY(launch_grad_scale(a->d_grad, f->d_a, b.ex, b.ey, b.ez, b.order, b.nxp, f->d_w, a->mesh->geo.detJ,
                               (double)a->dt * a->dt, f->stream));
    if ((rc = sem_solver_synchronize(g)) != SEM_OK) return rc;
    int status = 0;
    CUDA_TRY(cudaMemcpy(&status, f->d_status, 4, cudaMemcpyDeviceToHost));
    if (status != 0) return sem_fail(SEM_ERR_TIMEOUT, "a bounded wait for a TMA tile gave up in the recompute");
    if (grad)
        CUDA_TRY(field_to_host(grad, a->d_grad, b.nx, b.nxp, b.nz * b.ny, f->stream));
    return SEM_OK;
    GUARD_END
}

int sem_adjoint_gradient(sem_adjoint *a, const float *observed, double *loss, float *grad)
{
    GUARD_BEGIN
    int rc = check_ready(a);
    if (rc) return rc;
    if (!a->have_forward) return sem_fail(SEM_ERR_STATE, "sem_adjoint_forward must run first");
    if (a->nrec > 0 && !observed) return sem_fail(SEM_ERR_ARG, "NULL observed traces");
    const size_t n = (size_t)a->nsteps * a->nrec;
    std::vector<float> res(n);
    if (n > 0 && (rc = sem_solver_get_traces(a->fwd, res.data())) != SEM_OK) return rc;
    double l = 0.0;
    for (size_t i = 0; i < n; i++) {
        res[i] -= observed[i];
        l += 0.5 * (double)res[i] * (double)res[i];
    }
    if (loss) *loss = l;
    return sem_adjoint_backward(a, res.data(), grad);
    GUARD_END
}

int sem_adjoint_get_adjoint_traces(sem_adjoint *a, float *out)
{
    int rc = check_ready(a);
    if (rc) return rc;
    return sem_solver_get_traces(a->adj, out);
}

}  // extern "C"
