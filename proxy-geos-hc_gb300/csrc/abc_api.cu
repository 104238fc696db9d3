// abc_api.cu -- C ABI of the learned absorbing boundary: the boundary network (sem_mlp_*) and
// its attachment to a solver (sem_abc_*).
//
// After every solver step the network corrects the new level on the strip nodes -- the boundary
// nodes themselves (layer 0), or the interior nodes within `layer` elements of a face -- from
// p^{n+1}, p^n and p^{n-1} on each node's 3x3x3
// neighbourhood (81 features, divided by their largest magnitude; the output, clipped to [-1, 1],
// is multiplied back).  On the boundary nodes it is the node's new value (so it never exceeds
// the largest magnitude of its neighbourhood), on interior strip nodes a correction.
// p^{n-1} of the strip and of its inner neighbour layer is kept in a history array.  The
// sponge of the solver (if any) still applies; the network replaces most of its thickness.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <random>
#include <vector>

#include "abi.h"
#include "mlp.h"
#include "solver.h"

using namespace semgb;

struct sem_mlp {
    float *d_master = nullptr;  // FP32 parameters (mlp.h layout)
    float *d_m = nullptr, *d_v = nullptr, *d_grad = nullptr;
    float *d_part = nullptr;       // per-CTA partial gradients [kMlpMaxCTAs][kMlpParams]
    double *d_part_loss = nullptr;  // per-CTA partial losses [kMlpMaxCTAs]
    uint16_t *d_w1 = nullptr, *d_w2 = nullptr;
    float *d_b1 = nullptr, *d_b2 = nullptr, *d_w3 = nullptr, *d_b3 = nullptr;
    double *d_loss = nullptr;
    int adam_t = 0;
    cudaStream_t stream = nullptr;
    MlpDev dev() const { return MlpDev{d_w1, d_w2, d_b1, d_b2, d_w3, d_b3}; }
};

struct sem_abc {
    sem_solver *s = nullptr;
    sem_mlp *net = nullptr;
    int layer = 0;
    int64_t *d_nodes = nullptr;  // strip nodes (device layout)
    int64_t n = 0;
    int64_t *d_shell = nullptr;  // history nodes: strip and its inner neighbours
    int64_t n_shell = 0;
    float *d_hist = nullptr;     // [n_int]
    float *d_corr = nullptr;     // [n]
    // layer 0: face tiles (abc_face) and a second history buffer: a step reads p^{n-1} from
    // hbuf[hcur] and writes p^n into the other
    bool face = false;
    int4 *d_tiles = nullptr;
    int64_t ntiles = 0;
    float *d_hist_alt = nullptr;
    int hcur = 0;
    FaceDesc faces[6];
    // two corrected steps replayed as one CUDA graph, per (current level, history buffer)
    // parity; valid while the solver's captured parameters are (graph_gen)
    cudaGraphExec_t graph2[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    uint64_t graph_gen = 0;
    float *hist_now() const { return face && hcur ? d_hist_alt : d_hist; }
    float *hist_next() const { return face && !hcur ? d_hist_alt : d_hist; }
};

namespace {

int net_upload(sem_mlp *m)
{
    CUDA_TRY(mlp_pack(m->d_master, m->d_w1, m->d_w2, m->d_b1, m->d_b2, m->d_w3, m->d_b3, m->stream));
    CUDA_TRY(cudaStreamSynchronize(m->stream));
    return SEM_OK;
}

AbcArgs abc_args(const sem_abc *a)
{
    const sem_solver *s = a->s;
    const Box &b = s->mesh->box;
    AbcArgs x{};
    x.nodes = a->d_nodes;
    x.n = a->n;
    x.p_new = s->d_p[s->cur];      // after a step the new level is the current one
    x.p_cur = s->d_p[1 - s->cur];  // and p^n the stored previous one
    x.hist = a->hist_now();
    x.sx = s->sponge ? s->d_sx : nullptr;
    x.sy = s->sponge ? s->d_sy : nullptr;
    x.sz = s->sponge ? s->d_sz : nullptr;
    x.nx = b.nx;
    x.nxp = b.nxp;
    x.ny = b.ny;
    x.nz = b.nz;
    x.corr = a->d_corr;
    x.absolute = a->layer == 0 ? 1 : 0;
    return x;
}

// correction after the step that just ran (levels as abc_args reads them)
cudaError_t enqueue_correction(sem_abc *a)
{
    sem_solver *s = a->s;
    const AbcArgs x = abc_args(a);
    if (a->face) {
        AbcFaceArgs f{};
        for (int k = 0; k < 6; k++) f.face[k] = a->faces[k];
        f.tiles = a->d_tiles;
        f.ntiles = a->ntiles;
        f.p_new = s->d_p[s->cur];
        f.p_cur = x.p_cur;
        f.hist = a->hist_now();
        f.hist_next = a->hist_next();
        f.sx = x.sx; f.sy = x.sy; f.sz = x.sz;
        f.nx = x.nx; f.nxp = x.nxp; f.ny = x.ny; f.nz = x.nz;
        cudaError_t e = abc_face(a->net->dev(), f, s->stream);  // writes the new values in place
        if (e != cudaSuccess) return e;
        a->hcur ^= 1;
        return cudaSuccess;
    }
    cudaError_t e = abc_correction(a->net->dev(), x, s->stream);
    if (e != cudaSuccess) return e;
    if ((e = abc_apply(x, s->d_p[s->cur], a->d_hist, s->stream)) != cudaSuccess) return e;
    const Box &b = s->mesh->box;
    return abc_history(a->d_shell, a->n_shell, s->d_p[1 - s->cur], x.sx, x.sy, x.sz, b.nxp, b.nz, a->d_hist,
                       s->stream);
}

}  // namespace

extern "C" {

// ---- network -------------------------------------------------------------------------------

int sem_mlp_destroy(sem_mlp *m)
{
    if (!m) return SEM_OK;
    if (m->stream) cudaStreamSynchronize(m->stream);
    dfree(m->d_master); dfree(m->d_m); dfree(m->d_v); dfree(m->d_grad);
    dfree(m->d_part); dfree(m->d_part_loss);
    dfree(m->d_w1); dfree(m->d_w2); dfree(m->d_b1); dfree(m->d_b2); dfree(m->d_w3); dfree(m->d_b3);
    dfree(m->d_loss);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return SEM_OK;
}

int sem_mlp_create(uint64_t seed, sem_mlp **out)
{
    GUARD_BEGIN
    if (!out) return sem_fail(SEM_ERR_ARG, "NULL argument");
    *out = nullptr;
    sem_mlp *m = new sem_mlp();
    cudaError_t e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = dalloc(&m->d_master, kMlpParams);
    if (e == cudaSuccess) e = dalloc(&m->d_m, kMlpParams);
    if (e == cudaSuccess) e = dalloc(&m->d_v, kMlpParams);
    if (e == cudaSuccess) e = dalloc(&m->d_grad, kMlpParams);
    if (e == cudaSuccess) e = dalloc(&m->d_part, (size_t)kMlpMaxCTAs * kMlpParams);
    if (e == cudaSuccess) e = dalloc(&m->d_part_loss, (size_t)kMlpMaxCTAs);
    if (e == cudaSuccess) e = dalloc(&m->d_w1, kMlpHidden * kMlpInPad);
    if (e == cudaSuccess) e = dalloc(&m->d_w2, kMlpHidden * kMlpHidden);
    if (e == cudaSuccess) e = dalloc(&m->d_b1, kMlpHidden);
    if (e == cudaSuccess) e = dalloc(&m->d_b2, kMlpHidden);
    if (e == cudaSuccess) e = dalloc(&m->d_w3, kMlpHidden);
    if (e == cudaSuccess) e = dalloc(&m->d_b3, 1);
    if (e == cudaSuccess) e = dalloc(&m->d_loss, 1);
    if (e != cudaSuccess) {
        sem_mlp_destroy(m);
        return sem_fail(SEM_ERR_OOM, cudaGetErrorString(e));
    }
    // He-normal hidden layers, a small output layer (the initial correction is close to zero)
    std::mt19937_64 rng(seed);
    std::normal_distribution<float> nd(0.f, 1.f);
    std::vector<float> p(kMlpParams, 0.f);
    for (int i = 0; i < kMlpHidden * kMlpIn; i++) p[kOffW1 + i] = nd(rng) * std::sqrt(2.f / kMlpIn);
    for (int i = 0; i < kMlpHidden * kMlpHidden; i++) p[kOffW2 + i] = nd(rng) * std::sqrt(2.f / kMlpHidden);
    for (int i = 0; i < kMlpHidden; i++) p[kOffW3 + i] = nd(rng) * 0.01f;
    int rc = sem_mlp_set_params(m, p.data());
    if (rc) {
        sem_mlp_destroy(m);
        return rc;
    }
    *out = m;
    return SEM_OK;
    GUARD_END
}

int sem_mlp_n_params(void) { return kMlpParams; }

int sem_mlp_set_params(sem_mlp *m, const float *params)
{
    GUARD_BEGIN
    if (!m || !params) return sem_fail(SEM_ERR_ARG, "NULL argument");
    for (int i = 0; i < kMlpParams; i++)
        if (!std::isfinite(params[i])) return sem_fail(SEM_ERR_ARG, "non-finite parameter");
    CUDA_TRY(cudaMemcpy(m->d_master, params, kMlpParams * 4, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemset(m->d_m, 0, kMlpParams * 4));
    CUDA_TRY(cudaMemset(m->d_v, 0, kMlpParams * 4));
    m->adam_t = 0;
    return net_upload(m);
    GUARD_END
}

int sem_mlp_get_params(sem_mlp *m, float *params)
{
    GUARD_BEGIN
    if (!m || !params) return sem_fail(SEM_ERR_ARG, "NULL argument");
    CUDA_TRY(cudaStreamSynchronize(m->stream));
    CUDA_TRY(cudaMemcpy(params, m->d_master, kMlpParams * 4, cudaMemcpyDeviceToHost));
    return SEM_OK;
    GUARD_END
}

int sem_mlp_forward(sem_mlp *m, int64_t n, const float *x, float *y)
{
    GUARD_BEGIN
    if (!m || n < 0 || (n > 0 && (!x || !y))) return sem_fail(SEM_ERR_ARG, "bad arguments");
    if (n == 0) return SEM_OK;
    float *dx = nullptr, *dy = nullptr;
    CUDA_TRY(dalloc(&dx, (size_t)n * kMlpIn));
    cudaError_t e = dalloc(&dy, (size_t)n);
    if (e == cudaSuccess) e = cudaMemcpy(dx, x, (size_t)n * kMlpIn * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = mlp_forward(m->dev(), dx, dy, n, m->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    if (e == cudaSuccess) e = cudaMemcpy(y, dy, (size_t)n * 4, cudaMemcpyDeviceToHost);
    dfree(dx);
    dfree(dy);
    CUDA_TRY(e);
    return SEM_OK;
    GUARD_END
}

int sem_mlp_loss_grad(sem_mlp *m, int64_t n, const float *x, const float *t, double *loss, float *grad)
{
    GUARD_BEGIN
    if (!m || n < 1 || !x || !t) return sem_fail(SEM_ERR_ARG, "bad arguments");
    float *dx = nullptr, *dt = nullptr;
    CUDA_TRY(dalloc(&dx, (size_t)n * kMlpIn));
    cudaError_t e = dalloc(&dt, (size_t)n);
    if (e == cudaSuccess) e = cudaMemcpy(dx, x, (size_t)n * kMlpIn * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dt, t, (size_t)n * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->d_grad, 0, kMlpParams * 4, m->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->d_loss, 0, 8, m->stream);
    if (e == cudaSuccess) e = mlp_loss_grad(m->dev(), dx, dt, n, m->d_loss, m->d_grad, m->d_part, m->d_part_loss, m->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    if (e == cudaSuccess && loss) e = cudaMemcpy(loss, m->d_loss, 8, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && grad) e = cudaMemcpy(grad, m->d_grad, kMlpParams * 4, cudaMemcpyDeviceToHost);
    dfree(dx);
    dfree(dt);
    CUDA_TRY(e);
    return SEM_OK;
    GUARD_END
}

int sem_mlp_train(sem_mlp *m, int64_t n, const float *x, const float *t, int epochs, int batch, float lr,
                  uint64_t seed, double *losses)
{
    GUARD_BEGIN
    if (!m || n < 1 || !x || !t || epochs < 0 || batch < 1 || !(lr > 0))
        return sem_fail(SEM_ERR_ARG, "bad arguments");
    // samples resident on the device, shuffled once per epoch on the host (index order)
    float *dx = nullptr, *dt = nullptr, *bx = nullptr, *bt = nullptr;
    const int64_t nb = std::min<int64_t>(batch, n);
    CUDA_TRY(dalloc(&dx, (size_t)n * kMlpIn));
    cudaError_t e = dalloc(&dt, (size_t)n);
    if (e == cudaSuccess) e = dalloc(&bx, (size_t)nb * kMlpIn);
    if (e == cudaSuccess) e = dalloc(&bt, (size_t)nb);
    if (e == cudaSuccess) e = cudaMemcpy(dx, x, (size_t)n * kMlpIn * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dt, t, (size_t)n * 4, cudaMemcpyHostToDevice);
    std::vector<int64_t> perm(n);
    for (int64_t i = 0; i < n; i++) perm[i] = i;
    int64_t *dperm = nullptr;
    if (e == cudaSuccess) e = dalloc(&dperm, (size_t)n);
    std::mt19937_64 rng(seed);
    for (int ep = 0; ep < epochs && e == cudaSuccess; ep++) {
        std::shuffle(perm.begin(), perm.end(), rng);
        e = cudaMemcpyAsync(dperm, perm.data(), (size_t)n * 8, cudaMemcpyHostToDevice, m->stream);
        double lsum = 0.0;
        int64_t seen = 0;
        for (int64_t b0 = 0; b0 + nb <= n && e == cudaSuccess; b0 += nb) {
            e = mlp_gather_rows(dx, dt, dperm + b0, nb, bx, bt, m->stream);
            if (e == cudaSuccess) e = cudaMemsetAsync(m->d_grad, 0, kMlpParams * 4, m->stream);
            if (e == cudaSuccess) e = cudaMemsetAsync(m->d_loss, 0, 8, m->stream);
            if (e == cudaSuccess) e = mlp_loss_grad(m->dev(), bx, bt, nb, m->d_loss, m->d_grad, m->d_part, m->d_part_loss, m->stream);
            if (e == cudaSuccess) e = mlp_adam(m->d_master, m->d_grad, m->d_m, m->d_v, ++m->adam_t, lr, m->stream);
            if (e == cudaSuccess)
                e = mlp_pack(m->d_master, m->d_w1, m->d_w2, m->d_b1, m->d_b2, m->d_w3, m->d_b3, m->stream);
            double l = 0;
            if (e == cudaSuccess) e = cudaMemcpyAsync(&l, m->d_loss, 8, cudaMemcpyDeviceToHost, m->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
            lsum += l * nb;
            seen += nb;
        }
        if (losses) losses[ep] = seen ? lsum / seen : 0.0;
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    dfree(dx); dfree(dt); dfree(bx); dfree(bt); dfree(dperm);
    CUDA_TRY(e);
    return SEM_OK;
    GUARD_END
}

int sem_mlp_adam_step(sem_mlp *m, const float *grad, float lr)
{
    GUARD_BEGIN
    if (!m || !grad || !(lr > 0)) return sem_fail(SEM_ERR_ARG, "bad arguments");
    CUDA_TRY(cudaMemcpyAsync(m->d_grad, grad, kMlpParams * 4, cudaMemcpyHostToDevice, m->stream));
    CUDA_TRY(mlp_adam(m->d_master, m->d_grad, m->d_m, m->d_v, ++m->adam_t, lr, m->stream));
    CUDA_TRY(mlp_pack(m->d_master, m->d_w1, m->d_w2, m->d_b1, m->d_b2, m->d_w3, m->d_b3, m->stream));
    CUDA_TRY(cudaStreamSynchronize(m->stream));
    return SEM_OK;
    GUARD_END
}

// ---- boundary ------------------------------------------------------------------------------

int sem_abc_destroy(sem_abc *a)
{
    if (!a) return SEM_OK;
    // the solver may already be gone (handles closed in any order): wait for the device instead
    // of the solver's stream
    cudaDeviceSynchronize();
    for (auto &row : a->graph2)
        for (auto &g : row)
            if (g) cudaGraphExecDestroy(g);
    dfree(a->d_nodes);
    dfree(a->d_shell);
    dfree(a->d_hist);
    dfree(a->d_corr);
    dfree(a->d_tiles);
    dfree(a->d_hist_alt);
    delete a;
    return SEM_OK;
}

int sem_abc_create(sem_solver *s, sem_mlp *net, int layer_elems, sem_abc **out)
{
    GUARD_BEGIN
    if (!s || !net || !out) return sem_fail(SEM_ERR_ARG, "NULL argument");
    *out = nullptr;
    const Box &b = s->mesh->box;
    if (layer_elems < 0 || 2 * layer_elems > std::min({b.ex, b.ey, b.ez}))
        return sem_fail(SEM_ERR_ARG, "layer must be >= 0 elements and fit twice in every axis");
    // layer 0: the boundary nodes themselves (the network supplies the face values that the
    // Dirichlet update would hold fixed); layer w > 0: interior nodes within w elements of a face
    const int64_t w = (int64_t)layer_elems * b.order;
    std::vector<int64_t> nodes, shell;
    for (int64_t iy = 0; iy < b.ny; iy++)
        for (int64_t iz = 0; iz < b.nz; iz++)
            for (int64_t ix = 0; ix < b.nx; ix++) {
                const int64_t d = std::min({ix, b.nx - 1 - ix, iy, b.ny - 1 - iy, iz, b.nz - 1 - iz});
                const int64_t q = ix + iz * b.nxp + iy * b.nxp * b.nz;
                if (w == 0 ? d == 0 : (d >= 1 && d <= w)) nodes.push_back(q);
                if (d <= w + 1) shell.push_back(q);
            }
    sem_abc *a = new sem_abc();
    a->s = s;
    a->net = net;
    a->layer = layer_elems;
    a->n = (int64_t)nodes.size();
    a->n_shell = (int64_t)shell.size();
    cudaError_t e = dalloc(&a->d_nodes, nodes.size());
    if (e == cudaSuccess) e = dalloc(&a->d_shell, shell.size());
    if (e == cudaSuccess) e = dalloc(&a->d_hist, (size_t)b.n_int);
    if (e == cudaSuccess) e = dalloc(&a->d_corr, nodes.size());
    if (e == cudaSuccess) e = cudaMemcpy(a->d_nodes, nodes.data(), nodes.size() * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(a->d_shell, shell.data(), shell.size() * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(a->d_hist, 0, (size_t)b.n_int * 4);
    if (e == cudaSuccess && layer_elems == 0) {
        // face tiles: y-faces whole, z-faces without the rows on y-faces, x-faces without the
        // rows on y- and z-faces, so every boundary node lies on one face
        const int64_t nx = b.nx, ny = b.ny, nz = b.nz;
        const int64_t dims[3] = {nx, ny, nz};
        struct Spec { int n, u, v; int64_t ulo, uhi, vlo, vhi; };
        const Spec spec[3] = {{1, 0, 2, 0, nx, 0, nz}, {2, 0, 1, 0, nx, 1, ny - 1}, {0, 2, 1, 1, nz - 1, 1, ny - 1}};
        std::vector<int4> tiles;
        for (int k = 0; k < 6; k++) {
            const Spec &sp = spec[k / 2];
            FaceDesc &f = a->faces[k];
            f.axis_n = sp.n; f.axis_u = sp.u; f.axis_v = sp.v;
            f.side = (k % 2 == 0) ? 0 : (int)(dims[sp.n] - 1);
            f.inward = (k % 2 == 0) ? 1 : -1;
            f.ulo = (int)sp.ulo; f.uhi = (int)sp.uhi; f.vlo = (int)sp.vlo; f.vhi = (int)sp.vhi;
            // a tile row is a node of the face where it lies within [ulo, uhi) x [vlo, vhi); every
            // such node is a boundary node (the strip of layer 0)
            for (int64_t v0 = sp.vlo; v0 < sp.vhi; v0 += kFaceTV)
                for (int64_t u0 = sp.ulo; u0 < sp.uhi; u0 += kFaceTU) tiles.push_back(make_int4(k, (int)u0, (int)v0, 0));
        }
        a->face = true;
        a->ntiles = (int64_t)tiles.size();
        e = dalloc(&a->d_tiles, tiles.size());
        if (e == cudaSuccess) e = dalloc(&a->d_hist_alt, (size_t)b.n_int);
        if (e == cudaSuccess) e = cudaMemcpy(a->d_tiles, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemset(a->d_hist_alt, 0, (size_t)b.n_int * 4);
    }
    if (e != cudaSuccess) {
        sem_abc_destroy(a);
        return sem_fail(SEM_ERR_OOM, cudaGetErrorString(e));
    }
    *out = a;
    return SEM_OK;
    GUARD_END
}

int sem_abc_info(const sem_abc *a, int64_t *n_nodes, int64_t *n_history)
{
    if (!a) return sem_fail(SEM_ERR_ARG, "NULL boundary");
    if (n_nodes) *n_nodes = a->n;
    if (n_history) *n_history = a->n_shell;
    return SEM_OK;
}

int sem_abc_nodes(const sem_abc *a, int64_t *nodes)
{
    GUARD_BEGIN
    if (!a || !nodes) return sem_fail(SEM_ERR_ARG, "NULL argument");
    std::vector<int64_t> q(a->n);
    CUDA_TRY(cudaMemcpy(q.data(), a->d_nodes, a->n * 8, cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < a->n; i++) nodes[i] = to_reference(a->s->mesh->box, q[i]);
    return SEM_OK;
    GUARD_END
}

int sem_abc_reset(sem_abc *a)
{
    GUARD_BEGIN
    if (!a) return sem_fail(SEM_ERR_ARG, "NULL boundary");
    CUDA_TRY(cudaStreamSynchronize(a->s->stream));
    CUDA_TRY(cudaMemset(a->d_hist, 0, (size_t)a->s->mesh->box.n_int * 4));
    if (a->d_hist_alt) CUDA_TRY(cudaMemset(a->d_hist_alt, 0, (size_t)a->s->mesh->box.n_int * 4));
    a->hcur = 0;
    return SEM_OK;
    GUARD_END
}

int sem_abc_set_history(sem_abc *a, const float *p_prev)
{
    GUARD_BEGIN
    if (!a || !p_prev) return sem_fail(SEM_ERR_ARG, "NULL argument");
    const Box &b = a->s->mesh->box;
    CUDA_TRY(cudaStreamSynchronize(a->s->stream));
    CUDA_TRY(field_from_host(a->hist_now(), p_prev, b.nx, b.nxp, b.nz * b.ny, a->s->stream));
    return SEM_OK;
    GUARD_END
}

int sem_abc_step(sem_abc *a, int n_steps)
{
    GUARD_BEGIN
    if (!a || n_steps < 0) return sem_fail(SEM_ERR_ARG, "bad arguments");
    if (n_steps == 0) return SEM_OK;
    sem_solver *s = a->s;
    if (s->kernel == SEM_KERNEL_ELEMENT) return sem_fail(SEM_ERR_STATE, "the learned boundary runs with the stencil pass");
    int rc = solver_prepare(s, n_steps);
    if (rc) return rc;
    if (a->graph_gen != s->graph_gen) {
        for (auto &row : a->graph2)
            for (auto &g : row)
                if (g) { cudaGraphExecDestroy(g); g = nullptr; }
        a->graph_gen = s->graph_gen;
    }
    int done = 0;
    while (n_steps - done >= 2) {
        cudaGraphExec_t &ge = a->graph2[s->cur][a->hcur];
        if (!ge) {
            // capture two corrected steps; the level and history parities come back to where
            // they started
            cudaGraph_t g = nullptr;
            CUDA_TRY(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
            cudaError_t e = cudaSuccess;
            for (int k = 0; k < 2 && e == cudaSuccess; k++) {
                e = solver_enqueue_step(s, s->cur);
                s->cur ^= 1;
                if (e == cudaSuccess) e = enqueue_correction(a);
            }
            const cudaError_t e2 = cudaStreamEndCapture(s->stream, &g);
            if (e != cudaSuccess || e2 != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                return sem_fail(SEM_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
            }
            const cudaError_t e3 = cudaGraphInstantiate(&ge, g, 0);
            cudaGraphDestroy(g);
            if (e3 != cudaSuccess) return sem_fail(SEM_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e3));
        }
        CUDA_TRY(cudaGraphLaunch(ge, s->stream));
        done += 2;
    }
    for (; done < n_steps; done++) {
        CUDA_TRY(solver_enqueue_step(s, s->cur));
        s->cur ^= 1;
        CUDA_TRY(enqueue_correction(a));
    }
    s->steps_done += n_steps;
    return SEM_OK;
    GUARD_END
}

int sem_abc_bptt(sem_abc *a, int n_steps, int n_roi, const int64_t *roi_nodes, const float *ref, double *loss,
                 float *grad)
{
    GUARD_BEGIN
    if (!a || n_steps < 1 || n_roi < 0 || (n_roi > 0 && (!roi_nodes || !ref)) || !loss)
        return sem_fail(SEM_ERR_ARG, "bad arguments");
    if (!a->face) return sem_fail(SEM_ERR_STATE, "the adjoint runs with the network on the boundary nodes (layer 0)");
    sem_solver *s = a->s;
    const Box &b = s->mesh->box;
    // sources must lie outside every boundary node's neighbourhood: the recorded levels do not
    // hold the source term a step adds before it reads them
    for (int64_t q : s->src_node) {
        const int64_t iy = q / (b.nxp * b.nz), r = q - iy * b.nxp * b.nz, iz = r / b.nxp, ix = r - iz * b.nxp;
        if (ix < 2 || ix > b.nx - 3 || iy < 2 || iy > b.ny - 3 || iz < 2 || iz > b.nz - 3)
            return sem_fail(SEM_ERR_ARG, "a source lies within two nodes of the boundary");
    }
    std::vector<int64_t> roi(n_roi);
    for (int r = 0; r < n_roi; r++) {
        if (roi_nodes[r] < 0 || roi_nodes[r] >= b.n_nodes) return sem_fail(SEM_ERR_ARG, "region node out of range");
        roi[r] = to_internal(b, roi_nodes[r]);
    }
    int rc = sem_solver_reset(s);
    if (rc) return rc;
    if ((rc = sem_abc_reset(a))) return rc;
    if ((rc = solver_prepare(s, n_steps))) return rc;
    const int64_t n_int = b.n_int, nb = a->n;
    cudaStream_t st = s->stream;

    // work arrays (freed on every exit path)
    float *rec = nullptr, *x = nullptr, *dx = nullptr, *scale = nullptr, *y = nullptr, *g = nullptr, *dy = nullptr;
    float *A[3] = {nullptr, nullptr, nullptr}, *v = nullptr, *dref = nullptr;
    int *kstar = nullptr, *sidx = nullptr;
    int64_t *droi = nullptr;
    double *dloss = nullptr, *dnull = nullptr;
    auto release = [&]() {
        cudaStreamSynchronize(st);
        dfree(rec); dfree(x); dfree(dx); dfree(scale); dfree(y); dfree(g); dfree(dy);
        for (auto &p : A) dfree(p);
        dfree(v); dfree(dref); dfree(kstar); dfree(sidx); dfree(droi); dfree(dloss); dfree(dnull);
    };
    cudaError_t e = dalloc(&rec, (size_t)(n_steps + 2) * n_int);
    if (e == cudaSuccess) e = dalloc(&x, (size_t)nb * kMlpIn);
    if (e == cudaSuccess) e = dalloc(&dx, (size_t)nb * kMlpIn);
    if (e == cudaSuccess) e = dalloc(&scale, (size_t)nb);
    if (e == cudaSuccess) e = dalloc(&y, (size_t)nb);
    if (e == cudaSuccess) e = dalloc(&g, (size_t)nb);
    if (e == cudaSuccess) e = dalloc(&dy, (size_t)nb);
    for (auto &p : A)
        if (e == cudaSuccess) e = dalloc(&p, (size_t)n_int);
    if (e == cudaSuccess) e = dalloc(&v, (size_t)n_int);
    if (e == cudaSuccess && n_roi > 0) e = dalloc(&dref, (size_t)n_steps * n_roi);
    if (e == cudaSuccess) e = dalloc(&kstar, (size_t)nb);
    if (e == cudaSuccess) e = dalloc(&sidx, (size_t)n_int);
    if (e == cudaSuccess && n_roi > 0) e = dalloc(&droi, (size_t)n_roi);
    if (e == cudaSuccess) e = dalloc(&dloss, 1);
    if (e == cudaSuccess) e = dalloc(&dnull, 1);
    if (e == cudaSuccess) {
        std::vector<int64_t> nodes(nb);
        e = cudaMemcpy(nodes.data(), a->d_nodes, nb * 8, cudaMemcpyDeviceToHost);
        std::vector<int> map(n_int, -1);
        for (int64_t i = 0; i < nb; i++) map[nodes[i]] = (int)i;
        if (e == cudaSuccess) e = cudaMemcpy(sidx, map.data(), n_int * 4, cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess && n_roi > 0) e = cudaMemcpy(droi, roi.data(), n_roi * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && n_roi > 0)
        e = cudaMemcpy(dref, ref, (size_t)n_steps * n_roi * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemsetAsync(dloss, 0, 8, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(rec, 0, 2 * n_int * 4, st);  // p^{-1} = p^0 = 0: from rest
    // forward, the levels after every step recorded
    for (int m = 1; m <= n_steps && e == cudaSuccess; m++) {
        e = solver_enqueue_step(s, s->cur);
        s->cur ^= 1;
        if (e == cudaSuccess) e = enqueue_correction(a);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(rec + (size_t)(m + 1) * n_int, s->d_p[s->cur], n_int * 4, cudaMemcpyDeviceToDevice, st);
    }
    s->steps_done += n_steps;
    BpttFields f{};
    f.nx = (int)b.nx; f.ny = (int)b.ny; f.nz = (int)b.nz;
    f.nxp = b.nxp; f.n_int = n_int;
    f.sx = s->sponge ? s->d_sx : nullptr;
    f.sy = s->sponge ? s->d_sy : nullptr;
    f.sz = s->sponge ? s->d_sz : nullptr;
    f.nodes = a->d_nodes; f.nb = nb; f.sidx = sidx;
    f.x = x; f.scale = scale; f.kstar = kstar; f.y = y; f.g = g; f.dy = dy; f.dx = dx;
    for (int k = 0; k < 3; k++) f.a[k] = A[k];
    f.v = v; f.roi = droi; f.n_roi = n_roi;
    for (auto p : A)
        if (e == cudaSuccess) e = cudaMemsetAsync(p, 0, n_int * 4, st);
    if (!grad) {
        // the loss only
        for (int m = 1; m <= n_steps && e == cudaSuccess; m++)
            e = bptt_loss(f, rec + (size_t)(m + 1) * n_int, dref + (size_t)(m - 1) * n_roi, dloss, st);
    } else {
        BpttOperator op{};
        op.order = b.order;
        Gll gl;
        gll_tables(b.order, gl);
        stencil_table(gl, op.T);
        const int W = 2 * b.order + 1;
        for (int l = 0; l < b.order; l++) {
            // the direct form's diagonal: minus the rounded row sum, as the stencil pass uses it
            double sum = 0;
            for (int d = -b.order; d <= b.order; d++)
                if (d != 0) sum += op.T[l * W + d + b.order];
            op.T[l * W + b.order] = (float)-sum;
            op.wa[l] = s->stencil->wa[l];
        }
        for (int k = 0; k < 3; k++) op.g[k] = s->stencil->g[k];
        sem_mlp *net = a->net;
        if (e == cudaSuccess) e = cudaMemsetAsync(net->d_grad, 0, kMlpParams * 4, st);
        for (int m = n_steps; m >= 1 && e == cudaSuccess; m--) {
            const float *lm = rec + (size_t)(m + 1) * n_int, *lm1 = rec + (size_t)m * n_int,
                        *lm2 = rec + (size_t)(m - 1) * n_int;
            e = bptt_loss(f, lm, dref + (size_t)(m - 1) * n_roi, dloss, st);
            if (e == cudaSuccess) e = bptt_features(f, lm, lm1, lm2, st);
            if (e == cudaSuccess) e = mlp_forward(net->dev(), x, y, nb, st);
            if (e == cudaSuccess) e = bptt_dy(f, st);
            if (e == cudaSuccess)
                e = mlp_loss_grad(net->dev(), x, nullptr, nb, dnull, net->d_grad, net->d_part, net->d_part_loss, st,
                                  dy, dx);
            if (e == cudaSuccess) e = bptt_scatter(f, st);
            if (e == cudaSuccess) e = bptt_interior(f, op, s->d_a, st);
            // the adjoints move one level back: out^{m-1} becomes the newest
            float *old = f.a[0];
            f.a[0] = f.a[1];
            f.a[1] = f.a[2];
            f.a[2] = old;
            if (e == cudaSuccess) e = cudaMemsetAsync(old, 0, n_int * 4, st);
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(grad, net->d_grad, kMlpParams * 4, cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(loss, dloss, 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    release();
    CUDA_TRY(e);
    return SEM_OK;
    GUARD_END
}

int sem_abc_correct(sem_abc *a)
{
    GUARD_BEGIN
    if (!a) return sem_fail(SEM_ERR_ARG, "NULL boundary");
    CUDA_TRY(enqueue_correction(a));
    return SEM_OK;
    GUARD_END
}

int sem_abc_features(sem_abc *a, float *x, float *scale)
{
    GUARD_BEGIN
    if (!a || !x) return sem_fail(SEM_ERR_ARG, "NULL argument");
    // the features exactly as k_abc_correction gathers them (same order, sponge product and
    // scaling), from host copies of the levels: training sets are built from these
    sem_solver *s = a->s;
    const Box &b = s->mesh->box;
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    std::vector<float> pn(b.n_int), pc(b.n_int), ph(b.n_int);
    CUDA_TRY(cudaMemcpy(pn.data(), s->d_p[s->cur], b.n_int * 4, cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(pc.data(), s->d_p[1 - s->cur], b.n_int * 4, cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(ph.data(), a->hist_now(), b.n_int * 4, cudaMemcpyDeviceToHost));
    std::vector<float> sx(b.nx, 1.f), sy(b.ny, 1.f), sz(b.nz, 1.f);
    if (s->sponge) {
        CUDA_TRY(cudaMemcpy(sx.data(), s->d_sx, b.nx * 4, cudaMemcpyDeviceToHost));
        CUDA_TRY(cudaMemcpy(sy.data(), s->d_sy, b.ny * 4, cudaMemcpyDeviceToHost));
        CUDA_TRY(cudaMemcpy(sz.data(), s->d_sz, b.nz * 4, cudaMemcpyDeviceToHost));
    }
    std::vector<int64_t> q(a->n);
    CUDA_TRY(cudaMemcpy(q.data(), a->d_nodes, a->n * 8, cudaMemcpyDeviceToHost));
    const int64_t plane = b.nxp * b.nz;
    for (int64_t i = 0; i < a->n; i++) {
        const int64_t iy = q[i] / plane, rr = q[i] - iy * plane, iz = rr / b.nxp, ix = rr - iz * b.nxp;
        float m = 0.f;
        float *f = x + i * kMlpIn;
        for (int l = 0; l < 3; l++)
            for (int nb = 0; nb < 27; nb++) {
                const int dz = nb / 9 - 1, dy = (nb / 3) % 3 - 1, dx = nb % 3 - 1;
                const int64_t jx = ix + dx, jy = iy + dy, jz = iz + dz;
                float v = 0.f;
                if (jx >= 0 && jx < b.nx && jy >= 0 && jy < b.ny && jz >= 0 && jz < b.nz) {
                    const int64_t qj = jx + jz * b.nxp + jy * plane;
                    v = l == 0 ? pn[qj] : l == 1 ? pc[qj] * ((sx[jx] * sy[jy]) * sz[jz]) : ph[qj];
                }
                f[l * 27 + nb] = v;
                m = std::max(m, std::fabs(v));
            }
        const float sc = m + 1e-30f;
        for (int k = 0; k < kMlpIn; k++) f[k] /= sc;
        if (scale) scale[i] = sc;
    }
    return SEM_OK;
    GUARD_END
}

}  // extern "C"
