// batch_api.cu -- C ABI of the many-shot form (sem_batch_*): shots that share one mesh, model,
// sponge and receiver set advance together.  The levels hold the shots' fields one after
// another and one stencil pass (k_stencil.cu, nshot > 1) steps them all: the CTAs of all shots
// of a tile run together, so each dt^2/M plane comes from DRAM once for the batch (12 + 4/S
// bytes per shot-node-step against 16).  The time loop is replayed from a captured CUDA graph;
// the autotuner times the y-chunk length.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "abi.h"
#include "batch.h"
#include "stencil.h"

using namespace semgb;

struct sem_batch {
    sem_mesh *mesh = nullptr;
    float dt = 0;
    int nshot = 0;
    int64_t n_int = 0;  // floats per shot field (device layout)
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    float *d_p[2] = {nullptr, nullptr};  // [nshot][n_int]: the shots' fields one after another
    int cur = 0;
    float *d_a = nullptr;
    uint64_t a_version = 0;
    double *d_w = nullptr;
    bool sponge = false;
    float *d_sx = nullptr, *d_sy = nullptr, *d_sz = nullptr;
    int nsamples = 0;
    int64_t *d_src_node = nullptr;
    float *d_src_coef = nullptr;
    float *d_wavelet = nullptr;
    int nrec = 0;
    std::vector<int64_t> rec_sorted;  // device-layout nodes, sorted
    int64_t *d_rec_node = nullptr;
    int *d_rec_perm = nullptr;
    uint64_t rec_version = 0;
    float *d_traces = nullptr;  // [cap][nrec][nshot]
    int64_t trace_cap = 0;
    int *d_ctr = nullptr;
    int *d_status = nullptr;
    int64_t steps_done = 0;
    StencilTables *st = nullptr;
    BatchTuning tune;
    bool tuned = false;
    cudaGraphExec_t graph2[2] = {nullptr, nullptr};
};

namespace {

void invalidate(sem_batch *b)
{
    for (auto &g : b->graph2)
        if (g) { cudaGraphExecDestroy(g); g = nullptr; }
}

StencilArgs args_for(const sem_batch *b, int c, bool record)
{
    StencilArgs a{};
    a.cur = b->d_p[c];
    a.prev = b->d_p[1 - c];
    a.sx = b->d_sx; a.sy = b->d_sy; a.sz = b->d_sz;
    a.rec_node = b->d_rec_node;
    a.rec_perm = b->d_rec_perm;
    a.rec_off = b->st->d_rec_off;
    a.rec_idx = b->st->d_rec_idx;
    a.nrec = record ? b->nrec : 0;
    a.traces = b->d_traces;
    a.ctr = b->d_ctr;
    a.status = b->d_status;
    return a;
}

cudaError_t enqueue(sem_batch *b, int c)
{
    BatchSourceArgs sa{b->d_p[c], b->d_src_node, b->d_src_coef, b->d_wavelet, b->nsamples > 0 ? b->nshot : 0,
                       b->nsamples, b->n_int, b->d_ctr};
    cudaError_t e = launch_batch_source(sa, b->d_ctr, b->stream);
    if (e != cudaSuccess) return e;
    return launch_stencil(*b->st, args_for(b, c, true), c, b->sponge, b->stream);
}

// Sets the stencil pass's y-chunk (planes per CTA) and regroups the receivers by CTA.
cudaError_t set_chunk(sem_batch *b, int ychunk)
{
    StencilTables &t = *b->st;
    t.ychunk = std::max(1, std::min<int>(ychunk, (int)t.ny));
    t.grid[2] = (int)((t.ny + t.ychunk - 1) / t.ychunk);
    return stencil_set_receivers(t, b->rec_sorted.data(), b->nrec, b->rec_version);
}

int prepare(sem_batch *b, int64_t n_new)
{
    sem_mesh *m = b->mesh;
    if (b->a_version != m->model_version) {
        CUDA_TRY(launch_mass(b->d_a, m->d_slow2 ? nullptr : m->d_vel, m->d_slow2, m->box.ex, m->box.ey, m->box.ez,
                             m->box.order, m->box.nxp, b->d_w, m->geo.detJ, (double)b->dt * b->dt, b->stream));
        b->a_version = m->model_version;
    }
    if (stencil_bind(*b->st, b->d_p[0], b->d_p[1], b->d_a) != 0)
        return sem_fail(SEM_ERR_CUDA, "tensor-map encoding failed (driver entry point cuTensorMapEncodeTiled)");
    if (b->st->rec_version != b->rec_version) {
        CUDA_TRY(stencil_set_receivers(*b->st, b->rec_sorted.data(), b->nrec, b->rec_version));
        invalidate(b);
    }
    if (b->nrec > 0 && b->steps_done + n_new > b->trace_cap) {
        const int64_t cap = std::max<int64_t>(b->steps_done + n_new, std::max<int64_t>(64, 2 * b->trace_cap));
        float *nt = nullptr;
        const size_t per = (size_t)b->nrec * b->nshot;
        CUDA_TRY(dalloc(&nt, (size_t)cap * per));
        CUDA_TRY(cudaMemsetAsync(nt, 0, (size_t)cap * per * 4, b->stream));
        if (b->d_traces && b->steps_done > 0)
            CUDA_TRY(cudaMemcpyAsync(nt, b->d_traces, (size_t)b->steps_done * per * 4, cudaMemcpyDeviceToDevice, b->stream));
        CUDA_TRY(cudaStreamSynchronize(b->stream));
        dfree(b->d_traces);
        b->d_traces = nt;
        b->trace_cap = cap;
        invalidate(b);
    }
    return SEM_OK;
}

// y-chunk lengths the autotuner tries: the stencil pass's own choice (it balances waves from the
// measured occupancy) and whole columns, halves and quarters.
std::vector<int> candidates(const sem_batch *b, int own)
{
    const int ny = (int)b->mesh->box.ny;
    std::vector<int> v{own};
    for (int div : {1, 2, 4}) {
        const int c = (ny + div - 1) / div;
        if (std::find(v.begin(), v.end(), c) == v.end()) v.push_back(c);
    }
    return v;
}

}  // namespace

extern "C" {

int sem_batch_destroy(sem_batch *b)
{
    if (!b) return SEM_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    invalidate(b);
    for (auto &p : b->d_p) dfree(p);
    dfree(b->d_a);
    dfree(b->d_w);
    dfree(b->d_sx); dfree(b->d_sy); dfree(b->d_sz);
    dfree(b->d_src_node); dfree(b->d_src_coef); dfree(b->d_wavelet);
    dfree(b->d_rec_node);
    dfree(b->d_rec_perm);
    dfree(b->d_traces);
    dfree(b->d_ctr);
    dfree(b->d_status);
    stencil_tables_free(b->st);
    if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return SEM_OK;
}

int sem_batch_create(sem_mesh *m, float dt, int n_shots, sem_batch **out)
{
    GUARD_BEGIN
    if (!m || !out) return sem_fail(SEM_ERR_ARG, "NULL argument");
    *out = nullptr;
    if (!(dt > 0) || n_shots < 1) return sem_fail(SEM_ERR_ARG, "dt must be positive and n_shots >= 1");
    sem_batch *b = new sem_batch();
    b->mesh = m;
    b->dt = dt;
    b->nshot = n_shots;
    b->n_int = m->box.n_int;
    auto cleanup = [&](int code, const std::string &msg) {
        sem_batch_destroy(b);
        return sem_fail(code, msg);
    };
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cleanup(SEM_ERR_CUDA, cudaGetErrorString(e));
    b->own_stream = true;
    const size_t n = (size_t)b->n_int * b->nshot;
    for (auto &p : b->d_p)
        if ((e = dalloc(&p, n)) != cudaSuccess || (e = cudaMemset(p, 0, n * 4)) != cudaSuccess)
            return cleanup(SEM_ERR_OOM, std::string("pressure levels: ") + cudaGetErrorString(e));
    if ((e = dalloc(&b->d_a, b->n_int)) != cudaSuccess || (e = cudaMemset(b->d_a, 0, b->n_int * 4)) != cudaSuccess)
        return cleanup(SEM_ERR_OOM, cudaGetErrorString(e));
    if ((e = dalloc(&b->d_ctr, 2)) != cudaSuccess || (e = cudaMemset(b->d_ctr, 0, 8)) != cudaSuccess)
        return cleanup(SEM_ERR_CUDA, cudaGetErrorString(e));
    if ((e = dalloc(&b->d_status, 1)) != cudaSuccess || (e = cudaMemset(b->d_status, 0, 4)) != cudaSuccess)
        return cleanup(SEM_ERR_CUDA, cudaGetErrorString(e));
    if ((e = dalloc(&b->d_w, m->box.order + 1)) != cudaSuccess ||
        (e = cudaMemcpy(b->d_w, m->gll.w, (m->box.order + 1) * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess)
        return cleanup(SEM_ERR_CUDA, cudaGetErrorString(e));
    if ((e = stencil_kernel_setup()) != cudaSuccess) return cleanup(SEM_ERR_CUDA, std::string("kernel set-up: ") + cudaGetErrorString(e));
    if (stencil_tables_create(m->box, m->gll, m->geo, n_shots, &b->st, kTileDefault) != 0) return cleanup(SEM_ERR_CUDA, "stencil tables");
    b->tune.warps_per_cta = b->st->threads / 32;
    b->tune.ychunk = b->st->ychunk;
    *out = b;
    return SEM_OK;
    GUARD_END
}

int sem_batch_set_stream(sem_batch *b, void *stream)
{
    if (!b) return sem_fail(SEM_ERR_ARG, "NULL batch");
    cudaStreamSynchronize(b->stream);
    invalidate(b);
    if (b->own_stream) cudaStreamDestroy(b->stream);
    if (stream) {
        b->stream = (cudaStream_t)stream;
        b->own_stream = false;
    } else {
        CUDA_TRY(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
        b->own_stream = true;
    }
    return SEM_OK;
}

int sem_batch_set_sponge_profile(sem_batch *b, const float *sx, const float *sy, const float *sz)
{
    GUARD_BEGIN
    if (!b) return sem_fail(SEM_ERR_ARG, "NULL batch");
    const Box &x = b->mesh->box;
    cudaStreamSynchronize(b->stream);
    invalidate(b);
    if (!sx || !sy || !sz) { b->sponge = false; return SEM_OK; }
    if (!b->d_sx) {
        CUDA_TRY(dalloc(&b->d_sx, x.nx));
        CUDA_TRY(dalloc(&b->d_sy, x.ny));
        CUDA_TRY(dalloc(&b->d_sz, x.nz));
    }
    CUDA_TRY(cudaMemcpy(b->d_sx, sx, x.nx * 4, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(b->d_sy, sy, x.ny * 4, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(b->d_sz, sz, x.nz * 4, cudaMemcpyHostToDevice));
    b->sponge = true;
    return SEM_OK;
    GUARD_END
}

int sem_batch_set_sponge(sem_batch *b, int thickness, float sigma)
{
    GUARD_BEGIN
    if (!b) return sem_fail(SEM_ERR_ARG, "NULL batch");
    if (thickness < 0 || !(sigma >= 0)) return sem_fail(SEM_ERR_ARG, "bad sponge parameters");
    if (thickness == 0) return sem_batch_set_sponge_profile(b, nullptr, nullptr, nullptr);
    std::vector<float> x, y, z;
    box_sponge_profile(b->mesh->box, b->mesh->gll, thickness, sigma, x, y, z);
    return sem_batch_set_sponge_profile(b, x.data(), y.data(), z.data());
    GUARD_END
}

int sem_batch_set_sources(sem_batch *b, const int64_t *elements, const float *wavelet, int n_samples)
{
    GUARD_BEGIN
    if (!b || !elements || (n_samples > 0 && !wavelet) || n_samples < 0) return sem_fail(SEM_ERR_ARG, "bad source arrays");
    const Box &x = b->mesh->box;
    std::vector<float> vel(x.n_elem);
    CUDA_TRY(cudaMemcpy(vel.data(), b->mesh->d_vel, x.n_elem * 4, cudaMemcpyDeviceToHost));
    std::vector<int64_t> node(b->nshot);
    std::vector<float> coef(b->nshot);
    for (int s = 0; s < b->nshot; s++) {
        if (elements[s] < 0) { node[s] = -1; coef[s] = 0.f; continue; }  // a shot without source
        if (elements[s] >= x.n_elem) return sem_fail(SEM_ERR_ARG, "source element out of range");
        node[s] = to_internal(x, box_node(x, elements[s], 0));
        const float c = vel[elements[s]];
        coef[s] = b->dt * b->dt * c * c;  // as SEMsolver.cpp:41-42 rounds it
    }
    cudaStreamSynchronize(b->stream);
    invalidate(b);
    dfree(b->d_src_node); dfree(b->d_src_coef); dfree(b->d_wavelet);
    CUDA_TRY(dalloc(&b->d_src_node, b->nshot));
    CUDA_TRY(dalloc(&b->d_src_coef, b->nshot));
    CUDA_TRY(cudaMemcpy(b->d_src_node, node.data(), b->nshot * 8, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(b->d_src_coef, coef.data(), b->nshot * 4, cudaMemcpyHostToDevice));
    b->nsamples = n_samples;
    if (n_samples > 0) {
        CUDA_TRY(dalloc(&b->d_wavelet, (size_t)b->nshot * n_samples));
        CUDA_TRY(cudaMemcpy(b->d_wavelet, wavelet, (size_t)b->nshot * n_samples * 4, cudaMemcpyHostToDevice));
    }
    return SEM_OK;
    GUARD_END
}

int sem_batch_set_source_points(sem_batch *b, const float *xyz, const float *wavelet, int n_samples)
{
    GUARD_BEGIN
    if (!b || !xyz) return sem_fail(SEM_ERR_ARG, "NULL argument");
    std::vector<int64_t> el(b->nshot);
    for (int s = 0; s < b->nshot; s++) el[s] = box_element_from_point(b->mesh->box, xyz[3 * s], xyz[3 * s + 1], xyz[3 * s + 2]);
    return sem_batch_set_sources(b, el.data(), wavelet, n_samples);
    GUARD_END
}

int sem_batch_set_receiver_nodes(sem_batch *b, int n_rec, const int64_t *nodes)
{
    GUARD_BEGIN
    if (!b || n_rec < 0 || (n_rec > 0 && !nodes)) return sem_fail(SEM_ERR_ARG, "bad receiver array");
    if (b->steps_done > 0) return sem_fail(SEM_ERR_STATE, "receivers must be set before the first step");
    for (int r = 0; r < n_rec; r++)
        if (nodes[r] < 0 || nodes[r] >= b->mesh->box.n_nodes) return sem_fail(SEM_ERR_ARG, "receiver node out of range");
    // node-sorted (the stencil pass groups them by owning CTA); perm maps back to the caller's order
    std::vector<int> perm(n_rec);
    std::iota(perm.begin(), perm.end(), 0);
    std::stable_sort(perm.begin(), perm.end(), [&](int x, int y) { return nodes[x] < nodes[y]; });
    std::vector<int64_t> sorted(n_rec);
    for (int r = 0; r < n_rec; r++) sorted[r] = to_internal(b->mesh->box, nodes[perm[r]]);
    cudaStreamSynchronize(b->stream);
    invalidate(b);
    dfree(b->d_rec_node);
    dfree(b->d_rec_perm);
    dfree(b->d_traces);
    b->trace_cap = 0;
    b->nrec = n_rec;
    b->rec_sorted = sorted;
    b->rec_version++;
    if (n_rec > 0) {
        CUDA_TRY(dalloc(&b->d_rec_node, n_rec));
        CUDA_TRY(dalloc(&b->d_rec_perm, n_rec));
        CUDA_TRY(cudaMemcpy(b->d_rec_node, sorted.data(), n_rec * 8, cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(b->d_rec_perm, perm.data(), n_rec * 4, cudaMemcpyHostToDevice));
    }
    return SEM_OK;
    GUARD_END
}

int sem_batch_set_receivers(sem_batch *b, int n_rec, const float *xyz)
{
    GUARD_BEGIN
    if (!b || (n_rec > 0 && !xyz)) return sem_fail(SEM_ERR_ARG, "NULL argument");
    std::vector<int64_t> nodes(std::max(n_rec, 0));
    for (int r = 0; r < n_rec; r++)
        nodes[r] = box_nearest_node(b->mesh->box, b->mesh->gll, xyz[3 * r], xyz[3 * r + 1], xyz[3 * r + 2]);
    return sem_batch_set_receiver_nodes(b, n_rec, nodes.data());
    GUARD_END
}

int sem_batch_step(sem_batch *b, int n_steps)
{
    GUARD_BEGIN
    if (!b || n_steps < 0) return sem_fail(SEM_ERR_ARG, "bad arguments");
    if (n_steps == 0) return SEM_OK;
    int rc = prepare(b, n_steps);
    if (rc) return rc;
    int done = 0;
    while (n_steps - done >= 2) {
        if (!b->graph2[b->cur]) {
            cudaGraph_t g = nullptr;
            CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
            cudaError_t e1 = enqueue(b, b->cur);
            cudaError_t e2 = e1 == cudaSuccess ? enqueue(b, 1 - b->cur) : e1;
            cudaError_t e3 = cudaStreamEndCapture(b->stream, &g);
            if (e2 != cudaSuccess || e3 != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                return sem_fail(SEM_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e2 != cudaSuccess ? e2 : e3));
            }
            cudaError_t e4 = cudaGraphInstantiate(&b->graph2[b->cur], g, 0);
            cudaGraphDestroy(g);
            if (e4 != cudaSuccess) return sem_fail(SEM_ERR_CUDA, cudaGetErrorString(e4));
        }
        CUDA_TRY(cudaGraphLaunch(b->graph2[b->cur], b->stream));
        done += 2;
    }
    if (done < n_steps) {
        CUDA_TRY(enqueue(b, b->cur));
        b->cur ^= 1;
    }
    b->steps_done += n_steps;
    return SEM_OK;
    GUARD_END
}

int sem_batch_synchronize(sem_batch *b)
{
    if (!b) return sem_fail(SEM_ERR_ARG, "NULL batch");
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    int status = 0;
    CUDA_TRY(cudaMemcpy(&status, b->d_status, 4, cudaMemcpyDeviceToHost));
    if (status != 0) return sem_fail(SEM_ERR_TIMEOUT, "a bounded device wait gave up (TMA copy not completed)");
    return SEM_OK;
}

int sem_batch_get_traces(sem_batch *b, float *out)
{
    GUARD_BEGIN
    if (!b) return sem_fail(SEM_ERR_ARG, "NULL batch");
    if (b->nrec == 0 || b->steps_done == 0) return SEM_OK;
    if (!out) return sem_fail(SEM_ERR_ARG, "NULL output");
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    CUDA_TRY(cudaMemcpy(out, b->d_traces, (size_t)b->steps_done * b->nrec * b->nshot * 4, cudaMemcpyDeviceToHost));
    return SEM_OK;
    GUARD_END
}

int sem_batch_get_pressure(sem_batch *b, int shot, int level, float *out)
{
    GUARD_BEGIN
    if (!b || !out || shot < 0 || shot >= b->nshot) return sem_fail(SEM_ERR_ARG, "bad arguments");
    if (level != SEM_LEVEL_CURRENT && level != SEM_LEVEL_PREVIOUS) return sem_fail(SEM_ERR_ARG, "bad level");
    const Box &x = b->mesh->box;
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    const int idx = level == SEM_LEVEL_CURRENT ? b->cur : 1 - b->cur;
    // one shot is one contiguous field of the level; drop the row padding
    std::vector<float> col((size_t)x.n_int);
    CUDA_TRY(cudaMemcpy(col.data(), b->d_p[idx] + (size_t)shot * b->n_int, (size_t)x.n_int * 4, cudaMemcpyDeviceToHost));
    int64_t i = 0;
    for (int64_t r = 0; r < x.nz * x.ny; r++)
        for (int64_t c = 0; c < x.nx; c++) out[i++] = col[(size_t)r * x.nxp + c];
    if (level == SEM_LEVEL_PREVIOUS && b->sponge) {
        std::vector<float> sx(x.nx), sy(x.ny), sz(x.nz);
        CUDA_TRY(cudaMemcpy(sx.data(), b->d_sx, x.nx * 4, cudaMemcpyDeviceToHost));
        CUDA_TRY(cudaMemcpy(sy.data(), b->d_sy, x.ny * 4, cudaMemcpyDeviceToHost));
        CUDA_TRY(cudaMemcpy(sz.data(), b->d_sz, x.nz * 4, cudaMemcpyDeviceToHost));
        i = 0;
        for (int64_t iy = 0; iy < x.ny; iy++)
            for (int64_t iz = 0; iz < x.nz; iz++)
                for (int64_t ix = 0; ix < x.nx; ix++, i++) out[i] = (sx[ix] * sy[iy] * sz[iz]) * out[i];
    }
    return SEM_OK;
    GUARD_END
}

int sem_batch_time_step(sem_batch *b, int n_steps, float *ms_per_step)
{
    GUARD_BEGIN
    if (!b || !ms_per_step || n_steps < 1) return sem_fail(SEM_ERR_ARG, "bad arguments");
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    int rc = prepare(b, n_steps);
    if (rc == SEM_OK) {
        cudaEventRecord(e0, b->stream);
        rc = sem_batch_step(b, n_steps);
        cudaEventRecord(e1, b->stream);
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

int sem_batch_autotune(sem_batch *b, int *shots_per_cluster, int *warps_per_cta, int *ychunk)
{
    GUARD_BEGIN
    if (!b) return sem_fail(SEM_ERR_ARG, "NULL batch");
    // time every candidate on the current levels; a step only writes the previous level, which
    // is saved first and restored after, and the trials record no traces
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    int rc = prepare(b, 0);
    if (rc) return rc;
    const size_t n = (size_t)b->n_int * b->nshot;
    float *keep = nullptr;
    CUDA_TRY(dalloc(&keep, n));
    CUDA_TRY(cudaMemcpyAsync(keep, b->d_p[1 - b->cur], n * 4, cudaMemcpyDeviceToDevice, b->stream));
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    float best = 1e30f;
    int pick = b->st->ychunk, pick_cluster = b->st->cluster;
    const std::vector<int> chunks = candidates(b, b->st->ychunk);
    for (int cl : {1, 2, 4, 8}) {
        if (b->nshot % cl != 0) continue;
        b->st->cluster = cl;
        for (int chunk : chunks) {
            cudaError_t err = set_chunk(b, chunk);
            const StencilArgs a = args_for(b, b->cur, false);
            if (err == cudaSuccess) err = launch_stencil(*b->st, a, b->cur, b->sponge, b->stream);  // warm-up
            cudaEventRecord(e0, b->stream);
            for (int r = 0; r < 3 && err == cudaSuccess; r++) err = launch_stencil(*b->st, a, b->cur, b->sponge, b->stream);
            cudaEventRecord(e1, b->stream);
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (err != cudaSuccess) cudaGetLastError();  // a shape the device cannot launch: skipped
            else if (ms < best) { best = ms; pick = b->st->ychunk; pick_cluster = cl; }
        }
    }
    b->st->cluster = pick_cluster;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    CUDA_TRY(cudaMemcpyAsync(b->d_p[1 - b->cur], keep, n * 4, cudaMemcpyDeviceToDevice, b->stream));
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    dfree(keep);
    CUDA_TRY(set_chunk(b, pick));
    b->tune.ychunk = pick;
    b->tune.shots_per_cluster = pick_cluster;
    b->tuned = true;
    invalidate(b);
    if (shots_per_cluster) *shots_per_cluster = b->tune.shots_per_cluster;
    if (warps_per_cta) *warps_per_cta = b->tune.warps_per_cta;
    if (ychunk) *ychunk = pick;
    return SEM_OK;
    GUARD_END
}

}  // extern "C"
