// api.cu -- the C ABI (include/semgb.h): mesh and model set-up, solver state, the time loop
// (replayed from captured CUDA graphs), source and receiver I/O.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include "abi.h"
#include "solver.h"
#include "stencil.h"
#include "tma.cuh"

using namespace semgb;

static thread_local std::string g_err;

namespace semgb {
// Sets the message sem_last_error_string() returns (for entry points defined in other files).
void set_last_error(const std::string &msg) { g_err = msg; }
}  // namespace semgb

static int fail(int code, const std::string &msg) { return sem_fail(code, msg); }

void solver_invalidate_graphs(sem_solver *s)
{
    s->graph_gen++;
    for (auto &g : s->graph2)
        if (g) { cudaGraphExecDestroy(g); g = nullptr; }
}

namespace {

// Pinned staging for field_to_host / field_from_host, one set per device (its events must live
// on the device of the stream they are recorded on); allocated on first use on that device and
// kept for the life of the process; calls from several threads take turns.
struct Staging {
    static constexpr int64_t kFloats = int64_t(4) << 20;  // 16 MB per buffer
    std::mutex mu;
    int device = -1;
    float *buf[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaError_t init()
    {
        if (device < 0) return cudaErrorInvalidDevice;
        int prev = 0;
        cudaError_t e = cudaGetDevice(&prev);
        if (e == cudaSuccess && prev != device) e = cudaSetDevice(device);
        for (int k = 0; k < 2 && e == cudaSuccess; k++) {
            if (!buf[k]) e = cudaHostAlloc(reinterpret_cast<void **>(&buf[k]), kFloats * 4, cudaHostAllocDefault);
            if (e == cudaSuccess && !ev[k]) e = cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming);
        }
        if (prev != device) cudaSetDevice(prev);
        return e;
    }
};

constexpr int kMaxStagingDevices = 64;

// The staging of the device that stream s belongs to (null if that device cannot be told).
Staging *staging(cudaStream_t s)
{
    static Staging st[kMaxStagingDevices];
    int dev = -1;
    if (cudaStreamGetDevice(s, &dev) != cudaSuccess) {
        cudaGetLastError();
        if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    }
    if (dev < 0 || dev >= kMaxStagingDevices) return nullptr;
    st[dev].device = dev;
    return &st[dev];
}

}  // namespace

cudaError_t field_to_host(float *dst, const float *src, int64_t nx, int64_t nxp, int64_t rows, cudaStream_t s)
{
    Staging *stp = staging(s);
    if (!stp) {
        cudaGetLastError();
        cudaError_t e = cudaMemcpy2DAsync(dst, nx * 4, src, nxp * 4, nx * 4, rows, cudaMemcpyDeviceToHost, s);
        return e == cudaSuccess ? cudaStreamSynchronize(s) : e;
    }
    Staging &st = *stp;
    std::lock_guard<std::mutex> lock(st.mu);
    if (nx > Staging::kFloats || st.init() != cudaSuccess) {
        cudaGetLastError();
        cudaError_t e = cudaMemcpy2DAsync(dst, nx * 4, src, nxp * 4, nx * 4, rows, cudaMemcpyDeviceToHost, s);
        return e == cudaSuccess ? cudaStreamSynchronize(s) : e;
    }
    const int64_t per = Staging::kFloats / nx;  // rows per chunk
    int64_t prev_r0 = -1, prev_n = 0;
    int k = 0, prev_k = 0;
    cudaError_t e = cudaSuccess;
    for (int64_t r0 = 0; r0 < rows; r0 += per, k ^= 1) {
        // buffer k was emptied by the host during the previous chunk
        const int64_t n = std::min(per, rows - r0);
        if ((e = cudaMemcpy2DAsync(st.buf[k], nx * 4, src + r0 * nxp, nxp * 4, nx * 4, n, cudaMemcpyDeviceToHost,
                                   s)) != cudaSuccess ||
            (e = cudaEventRecord(st.ev[k], s)) != cudaSuccess)
            break;
        if (prev_r0 >= 0) {
            if ((e = cudaEventSynchronize(st.ev[prev_k])) != cudaSuccess) break;
            std::memcpy(dst + prev_r0 * nx, st.buf[prev_k], (size_t)(prev_n * nx) * 4);
        }
        prev_r0 = r0; prev_n = n; prev_k = k;
    }
    if (e == cudaSuccess && prev_r0 >= 0 && (e = cudaEventSynchronize(st.ev[prev_k])) == cudaSuccess)
        std::memcpy(dst + prev_r0 * nx, st.buf[prev_k], (size_t)(prev_n * nx) * 4);
    if (e != cudaSuccess) cudaStreamSynchronize(s);  // leave no copy into the staging in flight
    return e;
}

cudaError_t field_from_host(float *dst, const float *src, int64_t nx, int64_t nxp, int64_t rows, cudaStream_t s)
{
    Staging *stp = staging(s);
    if (!stp) {
        cudaGetLastError();
        cudaError_t e = cudaMemcpy2DAsync(dst, nxp * 4, src, nx * 4, nx * 4, rows, cudaMemcpyHostToDevice, s);
        return e == cudaSuccess ? cudaStreamSynchronize(s) : e;
    }
    Staging &st = *stp;
    std::lock_guard<std::mutex> lock(st.mu);
    if (nx > Staging::kFloats || st.init() != cudaSuccess) {
        cudaGetLastError();
        cudaError_t e = cudaMemcpy2DAsync(dst, nxp * 4, src, nx * 4, nx * 4, rows, cudaMemcpyHostToDevice, s);
        return e == cudaSuccess ? cudaStreamSynchronize(s) : e;
    }
    const int64_t per = Staging::kFloats / nx;
    bool used[2] = {false, false};
    int k = 0;
    cudaError_t e = cudaSuccess;
    for (int64_t r0 = 0; r0 < rows; r0 += per, k ^= 1) {
        const int64_t n = std::min(per, rows - r0);
        // the copy that last read buffer k (two chunks ago) must be done before it is refilled
        if (used[k] && (e = cudaEventSynchronize(st.ev[k])) != cudaSuccess) break;
        std::memcpy(st.buf[k], src + r0 * nx, (size_t)(n * nx) * 4);
        if ((e = cudaMemcpy2DAsync(dst + r0 * nxp, nxp * 4, st.buf[k], nx * 4, nx * 4, n, cudaMemcpyHostToDevice,
                                   s)) != cudaSuccess ||
            (e = cudaEventRecord(st.ev[k], s)) != cudaSuccess)
            break;
        used[k] = true;
    }
    const cudaError_t es = cudaStreamSynchronize(s);
    return e != cudaSuccess ? e : es;
}

static int resolved_kernel(const sem_solver *s)
{
    return s->kernel == SEM_KERNEL_AUTO ? SEM_KERNEL_STENCIL : s->kernel;
}

int solver_set_raw_sources(sem_solver *s, int n_src, const int64_t *nodes, const float *coef, const float *wavelet,
                           int n_samples)
{
    cudaStreamSynchronize(s->stream);
    solver_invalidate_graphs(s);
    dfree(s->d_src_node);
    dfree(s->d_src_coef);
    dfree(s->d_wavelet);
    s->nsrc = n_src;
    s->nsamples = n_samples;
    s->src_node.assign(nodes, nodes + n_src);
    s->src_coef.assign(coef, coef + n_src);
    std::vector<int64_t> sorted(nodes, nodes + n_src);
    std::sort(sorted.begin(), sorted.end());
    s->src_distinct = std::adjacent_find(sorted.begin(), sorted.end()) == sorted.end();
    if (n_src > 0) {
        CUDA_TRY(dalloc(&s->d_src_node, n_src));
        CUDA_TRY(dalloc(&s->d_src_coef, n_src));
        CUDA_TRY(cudaMemcpy(s->d_src_node, nodes, n_src * 8, cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(s->d_src_coef, coef, n_src * 4, cudaMemcpyHostToDevice));
        if (n_samples > 0) {
            CUDA_TRY(dalloc(&s->d_wavelet, (size_t)n_src * n_samples));
            CUDA_TRY(cudaMemcpy(s->d_wavelet, wavelet, (size_t)n_src * n_samples * 4, cudaMemcpyHostToDevice));
        }
    }
    return SEM_OK;
}

namespace {

// One CTA waits on an mbarrier phase that nothing completes (no arrival, no copy), so the
// bounded wait can only end at its limit; thread 0 reports the outcome and the time waited.
__global__ void k_wait_selftest(uint64_t limit_ns, int *status, unsigned long long *waited_ns)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        semgb::bar_init(&bar, 1);
        semgb::fence_barrier_init();
    }
    __syncthreads();
    const uint64_t t0 = semgb::global_ns();
    const bool done = semgb::bar_wait(&bar, 0, limit_ns);
    if (threadIdx.x == 0) {
        *status = done ? 0 : 1;
        *waited_ns = (unsigned long long)(semgb::global_ns() - t0);
    }
}

}  // namespace

extern "C" {

const char *sem_last_error_string(void) { return g_err.c_str(); }

int sem_version(void) { return 100; }

int sem_selftest_bounded_wait(double limit_seconds, double *waited_seconds)
{
    if (!(limit_seconds > 0) || limit_seconds > 2.0) return fail(SEM_ERR_ARG, "limit_seconds must be in (0, 2]");
    int *d_status = nullptr;
    unsigned long long *d_ns = nullptr;
    CUDA_TRY(dalloc(&d_status, 1));
    cudaError_t e = dalloc(&d_ns, 1);
    if (e == cudaSuccess) {
        k_wait_selftest<<<1, 32>>>((uint64_t)(limit_seconds * 1e9), d_status, d_ns);
        e = cudaGetLastError();
    }
    int status = 0;
    unsigned long long ns = 0;
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(&status, d_status, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&ns, d_ns, sizeof(ns), cudaMemcpyDeviceToHost);
    dfree(d_status);
    dfree(d_ns);
    if (e != cudaSuccess) return fail(SEM_ERR_CUDA, cudaGetErrorString(e));
    if (waited_seconds) *waited_seconds = ns * 1e-9;
    if (status != 0) return fail(SEM_ERR_TIMEOUT, "bounded wait gave up at its limit (self-test)");
    return SEM_OK;
}

// ----------------------------------------------------------------------------------------------
// host-only utilities
// ----------------------------------------------------------------------------------------------

int sem_gll_tables(int order, double *xi, double *w, double *dphi)
{
    Gll g;
    if (!gll_tables(order, g)) return fail(SEM_ERR_ARG, "order must be 1..5");
    const int o1 = order + 1;
    if (xi) std::copy(g.xi, g.xi + o1, xi);
    if (w) std::copy(g.w, g.w + o1, w);
    if (dphi) std::copy(g.dphi, g.dphi + o1 * o1, dphi);
    return SEM_OK;
}

int sem_ricker(int nsamples, float dt, float f0, int order, float *out)
{
    if (nsamples < 0 || (nsamples > 0 && !out)) return fail(SEM_ERR_ARG, "bad buffer");
    if (order < 0 || order > 2) return fail(SEM_ERR_ARG, "Ricker order must be 0, 1 or 2");
    if (!(f0 > 0)) return fail(SEM_ERR_ARG, "f0 must be positive");
    for (int i = 0; i < nsamples; i++) out[i] = ricker(i * dt, f0, order);
    return SEM_OK;
}

int sem_box_counts(int ex, int ey, int ez, int order, int64_t *n_nodes, int64_t *n_elem,
                   int64_t *n_interior)
{
    Box b;
    if (!make_box(ex, ey, ez, 1.f, 1.f, 1.f, order, b)) return fail(SEM_ERR_ARG, "bad box");
    if (n_nodes) *n_nodes = b.n_nodes;
    if (n_elem) *n_elem = b.n_elem;
    if (n_interior) *n_interior = b.n_interior;
    return SEM_OK;
}

int sem_box_connectivity(int ex, int ey, int ez, int order, int64_t e0, int64_t count,
                         int64_t *conn)
{
    Box b;
    if (!make_box(ex, ey, ez, 1.f, 1.f, 1.f, order, b)) return fail(SEM_ERR_ARG, "bad box");
    if (e0 < 0 || count < 0 || e0 + count > b.n_elem || (count > 0 && !conn))
        return fail(SEM_ERR_ARG, "element range out of bounds");
    for (int64_t e = 0; e < count; e++)
        for (int l = 0; l < b.npe; l++) conn[e * b.npe + l] = box_node(b, e0 + e, l);
    return SEM_OK;
}

int sem_box_element_from_point(int ex, int ey, int ez, float lx, float ly, float lz, float x,
                               float y, float z, int64_t *element)
{
    Box b;
    if (!make_box(ex, ey, ez, lx, ly, lz, 1, b) || !element) return fail(SEM_ERR_ARG, "bad box");
    *element = box_element_from_point(b, x, y, z);
    return SEM_OK;
}

int sem_box_nearest_node(int ex, int ey, int ez, float lx, float ly, float lz, int order,
                         float x, float y, float z, int64_t *node)
{
    Box b;
    Gll g;
    if (!make_box(ex, ey, ez, lx, ly, lz, order, b) || !gll_tables(order, g) || !node)
        return fail(SEM_ERR_ARG, "bad box");
    *node = box_nearest_node(b, g, x, y, z);
    return SEM_OK;
}

int sem_box_sponge_profile(int ex, int ey, int ez, float lx, float ly, float lz, int order,
                           int thickness, float sigma, float *sx, float *sy, float *sz)
{
    GUARD_BEGIN
    Box b;
    Gll g;
    if (!make_box(ex, ey, ez, lx, ly, lz, order, b) || !gll_tables(order, g))
        return fail(SEM_ERR_ARG, "bad box");
    if (thickness < 0 || !(sigma >= 0) || !sx || !sy || !sz) return fail(SEM_ERR_ARG, "bad sponge");
    std::vector<float> a, bb, c;
    box_sponge_profile(b, g, thickness, sigma, a, bb, c);
    std::copy(a.begin(), a.end(), sx);
    std::copy(bb.begin(), bb.end(), sy);
    std::copy(c.begin(), c.end(), sz);
    return SEM_OK;
    GUARD_END
}

int sem_box_refround_rows(int ex, int ey, int ez, float lx, float ly, float lz, int order, float *rows)
{
    GUARD_BEGIN
    Box b;
    Gll g;
    if (!make_box(ex, ey, ez, lx, ly, lz, order, b) || !gll_tables(order, g) || !rows)
        return fail(SEM_ERR_ARG, "bad box");
    std::vector<float> r;
    reference_element_rows(g, 0.5 * lx / ex, 0.5 * lz / ez, 0.5 * ly / ey, r);
    std::copy(r.begin(), r.end(), rows);
    return SEM_OK;
    GUARD_END
}

int sem_box_refround_class_table(int ex, int ey, int ez, float lx, float ly, float lz, int order, float *tab)
{
    GUARD_BEGIN
    Box b;
    Gll g;
    if (!make_box(ex, ey, ez, lx, ly, lz, order, b) || !gll_tables(order, g) || !tab)
        return fail(SEM_ERR_ARG, "bad box");
    std::vector<float> t;
    reference_class_table(g, 0.5 * lx / ex, 0.5 * lz / ez, 0.5 * ly / ey, t);
    std::copy(t.begin(), t.end(), tab);
    return SEM_OK;
    GUARD_END
}

// ----------------------------------------------------------------------------------------------
// mesh and model
// ----------------------------------------------------------------------------------------------

int sem_mesh_create_box(int ex, int ey, int ez, float lx, float ly, float lz, int order,
                        sem_mesh **out)
{
    GUARD_BEGIN
    if (!out) return fail(SEM_ERR_ARG, "out is NULL");
    *out = nullptr;
    sem_mesh *m = new sem_mesh();
    if (!make_box(ex, ey, ez, lx, ly, lz, order, m->box) || !gll_tables(order, m->gll)) {
        delete m;
        return fail(SEM_ERR_ARG, "box needs ex,ey,ez >= 1, positive lengths and order 1..5");
    }
    const double jx = 0.5 * lx / ex, jz = 0.5 * lz / ez, jy = 0.5 * ly / ey;
    m->geo.detJ = jx * jz * jy;
    m->geo.g[0] = m->geo.detJ / (jx * jx);
    m->geo.g[1] = m->geo.detJ / (jz * jz);
    m->geo.g[2] = m->geo.detJ / (jy * jy);
    cudaGetDevice(&m->device);
    cudaError_t e = dalloc(&m->d_vel, m->box.n_elem);
    if (e == cudaSuccess) {
        std::vector<float> v(m->box.n_elem, 1500.0f);  // SEMmesh::getModel
        e = cudaMemcpy(m->d_vel, v.data(), v.size() * sizeof(float), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) {
        dfree(m->d_vel);
        delete m;
        return fail(e == cudaErrorMemoryAllocation ? SEM_ERR_OOM : SEM_ERR_CUDA,
                    std::string("mesh allocation: ") + cudaGetErrorString(e));
    }
    *out = m;
    return SEM_OK;
    GUARD_END
}

int sem_mesh_destroy(sem_mesh *m)
{
    if (!m) return SEM_OK;
    dfree(m->d_vel);
    dfree(m->d_slow2);
    dfree(m->d_conn);
    delete m;
    return SEM_OK;
}

int sem_mesh_info(const sem_mesh *m, int64_t *n_nodes, int64_t *n_elem, int *npe,
                  int64_t *n_interior)
{
    if (!m) return fail(SEM_ERR_ARG, "mesh is NULL");
    if (n_nodes) *n_nodes = m->box.n_nodes;
    if (n_elem) *n_elem = m->box.n_elem;
    if (npe) *npe = m->box.npe;
    if (n_interior) *n_interior = m->box.n_interior;
    return SEM_OK;
}

static int ensure_conn(sem_mesh *m, cudaStream_t s)
{
    if (m->d_conn) return SEM_OK;
    if (m->box.n_int > 0x7fffffffLL)
        return fail(SEM_ERR_ARG, "element kernel needs fewer than 2^31 nodes (int32 connectivity)");
    CUDA_TRY(dalloc(&m->d_conn, (size_t)m->box.n_elem * m->box.npe));
    CUDA_TRY(launch_connectivity(m->d_conn, m->box.ex, m->box.ey, m->box.ez, m->box.order, m->box.nxp, s));
    return SEM_OK;
}

int sem_mesh_get_connectivity(sem_mesh *m, int32_t *conn)
{
    GUARD_BEGIN
    if (!m || !conn) return fail(SEM_ERR_ARG, "NULL argument");
    int rc = ensure_conn(m, 0);
    if (rc) return rc;
    const size_t n = (size_t)m->box.n_elem * m->box.npe;
    CUDA_TRY(cudaMemcpy(conn, m->d_conn, n * sizeof(int32_t), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; i++) conn[i] = (int32_t)to_reference(m->box, conn[i]);  // device -> reference numbering
    return SEM_OK;
    GUARD_END
}

int sem_model_set_element_velocity(sem_mesh *m, const float *vel)
{
    GUARD_BEGIN
    if (!m || !vel) return fail(SEM_ERR_ARG, "NULL argument");
    for (int64_t e = 0; e < m->box.n_elem; e++)
        if (!(vel[e] > 0) || !std::isfinite(vel[e]))
            return fail(SEM_ERR_ARG, "velocities must be positive and finite (element " +
                                         std::to_string(e) + ")");
    CUDA_TRY(cudaMemcpy(m->d_vel, vel, m->box.n_elem * sizeof(float), cudaMemcpyHostToDevice));
    dfree(m->d_slow2);
    m->model_version++;
    return SEM_OK;
    GUARD_END
}

int sem_model_set_node_slowness2(sem_mesh *m, const float *s2)
{
    GUARD_BEGIN
    if (!m || !s2) return fail(SEM_ERR_ARG, "NULL argument");
    for (int64_t i = 0; i < m->box.n_nodes; i++)
        if (!(s2[i] > 0) || !std::isfinite(s2[i]))
            return fail(SEM_ERR_ARG, "squared slowness must be positive and finite");
    if (!m->d_slow2) {
        CUDA_TRY(dalloc(&m->d_slow2, m->box.n_int));
        CUDA_TRY(cudaMemset(m->d_slow2, 0, m->box.n_int * 4));
    }
    CUDA_TRY(field_from_host(m->d_slow2, s2, m->box.nx, m->box.nxp, m->box.nz * m->box.ny, 0));
    m->model_version++;
    return SEM_OK;
    GUARD_END
}

// ----------------------------------------------------------------------------------------------
// solver
// ----------------------------------------------------------------------------------------------

int sem_solver_destroy(sem_solver *s)
{
    if (!s) return SEM_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    solver_invalidate_graphs(s);
    for (auto &p : s->d_p) dfree(p);
    dfree(s->d_y);
    dfree(s->d_a);
    dfree(s->d_tab);
    dfree(s->d_rtab);
    dfree(s->d_mref);
    dfree(s->d_w);
    stencil_tables_free(s->stencil);
    dfree(s->d_sx);
    dfree(s->d_sy);
    dfree(s->d_sz);
    dfree(s->d_src_node);
    dfree(s->d_src_coef);
    dfree(s->d_wavelet);
    dfree(s->d_rec_node);
    dfree(s->d_rec_perm);
    dfree(s->d_traces);
    dfree(s->d_ctr);
    dfree(s->d_status);
    dfree(s->d_upd_rec_off);
    if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return SEM_OK;
}

int sem_solver_create(sem_mesh *m, float dt, sem_solver **out)
{
    GUARD_BEGIN
    if (!m || !out) return fail(SEM_ERR_ARG, "NULL argument");
    *out = nullptr;
    if (!(dt > 0) || !std::isfinite(dt)) return fail(SEM_ERR_ARG, "dt must be positive");
    sem_solver *s = new sem_solver();
    s->mesh = m;
    s->dt = dt;
    s->n_int = m->box.n_int;
    auto cleanup = [&](int code, const std::string &msg) {
        sem_solver_destroy(s);
        return fail(code, msg);
    };
    cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cleanup(SEM_ERR_CUDA, cudaGetErrorString(e));
    s->own_stream = true;
    for (auto &p : s->d_p)
        if ((e = dalloc(&p, s->n_int)) != cudaSuccess || (e = cudaMemset(p, 0, s->n_int * 4)) != cudaSuccess)
            return cleanup(SEM_ERR_OOM, std::string("pressure levels: ") + cudaGetErrorString(e));
    if ((e = dalloc(&s->d_a, s->n_int)) != cudaSuccess || (e = cudaMemset(s->d_a, 0, s->n_int * 4)) != cudaSuccess)
        return cleanup(SEM_ERR_OOM, std::string("mass coefficient: ") + cudaGetErrorString(e));
    if ((e = dalloc(&s->d_ctr, 2)) != cudaSuccess || (e = cudaMemset(s->d_ctr, 0, 8)) != cudaSuccess)
        return cleanup(SEM_ERR_CUDA, cudaGetErrorString(e));
    if ((e = dalloc(&s->d_status, 1)) != cudaSuccess || (e = cudaMemset(s->d_status, 0, 4)) != cudaSuccess)
        return cleanup(SEM_ERR_CUDA, cudaGetErrorString(e));
    if ((e = dalloc(&s->d_w, m->box.order + 1)) != cudaSuccess ||
        (e = cudaMemcpy(s->d_w, m->gll.w, (m->box.order + 1) * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess)
        return cleanup(SEM_ERR_CUDA, cudaGetErrorString(e));
    // element coefficient table: g_d * w_a * w_b per pencil
    {
        const int o1 = m->box.order + 1, np = o1 * o1;
        std::vector<float> tab(3 * np);
        for (int d = 0; d < 3; d++)
            for (int b = 0; b < o1; b++)
                for (int a2 = 0; a2 < o1; a2++)
                    tab[d * np + a2 + o1 * b] = (float)(m->geo.g[d] * m->gll.w[a2] * m->gll.w[b]);
        if ((e = dalloc(&s->d_tab, tab.size())) != cudaSuccess ||
            (e = cudaMemcpy(s->d_tab, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice)) != cudaSuccess)
            return cleanup(SEM_ERR_CUDA, cudaGetErrorString(e));
    }
    if ((e = element_kernel_setup()) != cudaSuccess || (e = stencil_kernel_setup()) != cudaSuccess)
        return cleanup(SEM_ERR_CUDA, std::string("kernel set-up: ") + cudaGetErrorString(e));
    *out = s;
    return SEM_OK;
    GUARD_END
}

int sem_solver_set_stream(sem_solver *s, void *stream)
{
    if (!s) return fail(SEM_ERR_ARG, "NULL solver");
    cudaStreamSynchronize(s->stream);
    solver_invalidate_graphs(s);
    if (s->own_stream) cudaStreamDestroy(s->stream);
    if (stream) {
        s->stream = (cudaStream_t)stream;
        s->own_stream = false;
    } else {
        CUDA_TRY(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
        s->own_stream = true;
    }
    return SEM_OK;
}

int sem_solver_set_kernel(sem_solver *s, int kernel)
{
    if (!s) return fail(SEM_ERR_ARG, "NULL solver");
    if (kernel < SEM_KERNEL_AUTO || kernel > SEM_KERNEL_STENCIL) return fail(SEM_ERR_ARG, "unknown kernel");
    if (kernel != s->kernel) {
        cudaStreamSynchronize(s->stream);
        solver_invalidate_graphs(s);
        s->kernel = kernel;
    }
    return SEM_OK;
}

int sem_solver_set_operator_form(sem_solver *s, int form)
{
    if (!s) return fail(SEM_ERR_ARG, "NULL solver");
    if (form != SEM_FORM_DIRECT && form != SEM_FORM_DIFFERENCE) return fail(SEM_ERR_ARG, "unknown operator form");
    if (form != s->form) {
        cudaStreamSynchronize(s->stream);
        solver_invalidate_graphs(s);
        s->form = form;
    }
    return SEM_OK;
}

int sem_solver_set_rounding(sem_solver *s, int rounding)
{
    if (!s) return fail(SEM_ERR_ARG, "NULL solver");
    if (rounding != SEM_ROUNDING_DEFAULT && rounding != SEM_ROUNDING_REFERENCE) return fail(SEM_ERR_ARG, "unknown rounding");
    if (rounding != s->rounding) {
        cudaStreamSynchronize(s->stream);
        solver_invalidate_graphs(s);
        s->rounding = rounding;
    }
    return SEM_OK;
}

int sem_solver_set_tile_shape(sem_solver *s, int shape)
{
    if (!s) return fail(SEM_ERR_ARG, "NULL solver");
    if (shape != SEM_TILE_AUTO && shape != SEM_TILE_DEFAULT && shape != SEM_TILE_SQUARE)
        return fail(SEM_ERR_ARG, "unknown tile shape");
    static_assert(SEM_TILE_DEFAULT == kTileDefault && SEM_TILE_SQUARE == kTileSquare, "tile shapes");
    if (shape != s->tile_shape) {
        cudaStreamSynchronize(s->stream);
        solver_invalidate_graphs(s);
        stencil_tables_free(s->stencil);  // rebuilt by the next step
        s->tile_shape = shape;
    }
    return SEM_OK;
}

int sem_solver_get_tile_shape(const sem_solver *s, int *shape)
{
    if (!s || !shape) return fail(SEM_ERR_ARG, "NULL argument");
    *shape = s->stencil ? s->stencil->shape : SEM_TILE_AUTO;
    return SEM_OK;
}

int sem_solver_set_sponge_profile(sem_solver *s, const float *sx, const float *sy, const float *sz)
{
    GUARD_BEGIN
    if (!s) return fail(SEM_ERR_ARG, "NULL solver");
    const Box &b = s->mesh->box;
    cudaStreamSynchronize(s->stream);
    solver_invalidate_graphs(s);
    if (!sx || !sy || !sz) {
        s->sponge = false;
        return SEM_OK;
    }
    for (const auto &pr : {std::make_pair(sx, b.nx), std::make_pair(sy, b.ny), std::make_pair(sz, b.nz)})
        for (int64_t i = 0; i < pr.second; i++)
            if (!(pr.first[i] >= 0) || !(pr.first[i] <= 1))
                return fail(SEM_ERR_ARG, "sponge factors must lie in [0, 1]");
    if (!s->d_sx) {
        CUDA_TRY(dalloc(&s->d_sx, b.nx));
        CUDA_TRY(dalloc(&s->d_sy, b.ny));
        CUDA_TRY(dalloc(&s->d_sz, b.nz));
    }
    CUDA_TRY(cudaMemcpy(s->d_sx, sx, b.nx * 4, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(s->d_sy, sy, b.ny * 4, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(s->d_sz, sz, b.nz * 4, cudaMemcpyHostToDevice));
    s->sponge = true;
    return SEM_OK;
    GUARD_END
}

int sem_solver_set_sponge(sem_solver *s, int thickness, float sigma)
{
    GUARD_BEGIN
    if (!s) return fail(SEM_ERR_ARG, "NULL solver");
    if (thickness < 0 || !(sigma >= 0)) return fail(SEM_ERR_ARG, "bad sponge parameters");
    if (thickness == 0) return sem_solver_set_sponge_profile(s, nullptr, nullptr, nullptr);
    std::vector<float> a, b, c;
    box_sponge_profile(s->mesh->box, s->mesh->gll, thickness, sigma, a, b, c);
    return sem_solver_set_sponge_profile(s, a.data(), b.data(), c.data());
    GUARD_END
}

int sem_solver_set_sources(sem_solver *s, int n_src, const int64_t *elements, const float *wavelet,
                           int n_samples)
{
    GUARD_BEGIN
    if (!s) return fail(SEM_ERR_ARG, "NULL solver");
    if (n_src < 0 || n_samples < 0 || (n_src > 0 && (!elements || (n_samples > 0 && !wavelet))))
        return fail(SEM_ERR_ARG, "bad source arrays");
    const Box &b = s->mesh->box;
    std::vector<float> vel(b.n_elem);
    if (n_src > 0)
        CUDA_TRY(cudaMemcpy(vel.data(), s->mesh->d_vel, b.n_elem * 4, cudaMemcpyDeviceToHost));
    std::vector<int64_t> node(n_src);
    std::vector<float> coef(n_src);
    const float dt = s->dt;
    for (int k = 0; k < n_src; k++) {
        if (elements[k] < 0 || elements[k] >= b.n_elem)
            return fail(SEM_ERR_ARG, "source element out of range");
        node[k] = to_internal(b, box_node(b, elements[k], 0));  // local node 0 (SEMsolver.cpp:40)
        const float c = vel[elements[k]];
        coef[k] = dt * dt * c * c;              // rounded as SEMsolver.cpp:41-42
    }
    return solver_set_raw_sources(s, n_src, node.data(), coef.data(), wavelet, n_samples);
    GUARD_END
}

int sem_solver_set_source_points(sem_solver *s, int n_src, const float *xyz, const float *wavelet,
                                 int n_samples)
{
    GUARD_BEGIN
    if (!s || (n_src > 0 && !xyz)) return fail(SEM_ERR_ARG, "NULL argument");
    std::vector<int64_t> el(std::max(n_src, 0));
    for (int k = 0; k < n_src; k++)
        el[k] = box_element_from_point(s->mesh->box, xyz[3 * k], xyz[3 * k + 1], xyz[3 * k + 2]);
    return sem_solver_set_sources(s, n_src, el.data(), wavelet, n_samples);
    GUARD_END
}

int sem_solver_set_receiver_nodes(sem_solver *s, int n_rec, const int64_t *nodes)
{
    GUARD_BEGIN
    if (!s) return fail(SEM_ERR_ARG, "NULL solver");
    if (n_rec < 0 || (n_rec > 0 && !nodes)) return fail(SEM_ERR_ARG, "bad receiver array");
    if (s->steps_done > 0) return fail(SEM_ERR_STATE, "receivers must be set before the first step (or after sem_solver_reset)");
    for (int r = 0; r < n_rec; r++)
        if (nodes[r] < 0 || nodes[r] >= s->mesh->box.n_nodes)
            return fail(SEM_ERR_ARG, "receiver node out of range");
    std::vector<int> perm(n_rec);
    std::iota(perm.begin(), perm.end(), 0);
    std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return nodes[a] < nodes[b]; });
    std::vector<int64_t> sorted(n_rec);  // device-layout indices (same order as reference indices)
    for (int r = 0; r < n_rec; r++) sorted[r] = to_internal(s->mesh->box, nodes[perm[r]]);
    cudaStreamSynchronize(s->stream);
    solver_invalidate_graphs(s);
    dfree(s->d_rec_node);
    dfree(s->d_rec_perm);
    dfree(s->d_traces);
    s->trace_cap = 0;
    s->traces_checked = 0;
    s->nrec = n_rec;
    s->rec_sorted = sorted;
    s->rec_version++;
    if (n_rec > 0) {
        CUDA_TRY(dalloc(&s->d_rec_node, n_rec));
        CUDA_TRY(dalloc(&s->d_rec_perm, n_rec));
        CUDA_TRY(cudaMemcpy(s->d_rec_node, sorted.data(), n_rec * 8, cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(s->d_rec_perm, perm.data(), n_rec * 4, cudaMemcpyHostToDevice));
    }
    return SEM_OK;
    GUARD_END
}

int sem_solver_set_receivers(sem_solver *s, int n_rec, const float *xyz)
{
    GUARD_BEGIN
    if (!s || (n_rec > 0 && !xyz)) return fail(SEM_ERR_ARG, "NULL argument");
    std::vector<int64_t> nodes(std::max(n_rec, 0));
    for (int r = 0; r < n_rec; r++)
        nodes[r] = box_nearest_node(s->mesh->box, s->mesh->gll, xyz[3 * r], xyz[3 * r + 1], xyz[3 * r + 2]);
    return sem_solver_set_receiver_nodes(s, n_rec, nodes.data());
    GUARD_END
}

// ---- time loop --------------------------------------------------------------------------------

}  // extern "C"

int solver_prepare(sem_solver *s, int64_t n_new)
{
    sem_mesh *m = s->mesh;
    const int kern = resolved_kernel(s);
    if (s->a_version != m->model_version) {
        CUDA_TRY(launch_mass(s->d_a, m->d_slow2 ? nullptr : m->d_vel, m->d_slow2, m->box.ex, m->box.ey,
                             m->box.ez, m->box.order, m->box.nxp, s->d_w, m->geo.detJ,
                             (double)s->dt * s->dt, s->stream));
        s->a_version = m->model_version;
    }
    if (kern == SEM_KERNEL_ELEMENT) {
        int rc = ensure_conn(m, s->stream);
        if (rc) return rc;
        if (!s->d_y) {
            CUDA_TRY(dalloc(&s->d_y, s->n_int));
            CUDA_TRY(cudaMemsetAsync(s->d_y, 0, s->n_int * 4, s->stream));
        }
        if (s->rounding == SEM_ROUNDING_REFERENCE && !s->d_rtab) {
            const Box &b = m->box;
            std::vector<float> rows;
            reference_element_rows(m->gll, 0.5 * b.lx / b.ex, 0.5 * b.lz / b.ez, 0.5 * b.ly / b.ey, rows);
            CUDA_TRY(dalloc(&s->d_rtab, rows.size()));
            CUDA_TRY(cudaMemcpy(s->d_rtab, rows.data(), rows.size() * 4, cudaMemcpyHostToDevice));
            solver_invalidate_graphs(s);
        }
        if (s->rounding == SEM_ROUNDING_REFERENCE && !m->d_slow2 && s->mref_version != m->model_version) {
            const Box &b = m->box;
            if (!s->d_mref) {
                CUDA_TRY(dalloc(&s->d_mref, s->n_int));
                solver_invalidate_graphs(s);
            }
            // detJ grouped as computeB forms it (SEMQkGLIntegrals.hpp:316-318)
            const double detJ = std::fabs((0.5 * b.lx / b.ex) * ((0.5 * b.lz / b.ez) * (0.5 * b.ly / b.ey)));
            CUDA_TRY(launch_mass_ref(s->d_mref, m->d_vel, b.ex, b.ey, b.ez, b.order, b.nxp, s->d_w, detJ, s->stream));
            s->mref_version = m->model_version;
        }
        if (s->upd_rec_version != s->rec_version) {
            dfree(s->d_upd_rec_off);
            if (s->nrec > 0) {
                const int64_t nb = update_grid(s->n_int);
                std::vector<int> off(nb + 1, 0);
                for (int64_t q : s->rec_sorted) off[q / kUpdateNodesPerBlock + 1]++;
                for (int64_t b = 0; b < nb; b++) off[b + 1] += off[b];
                CUDA_TRY(dalloc(&s->d_upd_rec_off, nb + 1));
                CUDA_TRY(cudaMemcpy(s->d_upd_rec_off, off.data(), (nb + 1) * sizeof(int), cudaMemcpyHostToDevice));
            }
            s->upd_rec_version = s->rec_version;
            solver_invalidate_graphs(s);
        }
    } else {
        const bool want_class = s->rounding == SEM_ROUNDING_REFERENCE;
        // the reference rounding runs on the default tile shape
        const int shape = want_class ? kTileDefault : s->tile_shape;
        if (s->stencil && shape == kTileDefault && s->stencil->shape != kTileDefault) {
            stencil_tables_free(s->stencil);
            solver_invalidate_graphs(s);
        }
        if (!s->stencil) {
            int rc = stencil_tables_create(m->box, m->gll, m->geo, 1, &s->stencil, shape);
            if (rc) return fail(SEM_ERR_CUDA, "stencil tables");
        }
        if (want_class != (s->stencil->class_tab != nullptr)) {
            std::vector<float> tab;
            const Box &b = m->box;
            if (want_class) reference_class_table(m->gll, 0.5 * b.lx / b.ex, 0.5 * b.lz / b.ez, 0.5 * b.ly / b.ey, tab);
            stencil_set_class_table(*s->stencil, want_class ? tab.data() : nullptr);
            solver_invalidate_graphs(s);
        }
        if (stencil_bind(*s->stencil, s->d_p[0], s->d_p[1], s->d_a) != 0)
            return fail(SEM_ERR_CUDA, "tensor-map encoding failed (driver entry point cuTensorMapEncodeTiled)");
        if (s->stencil->rec_version != s->rec_version) {
            CUDA_TRY(stencil_set_receivers(*s->stencil, s->rec_sorted.data(), s->nrec, s->rec_version));
            solver_invalidate_graphs(s);
        }
    }
    if (s->nrec > 0 && s->steps_done + n_new > s->trace_cap) {
        int64_t cap = std::max<int64_t>(s->steps_done + n_new, std::max<int64_t>(64, 2 * s->trace_cap));
        float *nt = nullptr;
        CUDA_TRY(dalloc(&nt, (size_t)cap * s->nrec));
        CUDA_TRY(cudaMemsetAsync(nt, 0, (size_t)cap * s->nrec * 4, s->stream));
        if (s->d_traces && s->steps_done > 0)
            CUDA_TRY(cudaMemcpyAsync(nt, s->d_traces, (size_t)s->steps_done * s->nrec * 4,
                                     cudaMemcpyDeviceToDevice, s->stream));
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        dfree(s->d_traces);
        s->d_traces = nt;
        s->trace_cap = cap;
        solver_invalidate_graphs(s);
    }
    return SEM_OK;
}

// One step with the current level index c; the new level lands in 1-c.  Optional events time
// the source, stiffness and update launches; `extra` selects an adjoint-support mode of the
// stencil pass (its side buffers for this step).
cudaError_t solver_enqueue_step(sem_solver *s, int c, cudaEvent_t *ev, const StepExtra *extra)
{
    sem_mesh *m = s->mesh;
    const Box &b = m->box;
    cudaError_t e;
    SourceArgs sa{s->d_p[c], s->d_src_node, s->d_src_coef, s->d_wavelet, s->nsamples > 0 ? s->nsrc : 0,
                  s->nsamples, s->d_ctr, s->src_distinct ? 1 : 0};
    if (ev) cudaEventRecord(ev[0], s->stream);
    if ((e = launch_source(sa, s->stream)) != cudaSuccess) return e;
    if (ev) cudaEventRecord(ev[1], s->stream);
    if (resolved_kernel(s) == SEM_KERNEL_ELEMENT) {
        if (extra && extra->mode != STENCIL_PLAIN) return cudaErrorInvalidValue;  // stencil pass only
        ElementArgs ea{};
        ea.conn = m->d_conn;
        ea.p = s->d_p[c];
        ea.y = s->d_y;
        ea.tab = s->d_tab;
        ea.rtab = s->rounding == SEM_ROUNDING_REFERENCE ? s->d_rtab : nullptr;
        ea.n_elem = b.n_elem;
        element_stiffness_1d(m->gll, ea.S);
        if ((e = launch_element(b.order, ea, s->stream)) != cudaSuccess) return e;
        if (ev) cudaEventRecord(ev[2], s->stream);
        UpdateArgs ua{};
        ua.cur = s->d_p[c];
        ua.prev = s->d_p[1 - c];
        ua.y = s->d_y;
        ua.a = s->d_a;
        ua.sx = s->d_sx; ua.sy = s->d_sy; ua.sz = s->d_sz;
        ua.nx = b.nx; ua.nxp = b.nxp; ua.ny = b.ny; ua.nz = b.nz; ua.n_int = b.n_int;
        ua.rec_node = s->d_rec_node;
        ua.rec_perm = s->d_rec_perm;
        ua.rec_off = s->d_upd_rec_off;
        ua.nrec = s->nrec;
        ua.traces = s->d_traces;
        ua.ctr = s->d_ctr;
        if (s->rounding == SEM_ROUNDING_REFERENCE && !m->d_slow2) {
            ua.mref = s->d_mref;
            ua.dt2f = s->dt * s->dt;  // rounded as the reference's myTimeStep*myTimeStep
        }
        if ((e = launch_update(ua, s->sponge, s->stream)) != cudaSuccess) return e;
    } else {
        StencilArgs ta{};
        ta.cur = s->d_p[c];
        ta.prev = s->d_p[1 - c];
        ta.sx = s->d_sx; ta.sy = s->d_sy; ta.sz = s->d_sz;
        ta.status = s->d_status;
        ta.rec_node = s->d_rec_node;
        ta.rec_perm = s->d_rec_perm;
        ta.rec_off = s->stencil->d_rec_off;
        ta.rec_idx = s->stencil->d_rec_idx;
        ta.nrec = s->nrec;
        ta.traces = s->d_traces;
        ta.ctr = s->d_ctr;
        int mode = STENCIL_PLAIN;
        if (extra) {
            mode = extra->mode;
            ta.kp = extra->kp;
            ta.grad = extra->grad;
        }
        const bool direct = s->form == SEM_FORM_DIRECT || s->rounding == SEM_ROUNDING_REFERENCE;
        if ((e = launch_stencil(*s->stencil, ta, c, s->sponge, s->stream, mode, direct)) != cudaSuccess) return e;
        if (ev) cudaEventRecord(ev[2], s->stream);
    }
    if (ev) cudaEventRecord(ev[3], s->stream);
    return cudaSuccess;
}

extern "C" {

static int build_graph(sem_solver *s, int c)
{
    cudaGraph_t g = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e1 = solver_enqueue_step(s, c);
    cudaError_t e2 = e1 == cudaSuccess ? solver_enqueue_step(s, 1 - c) : e1;
    cudaError_t e3 = cudaStreamEndCapture(s->stream, &g);
    if (e2 != cudaSuccess || e3 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return fail(SEM_ERR_CUDA, std::string("graph capture: ") +
                                      cudaGetErrorString(e2 != cudaSuccess ? e2 : e3));
    }
    cudaError_t e4 = cudaGraphInstantiate(&s->graph2[c], g, 0);
    cudaGraphDestroy(g);
    if (e4 != cudaSuccess) return fail(SEM_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e4));
    return SEM_OK;
}

int sem_solver_step(sem_solver *s, int n_steps)
{
    GUARD_BEGIN
    if (!s) return fail(SEM_ERR_ARG, "NULL solver");
    if (n_steps < 0) return fail(SEM_ERR_ARG, "n_steps must be >= 0");
    if (n_steps == 0) return SEM_OK;
    int rc = solver_prepare(s, n_steps);
    if (rc) return rc;
    int done = 0;
    while (n_steps - done >= 2) {
        if (!s->graph2[s->cur]) {
            rc = build_graph(s, s->cur);
            if (rc) return rc;
        }
        CUDA_TRY(cudaGraphLaunch(s->graph2[s->cur], s->stream));
        done += 2;  // two swaps: the current level index is unchanged
    }
    if (done < n_steps) {
        CUDA_TRY(solver_enqueue_step(s, s->cur));
        s->cur ^= 1;
        done++;
    }
    s->steps_done += n_steps;
    return SEM_OK;
    GUARD_END
}

int sem_solver_step_host(sem_solver *s, int n_steps, const float *wavelet_samples, float *traces_out)
{
    GUARD_BEGIN
    if (!s) return fail(SEM_ERR_ARG, "NULL solver");
    if (n_steps < 0) return fail(SEM_ERR_ARG, "n_steps must be >= 0");
    if (n_steps == 0) return SEM_OK;
    const int64_t n0 = s->steps_done;
    if (wavelet_samples && s->nsrc > 0) {
        if (n0 + n_steps > s->nsamples)
            return fail(SEM_ERR_ARG, "wavelet storage shorter than the steps requested");
        // host [n_steps][nsrc] -> device [nsrc][nsamples] columns n0..n0+n_steps-1
        for (int k = 0; k < s->nsrc; k++)
            CUDA_TRY(cudaMemcpy2DAsync(s->d_wavelet + (size_t)k * s->nsamples + n0, sizeof(float),
                                       wavelet_samples + k, (size_t)s->nsrc * sizeof(float),
                                       sizeof(float), n_steps, cudaMemcpyHostToDevice, s->stream));
    }
    int rc = sem_solver_step(s, n_steps);
    if (rc) return rc;
    if (traces_out && s->nrec > 0)
        CUDA_TRY(cudaMemcpyAsync(traces_out, s->d_traces + (size_t)n0 * s->nrec,
                                 (size_t)n_steps * s->nrec * sizeof(float), cudaMemcpyDeviceToHost,
                                 s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    return SEM_OK;
    GUARD_END
}

int sem_solver_steps_done(const sem_solver *s, int64_t *n)
{
    if (!s || !n) return fail(SEM_ERR_ARG, "NULL argument");
    *n = s->steps_done;
    return SEM_OK;
}

int sem_solver_synchronize(sem_solver *s)
{
    GUARD_BEGIN
    if (!s) return fail(SEM_ERR_ARG, "NULL solver");
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    int status = 0;
    CUDA_TRY(cudaMemcpy(&status, s->d_status, 4, cudaMemcpyDeviceToHost));
    if (status != 0)
        return fail(SEM_ERR_TIMEOUT, "a bounded wait for a TMA tile gave up; results of this run are invalid");
    if (s->nrec > 0 && s->steps_done > s->traces_checked) {
        const int64_t n = (s->steps_done - s->traces_checked) * s->nrec;
        std::vector<float> t(n);
        CUDA_TRY(cudaMemcpy(t.data(), s->d_traces + (size_t)s->traces_checked * s->nrec, n * 4,
                            cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < n; i++)
            if (!std::isfinite(t[i]))
                return fail(SEM_ERR_UNSTABLE, "non-finite receiver sample at step " +
                                                  std::to_string(s->traces_checked + i / s->nrec) +
                                                  " (dt above the stability limit?)");
        s->traces_checked = s->steps_done;
    }
    return SEM_OK;
    GUARD_END
}

int sem_solver_get_traces(sem_solver *s, float *out)
{
    GUARD_BEGIN
    if (!s) return fail(SEM_ERR_ARG, "NULL solver");
    if (s->nrec == 0 || s->steps_done == 0) return SEM_OK;
    if (!out) return fail(SEM_ERR_ARG, "NULL output");
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    CUDA_TRY(cudaMemcpy(out, s->d_traces, (size_t)s->steps_done * s->nrec * 4, cudaMemcpyDeviceToHost));
    return SEM_OK;
    GUARD_END
}

// Per-node sponge factors of the reference layout, as the kernels form them: (sx*sy)*sz.
static int host_sponge(sem_solver *s, std::vector<float> &sx, std::vector<float> &sy, std::vector<float> &sz)
{
    const Box &b = s->mesh->box;
    sx.resize(b.nx); sy.resize(b.ny); sz.resize(b.nz);
    CUDA_TRY(cudaMemcpy(sx.data(), s->d_sx, b.nx * 4, cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(sy.data(), s->d_sy, b.ny * 4, cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(sz.data(), s->d_sz, b.nz * 4, cudaMemcpyDeviceToHost));
    return SEM_OK;
}

int sem_solver_get_pressure(sem_solver *s, int level, float *out)
{
    GUARD_BEGIN
    if (!s || !out) return fail(SEM_ERR_ARG, "NULL argument");
    if (level != SEM_LEVEL_CURRENT && level != SEM_LEVEL_PREVIOUS) return fail(SEM_ERR_ARG, "bad level");
    const Box &b = s->mesh->box;
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    const int idx = level == SEM_LEVEL_CURRENT ? s->cur : 1 - s->cur;
    // device layout (rows of nxp) -> reference layout (rows of nx)
    CUDA_TRY(field_to_host(out, s->d_p[idx], b.nx, b.nxp, b.nz * b.ny, s->stream));
    if (level == SEM_LEVEL_PREVIOUS && s->sponge) {
        // the stored previous level still lacks its last sponge factor
        std::vector<float> sx, sy, sz;
        int rc = host_sponge(s, sx, sy, sz);
        if (rc) return rc;
        int64_t i = 0;
        for (int64_t iy = 0; iy < b.ny; iy++)
            for (int64_t iz = 0; iz < b.nz; iz++)
                for (int64_t ix = 0; ix < b.nx; ix++, i++) {
                    const float f = sx[ix] * sy[iy] * sz[iz];
                    out[i] = f * out[i];
                }
    }
    return SEM_OK;
    GUARD_END
}

int sem_solver_set_pressure(sem_solver *s, int level, const float *in)
{
    GUARD_BEGIN
    if (!s || !in) return fail(SEM_ERR_ARG, "NULL argument");
    if (level != SEM_LEVEL_CURRENT && level != SEM_LEVEL_PREVIOUS) return fail(SEM_ERR_ARG, "bad level");
    const Box &b = s->mesh->box;
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    const int idx = level == SEM_LEVEL_CURRENT ? s->cur : 1 - s->cur;
    std::vector<float> v(in, in + b.n_nodes);
    if (level == SEM_LEVEL_PREVIOUS && s->sponge) {
        // stored without its last sponge factor: divide it out where it is non-zero, so that the
        // next step sees (to within one rounding) the damped level the caller passed
        std::vector<float> sx, sy, sz;
        int rc = host_sponge(s, sx, sy, sz);
        if (rc) return rc;
        int64_t i = 0;
        for (int64_t iy = 0; iy < b.ny; iy++)
            for (int64_t iz = 0; iz < b.nz; iz++)
                for (int64_t ix = 0; ix < b.nx; ix++, i++) {
                    const float f = sx[ix] * sy[iy] * sz[iz];
                    if (f > 0) v[i] = v[i] / f;
                }
    }
    CUDA_TRY(field_from_host(s->d_p[idx], v.data(), b.nx, b.nxp, b.nz * b.ny, s->stream));
    return SEM_OK;
    GUARD_END
}

int sem_solver_reset(sem_solver *s)
{
    GUARD_BEGIN
    if (!s) return fail(SEM_ERR_ARG, "NULL solver");
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    for (auto p : s->d_p) CUDA_TRY(cudaMemset(p, 0, s->n_int * 4));
    if (s->d_y) CUDA_TRY(cudaMemset(s->d_y, 0, s->n_int * 4));
    CUDA_TRY(cudaMemset(s->d_ctr, 0, 8));
    CUDA_TRY(cudaMemset(s->d_status, 0, 4));
    if (s->d_traces) CUDA_TRY(cudaMemset(s->d_traces, 0, (size_t)s->trace_cap * s->nrec * 4));
    s->steps_done = 0;
    s->traces_checked = 0;
    s->cur = 0;
    return SEM_OK;
    GUARD_END
}

int sem_solver_time_kernels(sem_solver *s, int n_steps, float *ms)
{
    GUARD_BEGIN
    if (!s || !ms || n_steps < 1) return fail(SEM_ERR_ARG, "bad arguments");
    int rc = solver_prepare(s, n_steps);
    if (rc) return rc;
    cudaEvent_t ev[4];
    for (auto &e : ev) CUDA_TRY(cudaEventCreate(&e));
    double acc[3] = {0, 0, 0};
    for (int i = 0; i < n_steps; i++) {
        cudaError_t e = solver_enqueue_step(s, s->cur, ev);
        if (e != cudaSuccess) {
            for (auto &x : ev) cudaEventDestroy(x);
            return fail(SEM_ERR_CUDA, cudaGetErrorString(e));
        }
        s->cur ^= 1;
        s->steps_done++;
        cudaEventSynchronize(ev[3]);
        float t;
        cudaEventElapsedTime(&t, ev[0], ev[1]); acc[0] += t;
        cudaEventElapsedTime(&t, ev[1], ev[2]); acc[1] += t;
        cudaEventElapsedTime(&t, ev[2], ev[3]); acc[2] += t;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    for (int k = 0; k < 3; k++) ms[k] = (float)(acc[k] / n_steps);
    return SEM_OK;
    GUARD_END
}

}  // extern "C"
