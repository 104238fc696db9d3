// group_api.cu -- many independent problems of uneven size advanced together (sem_group_*).
//
// Each member is an ordinary solver (its own mesh, order, model, dt, sources and receivers).
// Two ways to advance them, both replayed from one CUDA graph per two steps:
//  - one launch (default where every member allows it: stencil pass, orders 1-4, direct form,
//    default rounding): per step one source launch and one pass launch over all members' CTAs
//    (k_group.cu).  The members' tiles are cut along y into chunks of about the same number of
//    planes, chosen for the whole group, and the longest CTAs come first in the launch;
//  - branches: the group stream forks into the members' streams, each branch holds that member's
//    own steps (source, stencil pass), and the branches join back; largest member first.
// Each member's results are bit for bit those of the member stepped alone, either way.  Members
// may also be stepped alone between group steps: the group follows each member's current level.
#include <cuda_runtime.h>

#include <algorithm>
#include <numeric>
#include <utility>
#include <vector>

#include "abi.h"
#include "solver.h"

using semgb::Box;
using semgb::GroupMember;
using semgb::StencilTables;

struct sem_group {
    std::vector<sem_solver *> members;  // capture order: largest first
    cudaStream_t stream = nullptr;
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> join;
    int want = SEM_GROUP_ONE_LAUNCH;   // requested launch form
    int form = -1;                     // form of the graphs and state below
    cudaGraphExec_t graph[2] = {nullptr, nullptr};  // [f]: two steps starting at parity f
    std::vector<uint64_t> gen;         // members' graph generations at build
    std::vector<int> cur0;             // member's current level at parity 0
    int flip = 0;                      // parity of the next step
    // one-launch form
    std::vector<StencilTables *> tabs;  // the members' tables with the group's y-chunks
    std::vector<float *> ones;          // unit sponge factors of members without a sponge
    GroupMember *d_mem = nullptr;
    int *d_cta_member = nullptr;
    int n_ctas = 0, max_order = 0;
};

namespace {

void drop_graphs(sem_group *g)
{
    for (auto &x : g->graph)
        if (x) { cudaGraphExecDestroy(x); x = nullptr; }
}

void free_one_launch(sem_group *g)
{
    for (auto &t : g->tabs) semgb::stencil_tables_free(t);
    g->tabs.clear();
    for (float *p : g->ones)
        if (p) cudaFree(p);
    g->ones.clear();
    if (g->d_mem) { cudaFree(g->d_mem); g->d_mem = nullptr; }
    if (g->d_cta_member) { cudaFree(g->d_cta_member); g->d_cta_member = nullptr; }
    g->n_ctas = 0;
}

bool stale(const sem_group *g)
{
    if (g->gen.size() != g->members.size()) return true;
    for (size_t i = 0; i < g->members.size(); i++)
        if (g->members[i]->graph_gen != g->gen[i]) return true;
    return false;
}

bool one_launch_allowed(const sem_group *g)
{
    for (const sem_solver *s : g->members) {
        const int o = s->mesh->box.order;
        if (s->kernel == SEM_KERNEL_ELEMENT || o > semgb::kGroupMaxOrder || s->form != SEM_FORM_DIRECT ||
            s->rounding != SEM_ROUNDING_DEFAULT || !s->stencil || s->stencil->nshot != 1)
            return false;
    }
    return true;
}

// Fork the members from the group stream, enqueue `steps` steps on each from level
// cur0 ^ parity, join them back.
cudaError_t enqueue_branches(sem_group *g, int steps, int parity)
{
    cudaError_t e = cudaEventRecord(g->fork, g->stream);
    if (e != cudaSuccess) return e;
    for (size_t i = 0; i < g->members.size(); i++) {
        sem_solver *s = g->members[i];
        if ((e = cudaStreamWaitEvent(s->stream, g->fork, 0)) != cudaSuccess) return e;
        int c = g->cur0[i] ^ parity;
        for (int k = 0; k < steps; k++, c ^= 1)
            if ((e = solver_enqueue_step(s, c)) != cudaSuccess) return e;
        if ((e = cudaEventRecord(g->join[i], s->stream)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(g->stream, g->join[i], 0)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t enqueue_one_launch(sem_group *g, int steps, int parity)
{
    for (int k = 0; k < steps; k++) {
        cudaError_t e = semgb::launch_group_step(g->d_mem, (int)g->members.size(), g->d_cta_member, g->n_ctas,
                                                 g->max_order, parity ^ (k & 1), g->stream);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t enqueue(sem_group *g, int steps, int parity)
{
    return g->form == SEM_GROUP_ONE_LAUNCH ? enqueue_one_launch(g, steps, parity) : enqueue_branches(g, steps, parity);
}

int capture(sem_group *g, int parity)
{
    cudaGraph_t graph = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e1 = enqueue(g, 2, parity);
    cudaError_t e2 = cudaStreamEndCapture(g->stream, &graph);
    if (e1 != cudaSuccess || e2 != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return sem_fail(SEM_ERR_CUDA, std::string("group graph capture: ") +
                                          cudaGetErrorString(e1 != cudaSuccess ? e1 : e2));
    }
    cudaError_t e3 = cudaGraphInstantiate(&g->graph[parity], graph, 0);
    cudaGraphDestroy(graph);
    if (e3 != cudaSuccess) return sem_fail(SEM_ERR_CUDA, cudaGetErrorString(e3));
    return SEM_OK;
}

// y-chunk length of every member for one launch over the group: chunks of about L planes, L
// chosen to minimise the launch's makespan, estimated by placing the CTAs longest first on the
// resident CTA slots, each on the least loaded one (a member's CTAs all have the same work, so
// they go in whole rounds over the slots, the remainder on the least loaded); a CTA's work is
// its planes plus the 2o planes it reads before its first output.
std::vector<int> group_chunks(const sem_group *g, int64_t resident)
{
    const size_t n = g->members.size();
    int64_t ny_max = 1;
    for (const sem_solver *s : g->members) ny_max = std::max(ny_max, s->mesh->box.ny);
    double best = 1e300;
    int64_t best_l = ny_max;
    std::vector<std::pair<int64_t, int64_t>> jobs;  // (CTA work in planes, CTA count)
    std::vector<double> load((size_t)std::max<int64_t>(resident, 1));
    for (int64_t L = 1; L <= ny_max; L++) {
        jobs.clear();
        for (const sem_solver *s : g->members) {
            const Box &b = s->mesh->box;
            int tx = 0, tz = 0, hx = 0, th = 0;  // the member's own tile shape
            semgb::stencil_tile_dims(b.order, s->stencil->shape, tx, tz, hx, th);
            const int64_t cols = ((b.nx + tx - 1) / tx) * ((b.nz + tz - 1) / tz);
            const int64_t c = (b.ny + L - 1) / L, chunk = (b.ny + c - 1) / c;
            jobs.push_back({chunk + 2 * b.order, cols * c});
        }
        std::sort(jobs.begin(), jobs.end(), [](const auto &x, const auto &y) { return x.first > y.first; });
        std::fill(load.begin(), load.end(), 0.0);  // kept in ascending order
        const int64_t R = (int64_t)load.size();
        for (const auto &jb : jobs) {
            const double w = (double)jb.first;
            const int64_t rounds = jb.second / R, rem = jb.second % R;
            if (rounds > 0)
                for (double &x : load) x += w * (double)rounds;
            for (int64_t k = 0; k < rem; k++) load[k] += w;
            std::inplace_merge(load.begin(), load.begin() + rem, load.end());
        }
        const double makespan = load.back();
        if (makespan < best - 1e-9) { best = makespan; best_l = L; }
    }
    std::vector<int> out(n);
    for (size_t i = 0; i < n; i++) {
        const int64_t ny = g->members[i]->mesh->box.ny;
        const int64_t c = (ny + best_l - 1) / best_l;
        out[i] = (int)((ny + c - 1) / c);
    }
    return out;
}

// Member descriptors from the members' current state (levels cur0 ^ k at parity k).
int write_descriptors(sem_group *g)
{
    const size_t n = g->members.size();
    std::vector<GroupMember> h(n);
    int cta = 0;
    // launch order: longest CTAs first
    std::vector<size_t> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
        return g->tabs[a]->ychunk + 2 * g->tabs[a]->order > g->tabs[b]->ychunk + 2 * g->tabs[b]->order;
    });
    std::vector<int> cta_member;
    for (size_t oi = 0; oi < n; oi++) {
        const size_t i = order[oi];
        sem_solver *s = g->members[i];
        const StencilTables &t = *g->tabs[i];
        GroupMember &m = h[i];
        m.t = t;
        m.t.class_tab = nullptr;
        m.order = t.order;
        m.cur0 = g->cur0[i];
        m.cta0 = cta;
        const float *ones = g->ones[i];
        for (int k = 0; k < 2; k++) {
            const int c = g->cur0[i] ^ k;
            semgb::StencilArgs &a = m.a[k];
            a = semgb::StencilArgs{};
            a.cur = s->d_p[c];
            a.prev = s->d_p[1 - c];
            a.sx = s->sponge ? s->d_sx : ones;
            a.sy = s->sponge ? s->d_sy : ones;
            a.sz = s->sponge ? s->d_sz : ones;
            a.status = s->d_status;
            a.rec_node = s->d_rec_node;
            a.rec_perm = s->d_rec_perm;
            a.rec_off = t.d_rec_off;
            a.rec_idx = t.d_rec_idx;
            a.nrec = s->nrec;
            a.traces = s->d_traces;
            a.ctr = s->d_ctr;
            m.src[k] = semgb::SourceArgs{s->d_p[c], s->d_src_node, s->d_src_coef, s->d_wavelet,
                                         s->nsamples > 0 ? s->nsrc : 0, s->nsamples, s->d_ctr, s->src_distinct ? 1 : 0};
        }
        const int64_t nc = (int64_t)t.grid[0] * t.grid[1] * t.grid[2];
        if (cta + nc > (int64_t)0x7fffffff) return sem_fail(SEM_ERR_ARG, "group too large for one launch");
        cta_member.insert(cta_member.end(), (size_t)nc, (int)i);
        cta += (int)nc;
    }
    if (!g->d_mem) {
        CUDA_TRY(cudaMalloc(&g->d_mem, n * sizeof(GroupMember)));
        CUDA_TRY(cudaMalloc(&g->d_cta_member, cta_member.size() * sizeof(int)));
    } else if ((int)cta_member.size() != g->n_ctas) {
        return sem_fail(SEM_ERR_STATE, "group launch changed size");
    }
    g->n_ctas = (int)cta_member.size();
    // the group stream is idle here (callers synchronise it first), so plain copies are ordered
    CUDA_TRY(cudaMemcpy(g->d_mem, h.data(), n * sizeof(GroupMember), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(g->d_cta_member, cta_member.data(), cta_member.size() * sizeof(int), cudaMemcpyHostToDevice));
    return SEM_OK;
}

// Tables, unit sponges and descriptors of the one-launch form from the members' current state.
int build_one_launch(sem_group *g)
{
    CUDA_TRY(cudaStreamSynchronize(g->stream));  // no launch of the group still reads the old state
    CUDA_TRY(semgb::group_kernel_setup());
    const size_t n = g->members.size();
    int max_order = 1;
    for (const sem_solver *s : g->members) max_order = std::max(max_order, s->mesh->box.order);
    int dev = 0, sms = 152;
    CUDA_TRY(cudaGetDevice(&dev));
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int per_sm = std::max(1, semgb::group_blocks_per_sm(max_order));
    const std::vector<int> chunks = group_chunks(g, (int64_t)sms * per_sm);
    for (auto &t : g->tabs) semgb::stencil_tables_free(t);
    g->tabs.assign(n, nullptr);
    if (g->ones.size() != n) g->ones.assign(n, nullptr);
    for (size_t i = 0; i < n; i++) {
        sem_solver *s = g->members[i];
        // tables of the member's own tile shape over its levels, with the group's chunking
        StencilTables *t = nullptr;
        if (semgb::stencil_tables_create(s->mesh->box, s->mesh->gll, s->mesh->geo, 1, &t, s->stencil->shape) != 0)
            return sem_fail(SEM_ERR_CUDA, "stencil tables");
        g->tabs[i] = t;
        if (semgb::stencil_bind(*t, s->d_p[0], s->d_p[1], s->d_a) != 0)
            return sem_fail(SEM_ERR_CUDA, "tensor-map encoding failed (driver entry point cuTensorMapEncodeTiled)");
        t->ychunk = chunks[i];
        t->grid[2] = (int)((t->ny + chunks[i] - 1) / chunks[i]);
        CUDA_TRY(semgb::stencil_set_receivers(*t, s->rec_sorted.data(), s->nrec, s->rec_version));
        if (!s->sponge && !g->ones[i]) {
            const Box &b = s->mesh->box;
            const size_t len = (size_t)std::max(b.nx, std::max(b.ny, b.nz));
            std::vector<float> one(len, 1.f);
            CUDA_TRY(cudaMalloc(&g->ones[i], len * sizeof(float)));
            CUDA_TRY(cudaMemcpy(g->ones[i], one.data(), len * sizeof(float), cudaMemcpyHostToDevice));
        }
    }
    g->max_order = max_order;
    return write_descriptors(g);
}

}  // namespace

extern "C" {

int sem_group_destroy(sem_group *g)
{
    if (!g) return SEM_OK;
    if (g->stream) cudaStreamSynchronize(g->stream);
    drop_graphs(g);
    free_one_launch(g);
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

int sem_group_set_launch(sem_group *g, int form)
{
    GUARD_BEGIN
    if (!g || (form != SEM_GROUP_ONE_LAUNCH && form != SEM_GROUP_BRANCHES)) return sem_fail(SEM_ERR_ARG, "bad arguments");
    g->want = form;
    return SEM_OK;
    GUARD_END
}

int sem_group_get_launch(sem_group *g, int *form)
{
    GUARD_BEGIN
    if (!g || !form) return sem_fail(SEM_ERR_ARG, "bad arguments");
    *form = g->form >= 0 ? g->form : g->want;
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
    const size_t n = g->members.size();
    const int form = g->want == SEM_GROUP_ONE_LAUNCH && one_launch_allowed(g) ? SEM_GROUP_ONE_LAUNCH : SEM_GROUP_BRANCHES;
    bool rebuild = stale(g) || form != g->form;
    if (!rebuild) {
        // members stepped alone since the last group step: follow their current levels
        for (size_t i = 0; i < n && !rebuild; i++)
            if ((g->cur0[i] ^ g->flip) != g->members[i]->cur) rebuild = true;
    }
    if (rebuild) {
        CUDA_TRY(cudaStreamSynchronize(g->stream));
        drop_graphs(g);
        g->form = form;
        g->flip = 0;
        g->cur0.resize(n);
        g->gen.resize(n);
        for (size_t i = 0; i < n; i++) {
            g->cur0[i] = g->members[i]->cur;
            g->gen[i] = g->members[i]->graph_gen;
        }
        if (form == SEM_GROUP_ONE_LAUNCH) {
            int rc = build_one_launch(g);
            if (rc) return rc;
        } else {
            free_one_launch(g);
        }
    }
    // order against work already on the members' own streams (set-up, earlier solo steps)
    for (size_t i = 0; i < n; i++) {
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
        CUDA_TRY(enqueue(g, 1, g->flip));
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
