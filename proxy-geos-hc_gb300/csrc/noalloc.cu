// noalloc.cu -- an element-path step that allocates no device memory.
//
// Some callers cannot allocate device memory while they advance the wavefield: a host code that
// hands all device memory to its own pool manager up front, or one that runs its time loop in a
// section where allocation is forbidden (a latency-critical loop, for instance).
// sem_element_step_noalloc serves them: the caller owns every input and output buffer, and the
// scratch memory the step needs -- the K.p accumulator that the element kernel scatters into,
// plus a small coefficient table -- is a fixed array in this library's device image instead of a
// cudaMalloc'd buffer.
//
// The array holds kNoAllocFloats floats (16 MiB on every GPU that loads the library, held until
// the process exits); meshes up to kNoAllocMaxNodes nodes fit.  Every call uses the same array:
// two calls whose work overlaps on the GPU (different streams, or different host threads) race
// on it.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/semgb.h"
#include "host_util.h"
#include "kernels.h"

namespace semgb {

void set_last_error(const std::string &msg);  // api.cu

namespace {

constexpr int64_t kNoAllocFloats = int64_t(1) << 22;      // 4,194,304 floats
constexpr int kTabFloats = 128;                            // coefficient table, at the end
constexpr int64_t kNoAllocMaxNodes = kNoAllocFloats - kTabFloats;

// The scratch array.  In host code this name denotes a host-side stand-in for the symbol, not a
// device address; the device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) float g_noalloc_scratch[kNoAllocFloats];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
float *g_scratch_dev[kMaxDevices] = {nullptr};

// Per-pencil coefficient table of the element kernel: tab[d][a + o1*b] = g_d * w_a * w_b.
struct TabArgs {
    float g[3];
    float w[6];
    int o1;
};

__global__ void k_fill_tab(float *tab, const TabArgs t)
{
    const int np = t.o1 * t.o1;
    for (int q = threadIdx.x; q < 3 * np; q += blockDim.x) {
        const int d = q / np, r = q - d * np, a = r % t.o1, b = r / t.o1;
        float wa = 0.f, wb = 0.f;
#pragma unroll
        for (int k = 0; k < 6; k++) {  // static indices keep the parameter struct out of local memory
            if (k == a) wa = t.w[k];
            if (k == b) wb = t.w[k];
        }
        const float gd = d == 0 ? t.g[0] : (d == 1 ? t.g[1] : t.g[2]);
        tab[q] = gd * wa * wb;
    }
}

// p_next = 2 p_cur - p_prev - coef * y on interior nodes, p_prev on boundary nodes (reference
// node numbering); then both levels take the sponge factor, as the solver's sponge does after
// each step.  Clears y behind it.
__global__ void k_update_ref(float *p_cur, float *p_prev, float *y, const float *__restrict__ coef,
                             const float *sx, const float *sy, const float *sz, int64_t nx, int64_t ny,
                             int64_t nz)
{
    const int64_t n = nx * ny * nz;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t iy = i / (nx * nz), r = i - iy * nx * nz, iz = r / nx, ix = r - iz * nx;
        const float pc = p_cur[i], q = p_prev[i];
        const bool interior = ix > 0 && ix < nx - 1 && iz > 0 && iz < nz - 1 && iy > 0 && iy < ny - 1;
        const float v = interior ? (2.f * pc - q) - coef[i] * y[i] : q;
        y[i] = 0.f;
        if (sx) {
            const float s = sx[ix] * sy[iy] * sz[iz];
            p_prev[i] = s * v;
            p_cur[i] = s * pc;
        } else {
            p_prev[i] = v;
        }
    }
}

// Device address of the scratch array on the current device: resolved on the first call made
// with that device current, then cached.  That first call also loads, under CUDA's lazy module
// loading, the code of every kernel the step launches and the array itself: this is the one
// point at which the entry point can make the driver allocate device memory.
int scratch_for_current_device(float **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        set_last_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
        return SEM_ERR_CUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        set_last_error("device index out of range");
        return SEM_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_dev[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            set_last_error(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            return SEM_ERR_CUDA;
        }
        e = element_kernel_setup();
        cudaFuncAttributes fa;
        if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_fill_tab);
        if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_update_ref);
        if (e != cudaSuccess) {
            set_last_error(std::string("element kernel set-up: ") + cudaGetErrorString(e));
            return SEM_ERR_CUDA;
        }
        g_scratch_dev[dev] = static_cast<float *>(p);
    }
    *out = g_scratch_dev[dev];
    return SEM_OK;
}

}  // namespace

}  // namespace semgb

using namespace semgb;

extern "C" int sem_element_step_noalloc(int ex, int ey, int ez, float lx, float ly, float lz, int order,
                                        const int32_t *conn, float *p_cur, float *p_prev, const float *coef,
                                        const float *sx, const float *sy, const float *sz, void *stream)
{
    Box b;
    if (!make_box(ex, ey, ez, lx, ly, lz, order, b)) {
        set_last_error("box needs ex,ey,ez >= 1, positive lengths and order 1..5");
        return SEM_ERR_ARG;
    }
    if (!conn || !p_cur || !p_prev || !coef || (!sx != !sy) || (!sx != !sz)) {
        set_last_error("NULL device buffer (the sponge factors are all given or all NULL)");
        return SEM_ERR_ARG;
    }
    if (b.n_nodes > kNoAllocMaxNodes) {
        set_last_error("mesh has " + std::to_string(b.n_nodes) + " nodes; sem_element_step_noalloc handles at most " +
                       std::to_string(kNoAllocMaxNodes) + " (the size of its fixed scratch array)");
        return SEM_ERR_ARG;
    }
    float *scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc != SEM_OK) return rc;
    float *y = scratch;
    float *tab = scratch + kNoAllocMaxNodes;
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    Gll g;
    gll_tables(order, g);
    const double jx = 0.5 * lx / ex, jz = 0.5 * lz / ez, jy = 0.5 * ly / ey, detJ = jx * jz * jy;
    TabArgs ta{};
    ta.g[0] = (float)(detJ / (jx * jx));
    ta.g[1] = (float)(detJ / (jz * jz));
    ta.g[2] = (float)(detJ / (jy * jy));
    ta.o1 = order + 1;
    for (int i = 0; i <= order; i++) ta.w[i] = (float)g.w[i];
    ElementArgs ea{};
    ea.conn = conn;
    ea.p = p_cur;
    ea.y = y;
    ea.tab = tab;
    ea.n_elem = b.n_elem;
    ea.n_check = b.n_nodes;  // the caller's map: indices outside [0, n_nodes) are skipped
    element_stiffness_1d(g, ea.S);

    // the array keeps the last call's contents: clear the accumulator this call uses
    cudaError_t e = cudaMemsetAsync(y, 0, b.n_nodes * sizeof(float), s);
    if (e == cudaSuccess) {
        k_fill_tab<<<1, 128, 0, s>>>(tab, ta);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = launch_element(order, ea, s);
    if (e == cudaSuccess) {
        k_update_ref<<<152 * 8, 256, 0, s>>>(p_cur, p_prev, y, coef, sx, sy, sz, b.nx, b.ny, b.nz);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        set_last_error(std::string("CUDA: ") + cudaGetErrorString(e));
        return SEM_ERR_CUDA;
    }
    return SEM_OK;
}
