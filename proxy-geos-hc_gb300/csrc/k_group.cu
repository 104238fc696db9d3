// k_group.cu -- one launch per step over the boxes of a group (uneven batch: different meshes,
// orders 1-4, models, dt, sources and receivers).
//
// Every member keeps its own levels, tensor maps and tiling; the launch's CTAs are the members'
// tiles x y-chunks one after another (cta_member maps a CTA to its member), so the GPU's
// scheduler fills SMs with whatever CTAs are left of any member, and a step of the whole group
// is two launches (sources, then the pass) instead of two per member.  A CTA runs the same code
// as the single-box pass of its order (stencil_body.cuh), so each member's results are bit for
// bit those of the member stepped alone.  The CTA has kGroupThreads threads; at order 3 (three
// warps) the fourth warp only takes part in the barriers.
//
// Members without a sponge run the sponge code with unit factors: every factor multiplies by
// exactly 1, so the results are those of the pass without a sponge.  An order-4 member runs on
// the tile shape of its tables (the square 32 x 32 tile where the member stepped alone takes it).
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "stencil_body.cuh"

namespace semgb {

namespace {

static_assert(Cfg<1>::THREADS <= kGroupThreads && Cfg<2>::THREADS <= kGroupThreads &&
                  Cfg<3>::THREADS <= kGroupThreads && Cfg<4>::THREADS <= kGroupThreads &&
                  Cfg<4, kSquareRW>::THREADS <= kGroupThreads,
              "a group CTA holds every order's configuration");

constexpr int kGroupMinBlocks = 3;

// Make the member's tensor maps (written to device memory by a copy before the launch) visible
// to the TMA unit.
__device__ __forceinline__ void tensormap_acquire(const CUtensorMap *m)
{
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(reinterpret_cast<uint64_t>(m))
                 : "memory");
}

// Sources of every member (block m: member m), as k_source does for one box: sources on distinct
// nodes added by all threads, otherwise by one thread in source order; the member's step
// counter advanced.
__global__ void k_group_source(const GroupMember *__restrict__ mem, int k)
{
    const SourceArgs &a = mem[blockIdx.x].src[k];
    const int n = a.ctr[0];
    __syncthreads();  // every thread has read the step before thread 0 advances the counter
    if (n < a.nsamples) {
        if (a.distinct) {
            for (int i = threadIdx.x; i < a.nsrc; i += blockDim.x)
                a.cur[a.node[i]] += a.coef[i] * a.wavelet[(int64_t)i * a.nsamples + n];
        } else if (threadIdx.x == 0) {
            for (int i = 0; i < a.nsrc; i++)
                a.cur[a.node[i]] += a.coef[i] * a.wavelet[(int64_t)i * a.nsamples + n];
        }
    }
    if (threadIdx.x == 0) {
        a.ctr[1] = n;
        a.ctr[0] = n + 1;
    }
}

__global__ void __launch_bounds__(kGroupThreads, kGroupMinBlocks)
    k_group(const GroupMember *__restrict__ mem, const int *__restrict__ cta_member, int k)
{
    const GroupMember &g = mem[__ldg(cta_member + blockIdx.x)];
    const StencilTables &t = g.t;
    const int ci = g.cur0 ^ k;
    const int local = (int)blockIdx.x - g.cta0;  // CTA within the member: x-tile fastest, then z, then chunk
    const int bx = local % t.grid[0], rz = local / t.grid[0];
    const int bz = rz % t.grid[1], chunk = rz / t.grid[1];
    const CUtensorMap *rmap = &t.lv[ci].tile, *wmap = &t.lv[ci].win, *pmap = &t.lv[1 - ci].tile, *amap = &t.amap;
    if (threadIdx.x == 0) {
        tensormap_acquire(rmap);
        tensormap_acquire(wmap);
        tensormap_acquire(pmap);
        tensormap_acquire(amap);
    }
    const StencilArgs &a = g.a[k];
    const NoClassTable none{};
    switch (g.order) {
    case 1: stencil_cta<1, true, STENCIL_PLAIN, true, false, false, true>(rmap, wmap, pmap, amap, t, a, none, 0, bx, bz, chunk); break;
    case 2: stencil_cta<2, true, STENCIL_PLAIN, true, false, false, true>(rmap, wmap, pmap, amap, t, a, none, 0, bx, bz, chunk); break;
    case 3: stencil_cta<3, true, STENCIL_PLAIN, true, false, false, true>(rmap, wmap, pmap, amap, t, a, none, 0, bx, bz, chunk); break;
    default:
        if (t.shape == kTileSquare)
            stencil_cta<4, true, STENCIL_PLAIN, true, false, false, true, kSquareRW>(rmap, wmap, pmap, amap, t, a, none, 0,
                                                                                     bx, bz, chunk);
        else
            stencil_cta<4, true, STENCIL_PLAIN, true, false, false, true>(rmap, wmap, pmap, amap, t, a, none, 0, bx, bz, chunk);
        break;
    }
}

size_t smem_upto(int max_order)
{
    size_t m = Cfg<1>::SMEM;
    if (max_order >= 2) m = std::max(m, Cfg<2>::SMEM);
    if (max_order >= 3) m = std::max(m, Cfg<3>::SMEM);
    if (max_order >= 4) m = std::max(m, std::max(Cfg<4>::SMEM, Cfg<4, kSquareRW>::SMEM));
    return m;
}

}  // namespace

cudaError_t group_kernel_setup()
{
    static std::vector<int> done_devices;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    for (int d : done_devices)
        if (d == dev) return cudaSuccess;
    if ((e = upload_stencil_constants()) != cudaSuccess) return e;
    if ((e = cudaFuncSetAttribute(k_group, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_upto(kGroupMaxOrder))) !=
        cudaSuccess)
        return e;
    done_devices.push_back(dev);
    return cudaSuccess;
}

size_t group_smem(int max_order) { return smem_upto(max_order); }

int group_blocks_per_sm(int max_order)
{
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_group, kGroupThreads, smem_upto(max_order)) != cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    return n;
}

cudaError_t launch_group_step(const GroupMember *members, int n_members, const int *cta_member, int n_ctas,
                              int max_order, int k, cudaStream_t s)
{
    if (n_members < 1 || n_ctas < 1 || max_order < 1 || max_order > kGroupMaxOrder || (k & ~1))
        return cudaErrorInvalidValue;
    k_group_source<<<n_members, 256, 0, s>>>(members, k);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_group<<<n_ctas, kGroupThreads, smem_upto(max_order), s>>>(members, cta_member, k);
    return cudaGetLastError();
}

}  // namespace semgb
