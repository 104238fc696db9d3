// k_stencil.cu -- fused SEM step on a uniform box (operator in stencil.h), TMA-pipelined.
//
// Coefficients: for each axis the assembled 1-D stiffness row of a node depends only on its local
// index l = i mod o, so the three axis terms use one table
//     T[l][d + o] = coupling between a node with local index l and the node d places further
// along the same axis (zero outside the node's element or element pair), applied in difference
// form sum_d T[l][d] (p_{i+d} - p_i), exactly zero for a constant field.
//
// Work decomposition (HBM-bound pass: read p^n, p^{n-1}, dt^2/M, write p^{n+1}; 16 B/node):
//  - a CTA owns a tile of TX nodes along x by TZ rows along z and marches along y over a chunk
//    of planes; a lane holds one element's o consecutive x-nodes, so a node's local x index is a
//    compile-time constant (x-coefficients are immediates, zero terms are skipped); a warp covers
//    RW rows o apart (RW = 2 for o = 1, 2, 4: 16 lanes per row, TX = 16*o), so the z- and
//    y-local indices are warp-uniform and select specialised code;
//  - one elected thread streams y-planes into shared memory with 3-D TMA tile loads completed on
//    mbarriers: a ring of 2o+1+L planes of p^n (tile rows only) serves the y-neighbours, and
//    per-plane "aux" slots hold the p^{n-1} and dt^2/M tiles plus a window of the plane's p^n with
//    its z and x halos (the x- and z-neighbours and the node itself); keeping the halos out of
//    the ring halves its size, so three CTAs fit on an SM for o <= 4; loads run L planes ahead;
//  - one barrier per plane; every mbarrier wait is bounded (tma.cuh) and a timeout is reported
//    through a status word instead of hanging.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "stencil_body.cuh"

namespace semgb {

namespace {

template <int O, bool SPONGE, int MODE, bool DIRECT, bool MULTI, bool REF = false, int RWS = SEM_STENCIL_RW>
__global__ void __launch_bounds__(Cfg<O, RWS>::THREADS, Cfg<O, RWS>::MIN_BLOCKS)
    k_stencil(const __grid_constant__ CUtensorMap ring_map, const __grid_constant__ CUtensorMap win_map,
              const __grid_constant__ CUtensorMap prev_map, const __grid_constant__ CUtensorMap a_map,
              const StencilTables t, const StencilArgs a, const __grid_constant__ ClassParam<O, REF> ct)
{
    // CTA -> (x-tile, z-tile, y-chunk): grid (x-tiles, z-tiles, chunks).  MULTI (many shots, the
    // levels stacking the shots along y: plane p of shot s is plane s*ny + p): grid
    // (shots * z-tiles * x-tiles, chunks) with the shot varying fastest, then z, so that the CTAs
    // of all shots of a tile run together and share its dt^2/M planes and z-halo rows in L2.
    int shot = 0, bx, bz, chunk;
    if constexpr (MULTI) {
        const int tile = (int)(blockIdx.x / (unsigned)t.nshot);
        shot = (int)(blockIdx.x - (unsigned)tile * (unsigned)t.nshot);
        bz = tile % t.grid[1];
        bx = tile / t.grid[1];
        chunk = (int)blockIdx.y;
    } else {
        bx = (int)blockIdx.x;
        bz = (int)blockIdx.y;
        chunk = (int)blockIdx.z;
    }
    stencil_cta<O, SPONGE, MODE, DIRECT, MULTI, REF, false, RWS>(&ring_map, &win_map, &prev_map, &a_map, t, a, ct,
                                                                 shot, bx, bz, chunk);
}

template <int O, int RWS = SEM_STENCIL_RW>
size_t smem_of() { return Cfg<O, RWS>::SMEM; }

size_t smem_bytes(int order, int shape)
{
    switch (order) {
    case 1: return smem_of<1>();
    case 2: return smem_of<2>();
    case 3: return smem_of<3>();
    case 4: return shape == kTileSquare ? smem_of<4, kSquareRW>() : smem_of<4>();
    default: return smem_of<5>();
    }
}

template <int O, int RWS = SEM_STENCIL_RW>
void tile_of(int &tx, int &tz, int &hx, int &th)
{
    tx = Cfg<O, RWS>::TX; tz = Cfg<O, RWS>::TZ; hx = Cfg<O, RWS>::HX; th = Cfg<O, RWS>::THREADS;
}

// resident CTAs per SM of the sponge variant (the others use no more registers); 0 if unknown
template <int O, int RWS = SEM_STENCIL_RW>
int blocks_per_sm_of()
{
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_stencil<O, true, STENCIL_PLAIN, true, false, false, RWS>,
                                                      Cfg<O, RWS>::THREADS, Cfg<O, RWS>::SMEM) != cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    return n;
}

int blocks_per_sm(int order, int shape)
{
    switch (order) {
    case 1: return blocks_per_sm_of<1>();
    case 2: return blocks_per_sm_of<2>();
    case 3: return blocks_per_sm_of<3>();
    case 4: return shape == kTileSquare ? blocks_per_sm_of<4, kSquareRW>() : blocks_per_sm_of<4>();
    default: return blocks_per_sm_of<5>();
    }
}

template <int O, bool SPONGE, int MODE, bool DIRECT, bool MULTI, bool REF = false, int RWS = SEM_STENCIL_RW>
void launch_om(const dim3 &grid, const LevelMaps &cm, const LevelMaps &pm, const StencilTables &t,
               const StencilArgs &a, cudaStream_t s)
{
    using C = Cfg<O, RWS>;
    ClassParam<O, REF> ct{};
    if constexpr (REF) std::memcpy(ct.c, t.class_tab, sizeof ct.c);
    if (MULTI && t.cluster > 1) {
        // the CTAs of `cluster` consecutive shots of a tile (consecutive in x of the grid) start
        // together on one GPC and march along y side by side, so each dt^2/M tile they share is
        // still in L2 when the later ones read it
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = grid;
        cfg.blockDim = dim3(C::THREADS);
        cfg.dynamicSmemBytes = C::SMEM;
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)t.cluster;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        cudaLaunchKernelEx(&cfg, k_stencil<O, SPONGE, MODE, DIRECT, MULTI, REF>, cm.tile, cm.win, pm.tile, t.amap, t,
                           a, ct);
        return;
    }
    k_stencil<O, SPONGE, MODE, DIRECT, MULTI, REF, RWS>
        <<<grid, C::THREADS, C::SMEM, s>>>(cm.tile, cm.win, pm.tile, t.amap, t, a, ct);
}

template <int O, bool DIRECT>
cudaError_t launch_of(const StencilTables &t, const StencilArgs &a, int ci, bool sponge, int mode, cudaStream_t s)
{
    const LevelMaps &cm = t.lv[ci], &pm = t.lv[1 - ci];
    if (t.shape == kTileSquare) {
        // the square order-4 tile: single-shot plain steps in the tensor-product operator
        if constexpr (O == 4) {
            if (t.class_tab || t.nshot != 1 || mode != STENCIL_PLAIN) return cudaErrorInvalidValue;
            const dim3 grid(t.grid[0], t.grid[1], t.grid[2]);
            if (sponge) launch_om<O, true, STENCIL_PLAIN, DIRECT, false, false, kSquareRW>(grid, cm, pm, t, a, s);
            else launch_om<O, false, STENCIL_PLAIN, DIRECT, false, false, kSquareRW>(grid, cm, pm, t, a, s);
            return cudaGetLastError();
        }
        return cudaErrorInvalidValue;
    }
    if (t.class_tab) {
        // reference rounding: plain steps with the node-class table (one shot or many)
        if constexpr (DIRECT) {
            if (mode != STENCIL_PLAIN) return cudaErrorInvalidValue;
            if (t.nshot > 1) {
                const dim3 grid((unsigned)((int64_t)t.grid[0] * t.grid[1] * t.nshot), (unsigned)t.grid[2]);
                if (sponge) launch_om<O, true, STENCIL_PLAIN, true, true, true>(grid, cm, pm, t, a, s);
                else launch_om<O, false, STENCIL_PLAIN, true, true, true>(grid, cm, pm, t, a, s);
            } else {
                const dim3 grid(t.grid[0], t.grid[1], t.grid[2]);
                if (sponge) launch_om<O, true, STENCIL_PLAIN, true, false, true>(grid, cm, pm, t, a, s);
                else launch_om<O, false, STENCIL_PLAIN, true, false, true>(grid, cm, pm, t, a, s);
            }
            return cudaGetLastError();
        }
        return cudaErrorInvalidValue;
    }
    if (t.nshot > 1) {
        // many shots: plain steps in the direct form
        if constexpr (DIRECT) {
            if (mode != STENCIL_PLAIN) return cudaErrorInvalidValue;
            const dim3 grid((unsigned)((int64_t)t.grid[0] * t.grid[1] * t.nshot), (unsigned)t.grid[2]);
            if (sponge) launch_om<O, true, STENCIL_PLAIN, true, true>(grid, cm, pm, t, a, s);
            else launch_om<O, false, STENCIL_PLAIN, true, true>(grid, cm, pm, t, a, s);
            return cudaGetLastError();
        }
        return cudaErrorInvalidValue;
    }
    const dim3 grid(t.grid[0], t.grid[1], t.grid[2]);
    switch (mode * 2 + (sponge ? 1 : 0)) {
    case 0: launch_om<O, false, STENCIL_PLAIN, DIRECT, false>(grid, cm, pm, t, a, s); break;
    case 1: launch_om<O, true, STENCIL_PLAIN, DIRECT, false>(grid, cm, pm, t, a, s); break;
    case 2: launch_om<O, false, STENCIL_RECORD_KP, DIRECT, false>(grid, cm, pm, t, a, s); break;
    case 3: launch_om<O, true, STENCIL_RECORD_KP, DIRECT, false>(grid, cm, pm, t, a, s); break;
    case 4: launch_om<O, false, STENCIL_GRADIENT, DIRECT, false>(grid, cm, pm, t, a, s); break;
    case 5: launch_om<O, true, STENCIL_GRADIENT, DIRECT, false>(grid, cm, pm, t, a, s); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <int O>
cudaError_t launch_o(const StencilTables &t, const StencilArgs &a, int ci, bool sponge, int mode, bool direct,
                     cudaStream_t s)
{
    return direct ? launch_of<O, true>(t, a, ci, sponge, mode, s) : launch_of<O, false>(t, a, ci, sponge, mode, s);
}

template <int O, bool SPONGE, int MODE, bool DIRECT, bool MULTI = false, bool REF = false, int RWS = SEM_STENCIL_RW>
cudaError_t setup_om()
{
    return cudaFuncSetAttribute(k_stencil<O, SPONGE, MODE, DIRECT, MULTI, REF, RWS>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg<O, RWS>::SMEM);
}

template <int O, bool DIRECT>
cudaError_t setup_of()
{
    cudaError_t e;
    if ((e = setup_om<O, true, STENCIL_PLAIN, DIRECT>()) != cudaSuccess) return e;
    if ((e = setup_om<O, false, STENCIL_PLAIN, DIRECT>()) != cudaSuccess) return e;
    if ((e = setup_om<O, true, STENCIL_RECORD_KP, DIRECT>()) != cudaSuccess) return e;
    if ((e = setup_om<O, false, STENCIL_RECORD_KP, DIRECT>()) != cudaSuccess) return e;
    if ((e = setup_om<O, true, STENCIL_GRADIENT, DIRECT>()) != cudaSuccess) return e;
    return setup_om<O, false, STENCIL_GRADIENT, DIRECT>();
}

template <int O>
cudaError_t setup_o()
{
    cudaError_t e = setup_of<O, true>();
    if (e == cudaSuccess) e = setup_of<O, false>();
    if (e == cudaSuccess) e = setup_om<O, true, STENCIL_PLAIN, true, true>();
    if (e == cudaSuccess) e = setup_om<O, false, STENCIL_PLAIN, true, true>();
    if (e == cudaSuccess) e = setup_om<O, true, STENCIL_PLAIN, true, false, true>();
    if (e == cudaSuccess) e = setup_om<O, false, STENCIL_PLAIN, true, false, true>();
    if (e == cudaSuccess) e = setup_om<O, true, STENCIL_PLAIN, true, true, true>();
    if (e == cudaSuccess) e = setup_om<O, false, STENCIL_PLAIN, true, true, true>();
    if constexpr (O == 4) {
        if (e == cudaSuccess) e = setup_om<O, true, STENCIL_PLAIN, true, false, false, kSquareRW>();
        if (e == cudaSuccess) e = setup_om<O, false, STENCIL_PLAIN, true, false, false, kSquareRW>();
        if (e == cudaSuccess) e = setup_om<O, true, STENCIL_PLAIN, false, false, false, kSquareRW>();
        if (e == cudaSuccess) e = setup_om<O, false, STENCIL_PLAIN, false, false, false, kSquareRW>();
    }
    return e;
}

// 3-D map over the device layout (nxp, nz, planes) of float buffer `base` with box (bx, bz, 1);
// planes = ny, or ny * nshot for levels that stack the shots along y.
bool make_map(CUtensorMap &m, const float *base, const StencilTables &t, int bx, int bz, int64_t planes)
{
    return encode_map_3d(m, base, t.nxp, t.nz, planes, bx, bz);
}

}  // namespace

void stencil_tile_dims(int order, int shape, int &tx, int &tz, int &hx, int &threads)
{
    switch (order) {
    case 1: tile_of<1>(tx, tz, hx, threads); break;
    case 2: tile_of<2>(tx, tz, hx, threads); break;
    case 3: tile_of<3>(tx, tz, hx, threads); break;
    case 4:
        if (shape == kTileSquare) tile_of<4, kSquareRW>(tx, tz, hx, threads);
        else tile_of<4>(tx, tz, hx, threads);
        break;
    default: tile_of<5>(tx, tz, hx, threads); break;
    }
}

int stencil_tables_create(const Box &b, const Gll &g, const Geometry &geo, int nshot, StencilTables **out, int shape)
{
    if (nshot < 1) return (int)cudaErrorInvalidValue;
    StencilTables *t = new StencilTables();
    t->order = b.order;
    t->nx = b.nx; t->nxp = b.nxp; t->ny = b.ny; t->nz = b.nz;
    t->nshot = nshot;
    t->shot_stride = b.nxp * b.nz * b.ny;
    for (int d = 0; d < 3; d++) t->g[d] = (float)geo.g[d];
    for (int l = 0; l < b.order; l++) t->wa[l] = (float)(l == 0 ? g.w[0] + g.w[b.order] : g.w[l]);
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int smem_sm = 0;
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    // y-chunking of one tile shape: balance the last wave against the 2o warm-up planes of every
    // chunk; returns the cost in CTA-planes of the busiest slot and the chunk count
    struct Plan { double cost; int chunks; double lanes; };
    auto plan = [&](int sh) {
        int tx = 0, tz = 0, hx = 0, th = 0;
        stencil_tile_dims(b.order, sh, tx, tz, hx, th);
        int per_sm = blocks_per_sm(b.order, sh);  // kernel attributes are set up with the solver
        if (per_sm <= 0) per_sm = std::max(1, std::min(2048 / th, smem_sm / (int)(smem_bytes(b.order, sh) + 1024)));
        const int64_t gx = (b.nx + tx - 1) / tx, gz = (b.nz + tz - 1) / tz;
        const int64_t cols = gx * gz * nshot;
        const int64_t resident = (int64_t)sms * per_sm;
        Plan pl{1e300, 1, (double)(b.nx * b.nz) / (double)(gx * tx * gz * tz)};
        for (int c = 1; c <= 64 && c <= b.ny; c++) {
            const int64_t chunk = (b.ny + c - 1) / c;
            const int64_t waves = (cols * c + resident - 1) / resident;
            const double cost = (double)waves * (chunk + 2 * b.order);
            if (cost < pl.cost - 1e-9) { pl.cost = cost; pl.chunks = c; }
        }
        return pl;
    };
    // tile shape: the square order-4 tile for a single shot where it costs less, counting the
    // busiest slot's CTA-planes over the share of lanes on nodes (lanes past the box edge do the
    // same work; measured on GB300, 64 x 16 against 32 x 32: 801^3 nodes 369.1 against 367.0
    // Gnode-steps/s, 481^3 0.329 against 0.331 ms per step, 401^3 321.9 against 336.3, 345^3
    // 0.145 against 0.130 ms, which this ranking orders the same way)
    int sh = kTileDefault;
    if (b.order == 4 && nshot == 1) {
        if (shape == kTileSquare) {
            sh = kTileSquare;
        } else if (shape < 0) {
            const Plan p0 = plan(kTileDefault), p1 = plan(kTileSquare);
            if (p1.cost / p1.lanes < p0.cost / p0.lanes - 1e-9) sh = kTileSquare;
        }
    }
    t->shape = sh;
    int threads = 256;
    stencil_tile_dims(b.order, sh, t->tile_x, t->tile_z, t->halo_x, threads);
    t->threads = threads;
    t->smem = smem_bytes(b.order, sh);
    t->grid[0] = (int)((b.nx + t->tile_x - 1) / t->tile_x);
    t->grid[1] = (int)((b.nz + t->tile_z - 1) / t->tile_z);
    const int best_c = plan(sh).chunks;
    t->ychunk = (int)((b.ny + best_c - 1) / best_c);
    t->grid[2] = (int)((b.ny + t->ychunk - 1) / t->ychunk);
    *out = t;
    return 0;
}

int stencil_bind(StencilTables &t, const float *p0, const float *p1, const float *a)
{
    if (t.bound[0] == p0 && t.bound[1] == p1 && t.bound[2] == a) return 0;
    const int txp = t.tile_x + 2 * t.halo_x;
    const float *ps[2] = {p0, p1};
    for (int i = 0; i < 2; i++) {
        if (!make_map(t.lv[i].win, ps[i], t, txp, t.tile_z + 2 * t.order, t.ny * t.nshot) ||
            !make_map(t.lv[i].tile, ps[i], t, t.tile_x, t.tile_z, t.ny * t.nshot))
            return (int)cudaErrorInvalidValue;
    }
    if (!make_map(t.amap, a, t, t.tile_x, t.tile_z, t.ny)) return (int)cudaErrorInvalidValue;
    t.bound[0] = p0; t.bound[1] = p1; t.bound[2] = a;
    return 0;
}

cudaError_t stencil_set_receivers(StencilTables &t, const int64_t *sorted_nodes, int nrec, uint64_t version)
{
    if (t.d_rec_off) { cudaFree(t.d_rec_off); t.d_rec_off = nullptr; }
    if (t.d_rec_idx) { cudaFree(t.d_rec_idx); t.d_rec_idx = nullptr; }
    t.rec_version = version;
    if (nrec <= 0) return cudaSuccess;
    const int64_t ncta = (int64_t)t.grid[0] * t.grid[1] * t.grid[2];
    std::vector<int64_t> owner(nrec);
    std::vector<int> count(ncta + 1, 0);
    const int64_t nxz = t.nxp * t.nz;
    for (int r = 0; r < nrec; r++) {
        const int64_t n = sorted_nodes[r];
        const int64_t y = n / nxz, rem = n - y * nxz, z = rem / t.nxp, x = rem - z * t.nxp;
        owner[r] = x / t.tile_x + t.grid[0] * (z / t.tile_z + t.grid[1] * (y / t.ychunk));
        count[owner[r] + 1]++;
    }
    for (int64_t c = 0; c < ncta; c++) count[c + 1] += count[c];
    std::vector<int> idx(nrec), fill(count.begin(), count.end() - 1);
    for (int r = 0; r < nrec; r++) idx[fill[owner[r]]++] = r;
    cudaError_t e;
    if ((e = cudaMalloc(&t.d_rec_off, (ncta + 1) * sizeof(int))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&t.d_rec_idx, nrec * sizeof(int))) != cudaSuccess) return e;
    if ((e = cudaMemcpy(t.d_rec_off, count.data(), (ncta + 1) * sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess)
        return e;
    return cudaMemcpy(t.d_rec_idx, idx.data(), nrec * sizeof(int), cudaMemcpyHostToDevice);
}

int stencil_set_class_table(StencilTables &t, const float *tab)
{
    delete[] t.class_tab;
    t.class_tab = nullptr;
    if (!tab) return 0;
    const size_t n = (size_t)reference_class_table_size(t.order);
    t.class_tab = new float[n];
    std::memcpy(t.class_tab, tab, n * sizeof(float));
    return 0;
}

void stencil_tables_free(StencilTables *&t)
{
    if (!t) return;
    delete[] t->class_tab;
    if (t->d_rec_off) cudaFree(t->d_rec_off);
    if (t->d_rec_idx) cudaFree(t->d_rec_idx);
    delete t;
    t = nullptr;
}

cudaError_t stencil_kernel_setup()
{
    static std::vector<int> done_devices;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    for (int d : done_devices)
        if (d == dev) return cudaSuccess;
    if ((e = upload_stencil_constants()) != cudaSuccess) return e;
    if ((e = setup_o<1>()) != cudaSuccess) return e;
    if ((e = setup_o<2>()) != cudaSuccess) return e;
    if ((e = setup_o<3>()) != cudaSuccess) return e;
    if ((e = setup_o<4>()) != cudaSuccess) return e;
    if ((e = setup_o<5>()) != cudaSuccess) return e;
    done_devices.push_back(dev);
    return cudaSuccess;
}

cudaError_t launch_stencil(const StencilTables &t, const StencilArgs &a, int cur_index, bool sponge, cudaStream_t s,
                           int mode, bool direct)
{
    if (mode != STENCIL_PLAIN && (!a.kp || (mode == STENCIL_GRADIENT && !a.grad))) return cudaErrorInvalidValue;
    switch (t.order) {
    case 1: return launch_o<1>(t, a, cur_index, sponge, mode, direct, s);
    case 2: return launch_o<2>(t, a, cur_index, sponge, mode, direct, s);
    case 3: return launch_o<3>(t, a, cur_index, sponge, mode, direct, s);
    case 4: return launch_o<4>(t, a, cur_index, sponge, mode, direct, s);
    case 5: return launch_o<5>(t, a, cur_index, sponge, mode, direct, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace semgb
