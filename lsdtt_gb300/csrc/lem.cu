// lem.cu -- the landscape-evolution timestep on the GPU, and the host-buffer
// routing entry point.
//
// run_lem_step (src/cpu/lsdtt_lem_cpu.cpp:285-732) in the D8 coupled regime:
// save the boundary-flat elevations, D8 engine on the input surface, implicit
// stream power, implicit linear hillslope step, uplift U*dt on valid cells,
// boundary flats reset to their pre-step value minus base-level fall, then
// the step statistics. The benchmark configurations fill the surface first
// (fill_pits(z, min_slope, bc)); that fill is part of the step when
// fill_min_slope > 0. Every buffer lives in the handle; the only host
// traffic per step is the level offsets of the sweeps and the statistics.

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "engine.cuh"
#include "lem_cell.cuh"

namespace lsdtt_gb300
{
namespace
{

__global__ void boundary_flag(int nr, int nc, const char* bc4, const std::uint8_t* __restrict__ mask,
                              std::uint8_t* __restrict__ flag)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const std::int64_t n = static_cast<std::int64_t>(nr) * nc;
    if (i >= n) return;
    flag[i] = boundary_flat_cell(nr, nc, bc4, mask, i) ? 1 : 0;
}

__global__ void lem_uplift_restore(std::int64_t n, const std::uint8_t* __restrict__ mask,
                                   const std::uint8_t* __restrict__ bflag, const float* __restrict__ z_before, float udz,
                                   float bl, float* __restrict__ z)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float v = z[i];
    if (mask[i]) v = __fadd_rn(v, udz);
    if (bflag[i]) v = __fsub_rn(z_before[i], bl);
    z[i] = v;
}

// Per-step statistics: FP64 sums and maxima by warp reduction + atomics,
// and the |dz| values (as float bits) for the 99.9th-percentile selection.
__global__ void lem_stats(std::int64_t n, const std::uint8_t* __restrict__ mask, const float* __restrict__ zb,
                          const float* __restrict__ za, double udz, double* __restrict__ acc,
                          std::uint64_t* __restrict__ keys, std::uint32_t* __restrict__ vals)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    double sb = 0, sa = 0, mb = -1e30, ma = -1e30, ml = 0, se = 0, me = 0, nv = 0;
    if (i < n)
    {
        vals[i] = static_cast<std::uint32_t>(i);
        if (mask[i])
        {
            const double b = zb[i], a = za[i];
            sb = b;
            sa = a;
            mb = b;
            ma = a;
            const double d = fabs(a - b);
            ml = d;
            keys[i] = __float_as_uint(static_cast<float>(d));
            const double ero = b - (a - udz);
            if (ero > 0.0) { se = ero; me = ero; }
            nv = 1;
        }
        else
            keys[i] = 0xffffffffull;  // sorts after every finite |dz|
    }
    block_atomic_add(&acc[0], sb);
    block_atomic_add(&acc[1], sa);
    block_atomic_add(&acc[2], se);
    block_atomic_add(&acc[3], nv);
    auto amax = [](double* p, double v) {
        // order-preserving map of doubles to unsigned for atomicMax
        const double t = block_reduce_d(v, true);
        if (threadIdx.x == 0)
        {
            unsigned long long u = __double_as_longlong(t);
            u = (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
            atomicMax(reinterpret_cast<unsigned long long*>(p), u);
        }
    };
    amax(&acc[4], mb);
    amax(&acc[5], ma);
    amax(&acc[6], ml);
    amax(&acc[7], me);
}

double unmap_max(double stored)
{
    unsigned long long u;
    std::memcpy(&u, &stored, sizeof(u));
    u = (u & 0x8000000000000000ull) ? (u & ~0x8000000000000000ull) : ~u;
    double v;
    std::memcpy(&v, &u, sizeof(v));
    return v;
}

__global__ void copy_f(const float* __restrict__ a, float* __restrict__ b, std::int64_t n)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) b[i] = a[i];
}

}  // namespace
}  // namespace lsdtt_gb300

using namespace lsdtt_gb300;

struct lsdtt_gpu_lem
{
    lsdtt_gpu_grid grid{};
    lsdtt_gpu_lem_options opt{};
    lsdtt_gpu_flow* flow = nullptr;
    std::uint8_t* mask = nullptr;
    std::uint8_t* bflag = nullptr;
    char* bc4 = nullptr;
    float* zf = nullptr;       // filled surface = the step's input
    float* zsp = nullptr;      // after stream power
    double* acc = nullptr;     // statistics accumulators
    double* hacc = nullptr;
    std::uint64_t* k0 = nullptr;
    std::uint32_t* v0 = nullptr;
    std::uint64_t* k1 = nullptr;
    std::uint32_t* v1 = nullptr;
    Scratch ws{};
    lsdtt_gpu_unet* net = nullptr;  // learned preconditioner, not owned
};

extern "C" {

int lsdtt_gpu_lem_create(const lsdtt_gpu_grid* grid, const std::uint8_t* mask_dev, const lsdtt_gpu_lem_options* o,
                         lsdtt_gpu_lem** out, void* stream)
{
    if (!grid || !mask_dev || !o || !out) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_lem_create: null argument");
    *out = nullptr;
    if (!(o->timestep > 0.0f)) return fail(LSDTT_GPU_EINVAL, "run_lem_step: timestep must be positive");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    auto* L = new lsdtt_gpu_lem();
    L->grid = *grid;
    L->opt = *o;
    int s = lsdtt_gpu_flow_create(grid, &L->flow);
    if (s != LSDTT_GPU_OK)
    {
        delete L;
        return s;
    }
    const std::int64_t n = static_cast<std::int64_t>(grid->n_rows) * grid->n_cols;
    cudaError_t e = cudaMalloc(&L->mask, n);
    if (e == cudaSuccess) e = cudaMalloc(&L->bflag, n);
    if (e == cudaSuccess) e = cudaMalloc(&L->bc4, 4);
    if (e == cudaSuccess) e = cudaMalloc(&L->zf, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc(&L->zsp, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc(&L->acc, sizeof(double) * 8);
    if (e == cudaSuccess) e = cudaMallocHost(&L->hacc, sizeof(double) * 8);
    if (e == cudaSuccess) e = cudaMalloc(&L->k0, sizeof(std::uint64_t) * n);
    if (e == cudaSuccess) e = cudaMalloc(&L->k1, sizeof(std::uint64_t) * n);
    if (e == cudaSuccess) e = cudaMalloc(&L->v0, sizeof(std::uint32_t) * n);
    if (e == cudaSuccess) e = cudaMalloc(&L->v1, sizeof(std::uint32_t) * n);
    // Radix-sort scratch of the p99.9 statistic: two per-tile histograms of
    // 256 counts (tiles of kSortTile keys) plus the scan's partial sums.
    const std::size_t tiles = static_cast<std::size_t>((n + kSortTile - 1) / kSortTile);
    const std::size_t wsb = tiles * 256 * 4 * 3 + (std::size_t(16) << 20);
    if (e == cudaSuccess) e = cudaMalloc(&L->ws.base, wsb);
    L->ws.cap = wsb;
    if (e != cudaSuccess)
    {
        lsdtt_gpu_lem_destroy(L);
        return cuda_fail(e, "lsdtt_gpu_lem_create");
    }
    cudaMemcpyAsync(L->mask, mask_dev, n, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(L->bc4, grid->boundary_conditions, 4, cudaMemcpyHostToDevice, st);
    boundary_flag<<<grid_blocks(n, 256), 256, 0, st>>>(grid->n_rows, grid->n_cols, L->bc4, L->mask, L->bflag);
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
    {
        lsdtt_gpu_lem_destroy(L);
        return cuda_fail(e, "lsdtt_gpu_lem_create");
    }
    *out = L;
    return LSDTT_GPU_OK;
}

int lsdtt_gpu_lem_destroy(lsdtt_gpu_lem* L)
{
    if (!L) return LSDTT_GPU_OK;
    lsdtt_gpu_flow_destroy(L->flow);
    cudaFree(L->mask);
    cudaFree(L->bflag);
    cudaFree(L->bc4);
    cudaFree(L->zf);
    cudaFree(L->zsp);
    cudaFree(L->acc);
    cudaFreeHost(L->hacc);
    cudaFree(L->k0);
    cudaFree(L->k1);
    cudaFree(L->v0);
    cudaFree(L->v1);
    cudaFree(L->ws.base);
    delete L;
    return LSDTT_GPU_OK;
}

int lsdtt_gpu_lem_step(lsdtt_gpu_lem* L, float* z_dev, lsdtt_gpu_lem_stats* stats, void* stream)
{
    if (!L || !z_dev) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_lem_step: null argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const lsdtt_gpu_lem_options& o = L->opt;
    const std::int64_t n = static_cast<std::int64_t>(L->grid.n_rows) * L->grid.n_cols;
    const unsigned nb = grid_blocks(n, 256);
    int s;
    // 0. optional fill: the step's input surface
    if (o.fill_min_slope > 0.0f)
    {
        s = lsdtt_gpu_fill_pits(&L->grid, z_dev, L->mask, o.fill_min_slope, L->zf, stream);
        if (s != LSDTT_GPU_OK) return s;
    }
    else
        copy_f<<<nb, 256, 0, st>>>(z_dev, L->zf, n);
    // 1. D8 engine + stream power (interior nodata drains, pits are outlets)
    lsdtt_gpu_flow_options fo{1, 1, 1, 0, 1};
    s = lsdtt_gpu_flow_build(L->flow, L->zf, L->mask, &fo, nullptr, 0, stream);
    if (s != LSDTT_GPU_OK) return s;
    s = lsdtt_gpu_stream_power_d8(L->flow, L->zf, nullptr, o.erodibility, o.m_exponent, o.n_exponent, o.timestep, 0.0f,
                                  o.divide_area_by_dx, o.slope_clamp, L->zsp, stream);
    if (s != LSDTT_GPU_OK) return s;
    // 2. hillslope (coupled regime: no channel cells)
    int hs_it = 0;
    if (o.enable_hillslope)
    {
        lsdtt_gpu_solve_report rep{};
        const double tol = o.hillslope_rel_tol > 0 ? o.hillslope_rel_tol : 1e-8;
        if (o.hillslope_nonlinear || L->net)
        {
            // compute_hillslope_newton_transient over the whole timestep
            if (L->net)
                s = lsdtt_gpu_hillslope_implicit_learned(&L->grid, L->zsp, L->mask, nullptr, o.hillslope_diffusivity,
                                                         o.critical_slope, o.hillslope_nonlinear, o.timestep, tol,
                                                         o.hillslope_max_iter, 0.0, 0, L->net, z_dev, &rep, stream);
            else
                s = lsdtt_gpu_hillslope_implicit(&L->grid, L->zsp, L->mask, nullptr, o.hillslope_diffusivity,
                                                 o.critical_slope, o.hillslope_nonlinear, o.timestep, tol,
                                                 o.hillslope_max_iter, 0.0, 0, z_dev, &rep, stream);
        }
        else
            s = lsdtt_gpu_hillslope_linear_implicit(&L->grid, L->zsp, L->mask, nullptr, o.hillslope_diffusivity,
                                                    o.timestep, tol, o.hillslope_max_iter, z_dev, &rep, stream);
        if (s != LSDTT_GPU_OK) return s;
        hs_it = rep.iterations;
    }
    else
        copy_f<<<nb, 256, 0, st>>>(L->zsp, z_dev, n);
    // 3-4. uplift, boundary restore
    const float udz = o.uplift_rate * o.timestep;
    const float bl = o.baselevel_fall_rate * o.timestep;
    lem_uplift_restore<<<nb, 256, 0, st>>>(n, L->mask, L->bflag, L->zf, udz, bl, z_dev);
    // 5. statistics
    if (stats)
    {
        cudaMemsetAsync(L->acc, 0, sizeof(double) * 8, st);
        lem_stats<<<nb, 256, 0, st>>>(n, L->mask, L->zf, z_dev, static_cast<double>(udz), L->acc, L->k0, L->v0);
        cudaMemcpyAsync(L->hacc, L->acc, sizeof(double) * 8, cudaMemcpyDeviceToHost, st);
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_lem_step");
        const double nv = L->hacc[3];
        const double inv_dt = 1.0 / static_cast<double>(o.timestep);
        const double inv_n = nv > 0 ? 1.0 / nv : 0.0;
        stats->delta_max_elevation = static_cast<float>(std::fabs(unmap_max(L->hacc[5]) - unmap_max(L->hacc[4])));
        stats->delta_mean_elevation = static_cast<float>(std::fabs((L->hacc[1] - L->hacc[0]) * inv_n));
        stats->max_local_elevation_change = static_cast<float>(unmap_max(L->hacc[6]));
        const double me = unmap_max(L->hacc[7]);
        stats->mean_erosion_rate = static_cast<float>(L->hacc[2] * inv_n * inv_dt);
        stats->max_erosion_rate = static_cast<float>((me > 0 ? me : 0.0) * inv_dt);
        stats->hillslope_iterations = hs_it;
        stats->p999_local_elevation_change = 0.0f;
        const std::int64_t nvi = static_cast<std::int64_t>(nv);
        if (nvi > 0)
        {
            // compute_quantile_floor_in_place: element floor(0.999*(nv-1)) in
            // ascending order. |dz| >= 0, so float bit patterns sort like values.
            L->ws.used = 0;
            const int cur = radix_sort_pairs(L->k0, L->v0, L->k1, L->v1, n, 32, L->ws, st, &e);
            if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_lem_step");
            std::size_t k = static_cast<std::size_t>(0.999 * static_cast<double>(nvi - 1));
            std::uint64_t bits = 0;
            cudaMemcpyAsync(&bits, (cur ? L->k1 : L->k0) + k, sizeof(bits), cudaMemcpyDeviceToHost, st);
            e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_lem_step");
            const std::uint32_t b32 = static_cast<std::uint32_t>(bits);
            float v;
            std::memcpy(&v, &b32, sizeof(v));
            stats->p999_local_elevation_change = v;
        }
    }
    return LSDTT_GPU_OK;
}

int lsdtt_gpu_lem_set_preconditioner(lsdtt_gpu_lem* L, lsdtt_gpu_unet* net)
{
    if (!L) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_lem_set_preconditioner: lem is null");
    if (net)
        if (int sc = unet_check_shape(net, L->grid.n_rows, L->grid.n_cols)) return sc;
    L->net = net;
    return LSDTT_GPU_OK;
}

int lsdtt_gpu_route_host(const lsdtt_gpu_grid* grid, const float* z_host, const std::uint8_t* mask_host,
                         float min_slope, const lsdtt_gpu_flow_options* options, float* filled_host,
                         std::int64_t* receiver_host, std::int64_t* topo_host, std::uint64_t* counts_host,
                         void* stream)
{
    // One engine per grid shape, kept across calls on this thread.
    thread_local lsdtt_gpu_flow* flow = nullptr;
    thread_local float* zd = nullptr;
    thread_local float* fd = nullptr;
    thread_local std::uint8_t* md = nullptr;
    thread_local std::int64_t cap = 0;
    if (!grid || !z_host || !mask_host) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_route_host: null argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const std::int64_t n = static_cast<std::int64_t>(grid->n_rows) * grid->n_cols;
    if (!flow || flow->g.nr != grid->n_rows || flow->g.nc != grid->n_cols || flow->g.cell != grid->cell_size ||
        std::memcmp(flow->g.bc, grid->boundary_conditions, 4) != 0)
    {
        if (flow) lsdtt_gpu_flow_destroy(flow);
        flow = nullptr;
        int s = lsdtt_gpu_flow_create(grid, &flow);
        if (s != LSDTT_GPU_OK) return s;
    }
    if (cap < n)
    {
        cudaFree(zd);
        cudaFree(fd);
        cudaFree(md);
        cudaError_t e = cudaMalloc(&zd, sizeof(float) * n);
        if (e == cudaSuccess) e = cudaMalloc(&fd, sizeof(float) * n);
        if (e == cudaSuccess) e = cudaMalloc(&md, n);
        if (e != cudaSuccess)
        {
            cap = 0;
            return cuda_fail(e, "lsdtt_gpu_route_host");
        }
        cap = n;
    }
    cudaMemcpyAsync(zd, z_host, sizeof(float) * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(md, mask_host, n, cudaMemcpyHostToDevice, st);
    int s = lsdtt_gpu_fill_pits(grid, zd, md, min_slope, fd, stream);
    if (s != LSDTT_GPU_OK) return s;
    s = lsdtt_gpu_flow_build(flow, fd, md, options, nullptr, 0, stream);
    if (s != LSDTT_GPU_OK) return s;
    if (filled_host) cudaMemcpyAsync(filled_host, fd, sizeof(float) * n, cudaMemcpyDeviceToHost, st);
    if (receiver_host) cudaMemcpyAsync(receiver_host, flow->receiver, sizeof(std::int64_t) * n, cudaMemcpyDeviceToHost, st);
    if (topo_host && flow->has_topo)
        cudaMemcpyAsync(topo_host, flow->topo, sizeof(std::int64_t) * flow->n_valid, cudaMemcpyDeviceToHost, st);
    if (counts_host && flow->has_sv)
        cudaMemcpyAsync(counts_host, flow->sv_size, sizeof(std::uint64_t) * n, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_route_host");
    return LSDTT_GPU_OK;
}

}  // extern "C"

namespace lsdtt_gb300
{
LSDTT_DEFINE_LAUNCH_READER(lem)
}  // namespace lsdtt_gb300
