// stream_power.cu -- implicit D8 stream-power incision (Braun & Willett 2013).
//
// Reference: compute_d8_stream_power_incision (src/cpu/lsdtt_stream_power_cpu.
// cpp:159-326). The reference sweeps the reverse topological order; each
// cell reads only its own old elevation and its receiver's NEW elevation, so
// any order that finalises a receiver before its donors gives the same bits.
// Here cells are grouped by depth below their outlet (from the Euler tour)
// and each depth level is one parallel step. The arithmetic keeps the
// reference's operand types: float elevations, double kam = K*w*A^m,
// float dt/dx_eff, the n = 1 closed form in double rounded to float, and for
// n != 1 the same Newton iteration (double epsilon, float updates, at most
// 100 iterations, then the rise guard and the over-excavation clamp).

#include <cmath>
#include <cstdlib>
#include <vector>

#include "engine.cuh"

namespace lsdtt_gb300
{
namespace
{

__global__ void depth_hist(const std::uint8_t* __restrict__ mask, const std::int32_t* __restrict__ depth, std::int64_t n,
                           std::uint32_t* __restrict__ count, unsigned long long* __restrict__ maxd)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n || !mask[i]) return;
    const int d = depth[i];
    atomicAdd(&count[d], 1u);
    atomicMax(maxd, static_cast<unsigned long long>(d));
}

__global__ void depth_scatter(const std::uint8_t* __restrict__ mask, const std::int32_t* __restrict__ depth,
                              std::int64_t n, const std::uint32_t* __restrict__ start, std::uint32_t* __restrict__ fillc,
                              std::uint32_t* __restrict__ order)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n || !mask[i]) return;
    const int d = depth[i];
    const std::uint32_t p = start[d] + atomicAdd(&fillc[d], 1u);
    order[p] = static_cast<std::uint32_t>(i);
}

__global__ void copy_f32(const float* __restrict__ a, float* __restrict__ b, std::int64_t n)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) b[i] = a[i];
}

struct SpParams
{
    float K, m, n, dt, threshold, slope_clamp, dx, dx_diag;
    int divide_by_dx;
    int n_is_one;
};

__global__ void sp_level(Grid g, SpParams P, const std::uint32_t* __restrict__ order, std::uint32_t lo, std::uint32_t hi,
                         const std::int64_t* __restrict__ receiver, const std::uint8_t* __restrict__ dir,
                         const double* __restrict__ area_d, const float* __restrict__ z_old,
                         const float* __restrict__ kfield, float* __restrict__ z)
{
    LSDTT_COUNT();
    const std::uint32_t k = lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= hi) return;
    const std::uint32_t flat = order[k];
    const std::int64_t recv = receiver[flat];
    if (recv < 0 || recv >= g.n) return;  // outlets and nodata are not eroded
    const float dx_eff = (dir[flat] & 1u) ? P.dx_diag : P.dx;
    double area = area_d[flat];
    if (P.divide_by_dx) area = __ddiv_rn(area, static_cast<double>(P.dx));
    if (P.threshold > 0.0f && area < static_cast<double>(P.threshold)) return;
    const float zo = z_old[flat];
    const float zr = z[recv];
    if (zr >= zo) return;
    const double tol = __dmul_rn(static_cast<double>(P.slope_clamp), static_cast<double>(dx_eff));
    const float Ki = kfield ? kfield[flat] : P.K;
    const double kam = __dmul_rn(static_cast<double>(Ki), pow(area, static_cast<double>(P.m)));
    float zn = zo;
    if (P.n_is_one)
    {
        const double spf = __dmul_rn(kam, static_cast<double>(__fdiv_rn(P.dt, dx_eff)));
        const double num = __dadd_rn(static_cast<double>(zo), __dmul_rn(static_cast<double>(zr), spf));
        zn = static_cast<float>(__ddiv_rn(num, __dadd_rn(1.0, spf)));
        if (__fsub_rn(zn, zo) > static_cast<float>(tol) || isnan(zn)) zn = zo;
    }
    else
    {
        double eps = tol + 1.0;
        int it = 0;
        const double nd = static_cast<double>(P.n);
        const double kdt = __dmul_rn(kam, static_cast<double>(P.dt));
        const double ndx = static_cast<double>(__fdiv_rn(P.n, dx_eff));
        do
        {
            const double slope = static_cast<double>(__fdiv_rn(__fsub_rn(zn, zr), dx_eff));
            if (slope <= 0.0) eps = 0.0;
            else
            {
                const double fz = __dadd_rn(static_cast<double>(__fsub_rn(zn, zo)), __dmul_rn(kdt, pow(slope, nd)));
                const double fdz = __dadd_rn(1.0, __dmul_rn(__dmul_rn(kdt, ndx), pow(slope, __dsub_rn(nd, 1.0))));
                eps = __ddiv_rn(fz, fdz);
            }
            zn = __fsub_rn(zn, static_cast<float>(eps));
            ++it;
            if (it > 100) eps = tol / 2.0;
        } while (fabs(eps) > tol);
        if (__fsub_rn(zn, zo) > static_cast<float>(tol) || isnan(zn)) zn = zo;
        if (zn < zr) zn = __fadd_rn(zr, __fmul_rn(P.slope_clamp, dx_eff));
    }
    z[flat] = zn;
}

}  // namespace

// Device order of valid cells by depth below the outlet and the host copy of
// the level offsets; reused by every sweep of the same build.
struct DepthLevels
{
    std::uint32_t* order = nullptr;
    std::vector<std::uint32_t> start;  // [maxdepth + 2]
};

cudaError_t depth_levels(lsdtt_gpu_flow* f, DepthLevels& L, cudaStream_t st)
{
    const std::int64_t n = f->g.n;
    Scratch& ws = f->ws;
    std::uint32_t* count = ws.take<std::uint32_t>(static_cast<std::size_t>(n) + 2);
    std::uint32_t* start = ws.take<std::uint32_t>(static_cast<std::size_t>(n) + 2);
    std::uint32_t* fillc = ws.take<std::uint32_t>(static_cast<std::size_t>(n) + 2);
    L.order = ws.take<std::uint32_t>(static_cast<std::size_t>(n));
    unsigned long long* maxd = ws.take<unsigned long long>(1);
    if (!count || !start || !fillc || !L.order || !maxd) return cudaErrorMemoryAllocation;
    cudaMemsetAsync(count, 0, sizeof(std::uint32_t) * (n + 2), st);
    cudaMemsetAsync(fillc, 0, sizeof(std::uint32_t) * (n + 2), st);
    cudaMemsetAsync(maxd, 0, sizeof(unsigned long long), st);
    depth_hist<<<grid_blocks(n, 256), 256, 0, st>>>(f->mask, f->depth, n, count, maxd);
    unsigned long long hmax = 0;
    cudaMemcpyAsync(&hmax, maxd, sizeof(hmax), cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    const std::int64_t nlev = static_cast<std::int64_t>(hmax) + 1;
    e = exclusive_scan<std::uint32_t, std::uint32_t>(count, nlev + 1, start, static_cast<std::uint32_t*>(nullptr), ws,
                                                     st);
    if (e != cudaSuccess) return e;
    depth_scatter<<<grid_blocks(n, 256), 256, 0, st>>>(f->mask, f->depth, n, start, fillc, L.order);
    L.start.resize(static_cast<std::size_t>(nlev) + 1);
    cudaMemcpyAsync(L.start.data(), start, sizeof(std::uint32_t) * (nlev + 1), cudaMemcpyDeviceToHost, st);
    return cudaStreamSynchronize(st);
}

}  // namespace lsdtt_gb300

using namespace lsdtt_gb300;

extern "C" int lsdtt_gpu_stream_power_d8(lsdtt_gpu_flow* f, const float* z_dev, const float* k_field_dev, float K,
                                         float m, float n, float dt, float incision_threshold_area,
                                         std::int32_t divide_area_by_dx, float slope_clamp, float* z_out_dev,
                                         void* stream)
{
    if (!f || !z_dev || !z_out_dev) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_stream_power_d8: null argument");
    if (!f->built || !(f->has_topo || f->has_sv) || f->n_valid < 0)
        return fail(LSDTT_GPU_ESTATE, "compute_d8_stream_power_incision: the flow engine has no topological order");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const Grid& g = f->g;
    f->ws.used = 0;
    double* area = f->ws.take<double>(static_cast<std::size_t>(g.n));
    if (!area) return cuda_fail(cudaErrorMemoryAllocation, "lsdtt_gpu_stream_power_d8");
    bool exact = false;
    cudaError_t e = accumulate(f, nullptr, area, st, &exact);
    if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_stream_power_d8");
    DepthLevels L;
    e = depth_levels(f, L, st);
    if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_stream_power_d8");
    if (z_out_dev != z_dev) copy_f32<<<grid_blocks(g.n, 256), 256, 0, st>>>(z_dev, z_out_dev, g.n);
    const float* z_old = z_dev;
    float* z_tmp = nullptr;
    if (z_out_dev == z_dev)
    {
        // In place: keep the step's input as z_old.
        z_tmp = f->ws.take<float>(static_cast<std::size_t>(g.n));
        if (!z_tmp) return cuda_fail(cudaErrorMemoryAllocation, "lsdtt_gpu_stream_power_d8");
        cudaMemcpyAsync(z_tmp, z_dev, sizeof(float) * g.n, cudaMemcpyDeviceToDevice, st);
        z_old = z_tmp;
    }
    SpParams P{};
    P.K = K;
    P.m = m;
    P.n = n;
    P.dt = dt;
    P.threshold = incision_threshold_area;
    P.slope_clamp = slope_clamp;
    P.dx = static_cast<float>(g.cell);
    P.dx_diag = P.dx * static_cast<float>(1.4142135623730950488);
    P.divide_by_dx = divide_area_by_dx;
    P.n_is_one = std::fabs(n - 1.0f) < 1e-6f ? 1 : 0;
    for (std::size_t k = 1; k + 1 < L.start.size(); ++k)
    {
        const std::uint32_t lo = L.start[k], hi = L.start[k + 1];
        if (hi > lo)
            sp_level<<<grid_blocks(hi - lo, 128), 128, 0, st>>>(g, P, L.order, lo, hi, f->receiver, f->dir, area, z_old,
                                                              k_field_dev, z_out_dev);
    }
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_stream_power_d8");
    return LSDTT_GPU_OK;
}

namespace lsdtt_gb300
{
LSDTT_DEFINE_LAUNCH_READER(stream_power)
}  // namespace lsdtt_gb300
