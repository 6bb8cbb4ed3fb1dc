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
#include "sp_node.cuh"

namespace lsdtt_gb300
{
namespace
{

// Depth histogram and scatter with warp-aggregated atomics (lanes of a warp
// holding the same depth, as neighbouring cells mostly do, share one).
__global__ void depth_hist(const std::uint8_t* __restrict__ mask, const std::int32_t* __restrict__ depth, std::int64_t n,
                           std::uint32_t* __restrict__ count, unsigned long long* __restrict__ maxd)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int key = (i < n && mask[i]) ? depth[i] : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    if (key >= 0 && static_cast<int>(threadIdx.x & 31) == __ffs(peers) - 1)
    {
        atomicAdd(&count[key], static_cast<unsigned>(__popc(peers)));
        atomicMax(maxd, static_cast<unsigned long long>(key));
    }
}

__global__ void depth_scatter(const std::uint8_t* __restrict__ mask, const std::int32_t* __restrict__ depth,
                              std::int64_t n, const std::uint32_t* __restrict__ start, std::uint32_t* __restrict__ fillc,
                              std::uint32_t* __restrict__ order)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int key = (i < n && mask[i]) ? depth[i] : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    std::uint32_t base = 0;
    if (key >= 0 && lane == leader) base = atomicAdd(&fillc[key], static_cast<unsigned>(__popc(peers)));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (key >= 0) order[start[key] + base + __popc(peers & ((1u << lane) - 1u))] = static_cast<std::uint32_t>(i);
}

__global__ void copy_f32(const float* __restrict__ a, float* __restrict__ b, std::int64_t n)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) b[i] = a[i];
}

// K * A^m per node ahead of the sweep (fully parallel), in place over the
// accumulated area. With the exact accumulation path (area = count * dx^2)
// and a uniform K, counts below kKamTab take a table built with the same
// arithmetic.
constexpr int kKamTab = 4096;

__global__ void sp_kam_table(SpParams P, double dw, double* __restrict__ tab)
{
    LSDTT_COUNT();
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < kKamTab) tab[c] = sp_kam(P, static_cast<double>(c) * dw, P.K);
}

__global__ void sp_kam_pass(std::int64_t n, SpParams P, const std::uint8_t* __restrict__ mask,
                            const std::int64_t* __restrict__ receiver, const std::uint64_t* __restrict__ size,
                            const double* __restrict__ tab, const float* __restrict__ kfield, double* __restrict__ area)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n || !mask[i] || receiver[i] < 0) return;
    if (tab && size[i] < static_cast<std::uint64_t>(kKamTab))
        area[i] = tab[size[i]];
    else
        area[i] = sp_kam(P, area[i], kfield ? kfield[i] : P.K);
}

struct SweepArgs1
{
    SpParams P;
    std::int64_t n;
    const std::uint32_t* order;
    const std::uint32_t* start;  // device level offsets
    const std::int64_t* receiver;
    const std::uint8_t* dir;
    const double* kam;
    const float* z_old;
    float* z;
};

__global__ void sp_level(SweepArgs1 A, std::uint32_t lo, std::uint32_t hi)
{
    LSDTT_COUNT();
    const std::uint32_t k = lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= hi) return;
    const std::uint32_t flat = A.order[k];
    sp_node_kam(A.P, A.n, flat, A.receiver, A.dir, A.kam[flat], A.z_old, A.z);
}

// Levels k0 .. kmax in one block, a barrier between levels (the long tail
// of small levels costs one launch instead of one per level).
__global__ void __launch_bounds__(1024) sp_tail(SweepArgs1 A, int k0, int kmax)
{
    LSDTT_COUNT();
    for (int k = k0; k <= kmax; ++k)
    {
        const std::uint32_t lo = A.start[k], hi = A.start[k + 1];
        for (std::uint32_t j = lo + threadIdx.x; j < hi; j += blockDim.x)
        {
            const std::uint32_t flat = A.order[j];
            sp_node_kam(A.P, A.n, flat, A.receiver, A.dir, A.kam[flat], A.z_old, A.z);
        }
        __syncthreads();
    }
}

}  // namespace

// Device order of valid cells by depth below the outlet and the host copy of
// the level offsets; reused by every sweep of the same build.
struct DepthLevels
{
    std::uint32_t* order = nullptr;
    std::uint32_t* start_dev = nullptr;
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
    L.start_dev = start;
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
    // K * A^m per node, then the sweep: one launch per large level, the tail
    // of small levels (at most kTail cells each) in one block.
    double* tab = nullptr;
    if (exact && !k_field_dev)
    {
        tab = f->ws.take<double>(kKamTab);
        if (!tab) return cuda_fail(cudaErrorMemoryAllocation, "lsdtt_gpu_stream_power_d8");
        sp_kam_table<<<grid_blocks(kKamTab, 256), 256, 0, st>>>(P, g.cell * g.cell, tab);
    }
    sp_kam_pass<<<grid_blocks(g.n, 256), 256, 0, st>>>(g.n, P, f->mask, f->receiver, f->sv_size, tab, k_field_dev,
                                                       area);
    SweepArgs1 A{P, g.n, L.order, L.start_dev, f->receiver, f->dir, area, z_old, z_out_dev};
    constexpr std::uint32_t kTail = 2048;
    const int nlev = static_cast<int>(L.start.size()) - 1;  // levels 0 .. nlev-1
    int split = nlev;
    while (split > 1 && L.start[split] - L.start[split - 1] <= kTail) --split;
    for (int k = 1; k < split; ++k)
    {
        const std::uint32_t lo = L.start[k], hi = L.start[k + 1];
        if (hi > lo) sp_level<<<grid_blocks(hi - lo, 128), 128, 0, st>>>(A, lo, hi);
    }
    if (split < nlev) sp_tail<<<1, 1024, 0, st>>>(A, std::max(split, 1), nlev - 1);
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_stream_power_d8");
    return LSDTT_GPU_OK;
}

namespace lsdtt_gb300
{
LSDTT_DEFINE_LAUNCH_READER(stream_power)
}  // namespace lsdtt_gb300
