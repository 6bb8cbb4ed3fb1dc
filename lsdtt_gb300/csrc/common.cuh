// common.cuh -- shared device helpers for the lsdtt_gb300 kernels.
//
// Grid conventions follow lsdtt3: row-major float32 elevations z[r*nc+c],
// a u8 validity mask (1 = valid), D8 direction codes 0..7 clockwise from north
// (N, NE, E, SE, S, SW, W, NW; odd codes are diagonals), 255 = no direction,
// receiver sentinels -1 (nodata) and -2 (outlet)
// (src/utils/lsdtt_grid_neighbours.hpp:50-51, src/core/lsdtt_types.hpp:142-144).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/lsdtt_gb300.h"

namespace lsdtt_gb300
{

constexpr std::int64_t kNodataReceiver = -1;
constexpr std::int64_t kOutletReceiver = -2;
constexpr std::uint8_t kNoDir = 255;

__host__ __device__ constexpr int d8_dr(int d)
{
    return (d == 0 || d == 1 || d == 7) ? -1 : ((d == 3 || d == 4 || d == 5) ? 1 : 0);
}
__host__ __device__ constexpr int d8_dc(int d)
{
    return (d == 1 || d == 2 || d == 3) ? 1 : ((d == 5 || d == 6 || d == 7) ? -1 : 0);
}

// Boundary codes packed for the device: N, E, S, W.
struct Grid
{
    int nr;
    int nc;
    double cell;
    double nodata;
    char bc[4];
    std::int64_t n;
};

// Result of stepping from (r, c) in direction d under the D8 router's
// boundary rules (src/cpu/lsdtt_flowinfo_cpu.cpp:101-158): 'p' wraps, 'o'/'b'
// leaves the grid through an allowed outlet, 'n' is blocked.
struct Step
{
    int kind;  // 0 blocked, 1 inside, 2 off-grid outlet
    int r, c;
};

__host__ __device__ inline Step resolve_step(const Grid& g, int r, int c, int d)
{
    Step s{0, 0, 0};
    int rr = r + d8_dr(d), cc = c + d8_dc(d);
    bool out = false;
    if (rr < 0)
    {
        if (g.bc[0] == 'p') rr = g.nr - 1;
        else if (g.bc[0] == 'o' || g.bc[0] == 'b') out = true;
        else return s;
    }
    else if (rr >= g.nr)
    {
        if (g.bc[2] == 'p') rr = 0;
        else if (g.bc[2] == 'o' || g.bc[2] == 'b') out = true;
        else return s;
    }
    if (cc < 0)
    {
        if (g.bc[3] == 'p') cc = g.nc - 1;
        else if (g.bc[3] == 'o' || g.bc[3] == 'b') out = true;
        else return s;
    }
    else if (cc >= g.nc)
    {
        if (g.bc[1] == 'p') cc = 0;
        else if (g.bc[1] == 'o' || g.bc[1] == 'b') out = true;
        else return s;
    }
    if (out) { s.kind = 2; return s; }
    s.kind = 1;
    s.r = rr;
    s.c = cc;
    return s;
}

// Receiver flat index of a cell with direction code d (0..7), honouring
// periodic wrap. Only meaningful when d != kNoDir.
__host__ __device__ inline std::int64_t receiver_from_dir(const Grid& g, std::int64_t flat, int d)
{
    const int r = static_cast<int>(flat / g.nc), c = static_cast<int>(flat % g.nc);
    const Step s = resolve_step(g, r, c, d);
    return static_cast<std::int64_t>(s.r) * g.nc + s.c;
}

__host__ __device__ inline bool is_interior(const Grid& g, int r, int c)
{
    return r > 0 && r < g.nr - 1 && c > 0 && c < g.nc - 1;
}

inline unsigned grid_blocks(std::int64_t n, int threads)
{
    std::int64_t b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    return static_cast<unsigned>(b);
}

// Device-side error word. Kernels never trap: they record the first failure
// (code in the low 32 bits, detail in the high 32) and carry on or return.
__device__ inline void raise_error(unsigned long long* err, unsigned code, unsigned detail)
{
    const unsigned long long v = (static_cast<unsigned long long>(detail) << 32) | code;
    atomicCAS(err, 0ull, v);
}

// Block-wide sum (is_max: maximum) of v over a 1-D block; valid in thread 0.
// Every thread of the block must call it. One FP64 atomic per block instead
// of one per warp: same-address FP64 atomics serialise at the L2 and cost
// more than the memory traffic of the kernels that reduce.
__device__ __forceinline__ double block_reduce_d(double v, bool is_max)
{
    __shared__ double sh_block_reduce[32];
    for (int o = 16; o > 0; o >>= 1)
    {
        const double w = __shfl_down_sync(0xffffffffu, v, o);
        v = is_max ? fmax(v, w) : v + w;
    }
    __syncthreads();  // a previous call may still be reading
    if ((threadIdx.x & 31) == 0) sh_block_reduce[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = sh_block_reduce[0];
    if (threadIdx.x == 0)
        for (int k = 1; k < static_cast<int>(blockDim.x >> 5); ++k)
            t = is_max ? fmax(t, sh_block_reduce[k]) : t + sh_block_reduce[k];
    return t;
}

__device__ __forceinline__ void block_atomic_add(double* dst, double v)
{
    const double t = block_reduce_d(v, false);
    if (threadIdx.x == 0 && t != 0.0) atomicAdd(dst, t);
}

// Sum of a float quantity: FP32 within each warp (32 terms), FP64 across the
// warps of the block and across blocks (one atomic per block). The FP64
// stage carries the cancellation-prone part of a grid-wide dot product;
// per-thread FP64 arithmetic, scarce on this part, is avoided.
__device__ __forceinline__ void block_atomic_add_f(double* dst, float v)
{
    __shared__ double sh_block_add_f[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh_block_add_f[threadIdx.x >> 5] = static_cast<double>(v);
    __syncthreads();
    if (threadIdx.x == 0)
    {
        double t = sh_block_add_f[0];
        for (int k = 1; k < static_cast<int>(blockDim.x >> 5); ++k) t += sh_block_add_f[k];
        if (t != 0.0) atomicAdd(dst, t);
    }
}

// Maximum of non-negative values: their bit patterns order like the values.
__device__ __forceinline__ void block_atomic_max_nonneg(double* dst, double v)
{
    const double t = block_reduce_d(v, true);
    if (threadIdx.x == 0) atomicMax(reinterpret_cast<unsigned long long*>(dst), __double_as_longlong(t));
}

}  // namespace lsdtt_gb300

// ---------------------------------------------------------------------------
// Instrumentation.
//
// Launch counting: block (0,0,0) thread 0 of every kernel bumps a per-
// translation-unit device counter (LSDTT_COUNT() is the first statement of
// each kernel); lsdtt_gpu_launch_count() sums the counters of every unit.
//
// Kernel timing: hot launch sites record a CUDA event pair on their own
// stream when profiling is enabled (lsdtt_gpu_profile_enable); the totals
// per kernel name are resolved by lsdtt_gpu_profile_read.
// ---------------------------------------------------------------------------
static __device__ unsigned long long g_tu_launches;

#define LSDTT_COUNT()                                                                                  \
    do                                                                                                 \
    {                                                                                                  \
        if ((blockIdx.x | blockIdx.y | blockIdx.z | threadIdx.x | threadIdx.y | threadIdx.z) == 0)     \
            atomicAdd(&g_tu_launches, 1ull);                                                           \
    } while (0)

#define LSDTT_DEFINE_LAUNCH_READER(name)                                                               \
    unsigned long long launches_##name()                                                               \
    {                                                                                                  \
        unsigned long long v = 0;                                                                      \
        cudaMemcpyFromSymbol(&v, g_tu_launches, sizeof(v));                                            \
        return v;                                                                                      \
    }

namespace lsdtt_gb300
{
bool profiling_enabled();
// Returns the pair to record around one launch (nullptrs when disabled).
void profile_begin(const char* kernel, double bytes, cudaStream_t st, cudaEvent_t* b, cudaEvent_t* e);
}  // namespace lsdtt_gb300

#define LSDTT_TIMED(name, bytes, st, launch)                                                           \
    do                                                                                                 \
    {                                                                                                  \
        cudaEvent_t _b = nullptr, _e = nullptr;                                                        \
        if (::lsdtt_gb300::profiling_enabled()) ::lsdtt_gb300::profile_begin(name, bytes, st, &_b, &_e); \
        if (_b) cudaEventRecord(_b, st);                                                               \
        launch;                                                                                        \
        if (_e) cudaEventRecord(_e, st);                                                               \
    } while (0)
