// queries.cu -- the lsdtt_flow_base query rasters on the GB300 D8 engine.
//
// Reference: src/cpu/lsdtt_flowinfo_cpu.cpp:2255-2965. Each query is one or
// two passes over the s-vector: a forward pass (receiver before donor:
// distance from the outlet, height above / distance to the nearest channel,
// downstream path sums) or a reverse pass (donors before their receiver:
// upslope sums and means, the farthest-ridge maximum). A forward pass reads
// only the node's receiver, so any receiver-before-donor order gives the
// reference's bits; the reverse pass adds (or compares) a receiver's donors
// in the reverse s-vector order, which here is each receiver folding its
// donors in decreasing s-vector position.
//
// On the GPU both passes are level sweeps over the depth order (depth =
// cells to the outlet, from the s-vector build): a forward pass runs depth
// 1, 2, ... with every node of a level independent; a reverse pass runs the
// deepest level first, each node gathering its donors (which sit one level
// deeper). Large levels are one launch each; the small levels of the tail
// run inside one block with a barrier between levels.
//
// Arithmetic follows the reference: double accumulators, float outputs,
// step lengths cell_size and cell_size * sqrt(2) in double.

#include <cmath>
#include <string>
#include <vector>

#include "engine.cuh"

namespace lsdtt_gb300
{
namespace
{

enum QueryKind : int
{
    kDistOutlet = 0,
    kHandThreshold = 1,
    kHandMask = 2,
    kDistChannel = 3,
    kHeightRidge = 4,
    kDistRidge = 5,
    kDownstreamSum = 6,
    kUpslopeSum = 7,
    kUpslopeMean = 8,
    kQueryKinds = 9
};

struct QArgs
{
    Grid g;
    const std::int64_t* rec;
    const std::uint8_t* dir;
    const std::uint8_t* mask;
    const std::uint64_t* size;
    const std::int64_t* start;
    const float* val;
    const std::uint8_t* vmask;
    const std::uint8_t* cmask;
    std::int64_t thr;
    int include_self;
    double dx, dxy;
    double* d0;         // forward sums (distances, path sums)
    double* d1;         // reverse-pass values (upslope maximum / sum)
    std::int64_t* i0;   // nearest channel (HAND) or count (mean)
    float* f0;          // carried elevation
    std::uint8_t* ok;   // distance-to-channel validity
};

__device__ __forceinline__ double step_of(const QArgs& A, std::int64_t f)
{
    const std::uint8_t d = A.dir[f];
    return (d == 255u || (d & 1u) == 0u) ? A.dx : A.dxy;
}

// ---- per-cell set-up ---------------------------------------------------------
__global__ void q_init(QArgs A, int kind)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.g.n) return;
    A.d0[i] = 0.0;
    if (kind == kHandThreshold || kind == kHandMask)
    {
        A.f0[i] = 0.0f;
        A.i0[i] = -1;
    }
    else if (kind == kDistChannel)
        A.ok[i] = 0;
    else if (kind == kUpslopeSum || kind == kUpslopeMean)
    {
        const bool seed = A.mask[i] && A.include_self && A.vmask[i];
        A.d1[i] = seed ? static_cast<double>(A.val[i]) : 0.0;
        A.i0[i] = seed ? 1 : 0;
    }
}

// Before the reverse pass of the farthest-ridge queries: every cell is its
// own candidate (the distance the forward pass left, and its elevation).
__global__ void q_ridge_seed(QArgs A, int kind)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.g.n) return;
    A.d1[i] = A.d0[i];
    if (kind == kHeightRidge) A.f0[i] = (A.mask[i] && A.vmask[i]) ? A.val[i] : 0.0f;
}

// ---- forward pass: one node, its receiver final ------------------------------
__device__ __forceinline__ void forward_node(const QArgs& A, int kind, std::int64_t f)
{
    const std::int64_t r = A.rec[f];
    switch (kind)
    {
    case kDistOutlet:
    case kHeightRidge:
    case kDistRidge:
        if (r == -2) return;
        A.d0[f] = A.d0[r] + step_of(A, f);
        return;
    case kHandThreshold:
    case kHandMask:
    {
        if (!A.vmask[f]) return;
        const bool ch = kind == kHandThreshold ? static_cast<std::int64_t>(A.size[f]) >= A.thr : A.cmask[f] != 0;
        if (ch)
        {
            A.f0[f] = A.val[f];
            A.i0[f] = f;
        }
        else if (r != -2 && A.i0[r] >= 0)
        {
            A.f0[f] = A.f0[r];
            A.i0[f] = A.i0[r];
        }
        return;
    }
    case kDistChannel:
    {
        if (static_cast<std::int64_t>(A.size[f]) >= A.thr)
        {
            A.d0[f] = 0.0;
            A.ok[f] = 1;
            return;
        }
        if (r == -2) return;
        if (static_cast<std::int64_t>(A.size[r]) >= A.thr)
        {
            A.d0[f] = step_of(A, f);
            A.ok[f] = 1;
        }
        else if (A.ok[r])
        {
            A.d0[f] = step_of(A, f) + A.d0[r];
            A.ok[f] = 1;
        }
        return;
    }
    case kDownstreamSum:
    {
        if (A.cmask[f])
        {
            A.d0[f] = 0.0;
            return;
        }
        const double own = A.vmask[f] ? static_cast<double>(A.val[f]) : 0.0;
        const bool terminal = r == -2 || A.cmask[r] != 0;
        A.d0[f] = terminal ? own : own + A.d0[r];
        return;
    }
    default: return;
    }
}

// ---- reverse pass: one node, its donors final ---------------------------------
// The donors of f (cells whose receiver is f), in decreasing s-vector
// position: the order the reference's reverse pass reaches them.
__device__ __forceinline__ int donors_desc(const QArgs& A, std::int64_t f, std::int64_t out[8])
{
    const int row = static_cast<int>(f / A.g.nc), col = static_cast<int>(f % A.g.nc);
    int k = 0;
    for (int d = 0; d < 8; ++d)
    {
        const Step s = resolve_step(A.g, row, col, d);
        if (s.kind != 1) continue;
        const std::int64_t nf = static_cast<std::int64_t>(s.r) * A.g.nc + s.c;
        if (nf == f || !A.mask[nf] || A.rec[nf] != f) continue;
        bool dup = false;
        for (int i = 0; i < k; ++i) dup |= (out[i] == nf);
        if (!dup) out[k++] = nf;
    }
    for (int i = 1; i < k; ++i)
    {
        const std::int64_t v = out[i];
        const std::int64_t key = A.start[v];
        int j = i - 1;
        while (j >= 0 && A.start[out[j]] < key)
        {
            out[j + 1] = out[j];
            --j;
        }
        out[j + 1] = v;
    }
    return k;
}

__device__ __forceinline__ void reverse_node(const QArgs& A, int kind, std::int64_t f)
{
    std::int64_t d[8];
    const int k = donors_desc(A, f, d);
    if (kind == kHeightRidge || kind == kDistRidge)
    {
        double up = A.d1[f];
        float fe = kind == kHeightRidge ? A.f0[f] : 0.0f;
        for (int i = 0; i < k; ++i)
            if (A.d1[d[i]] > up)
            {
                up = A.d1[d[i]];
                if (kind == kHeightRidge) fe = A.f0[d[i]];
            }
        A.d1[f] = up;
        if (kind == kHeightRidge) A.f0[f] = fe;
    }
    else
    {
        double s = A.d1[f];
        std::int64_t c = A.i0[f];
        for (int i = 0; i < k; ++i)
        {
            s += A.d1[d[i]];
            c += A.i0[d[i]];
        }
        A.d1[f] = s;
        A.i0[f] = c;
    }
}

__device__ __forceinline__ void sweep_node(const QArgs& A, int kind, bool forward, std::int64_t f)
{
    if (forward) forward_node(A, kind, f);
    else reverse_node(A, kind, f);
}

// One level [lo, hi) of the depth order (grid-stride).
__global__ void q_level(QArgs A, int kind, int forward, const std::uint32_t* __restrict__ order, std::uint32_t lo,
                        std::uint32_t hi)
{
    LSDTT_COUNT();
    for (std::uint32_t j = lo + blockIdx.x * blockDim.x + threadIdx.x; j < hi; j += gridDim.x * blockDim.x)
        sweep_node(A, kind, forward != 0, order[j]);
}

// Levels k0 .. k1 (forward: ascending; reverse: k1 down to k0) inside one
// block, a barrier between levels (the small levels of the tail).
__global__ void __launch_bounds__(1024) q_tail(QArgs A, int kind, int forward, const std::uint32_t* __restrict__ order,
                                               const std::uint32_t* __restrict__ lstart, int k0, int k1)
{
    LSDTT_COUNT();
    for (int s = 0; s <= k1 - k0; ++s)
    {
        const int k = forward ? k0 + s : k1 - s;
        const std::uint32_t lo = lstart[k], hi = lstart[k + 1];
        for (std::uint32_t j = lo + threadIdx.x; j < hi; j += blockDim.x) sweep_node(A, kind, forward != 0, order[j]);
        __syncthreads();
    }
}

// ---- depth order -------------------------------------------------------------
__global__ void q_depth_hist(std::int64_t n, const std::uint8_t* __restrict__ mask, const std::int32_t* __restrict__ depth,
                             std::uint32_t* __restrict__ count, std::uint32_t* __restrict__ maxd)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n || !mask[i]) return;
    const std::uint32_t d = static_cast<std::uint32_t>(depth[i]);
    atomicAdd(count + d, 1u);
    atomicMax(maxd, d);
}

__global__ void q_depth_scatter(std::int64_t n, const std::uint8_t* __restrict__ mask,
                                const std::int32_t* __restrict__ depth, const std::uint32_t* __restrict__ start,
                                std::uint32_t* __restrict__ fill, std::uint32_t* __restrict__ order)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n || !mask[i]) return;
    const std::uint32_t d = static_cast<std::uint32_t>(depth[i]);
    order[start[d] + atomicAdd(fill + d, 1u)] = static_cast<std::uint32_t>(i);
}

// ---- outputs ------------------------------------------------------------------
__global__ void q_output(QArgs A, int kind, float nodata, float* __restrict__ out, std::uint8_t* __restrict__ out_mask,
                         std::int64_t* __restrict__ donor_out)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.g.n) return;
    float v = nodata;
    bool has = false;
    if (A.mask[i])
    {
        switch (kind)
        {
        case kDistOutlet: v = static_cast<float>(A.d0[i]); has = true; break;
        case kHandThreshold:
        case kHandMask:
            if (A.vmask[i] && A.i0[i] >= 0) { v = A.val[i] - A.f0[i]; has = true; }
            break;
        case kDistChannel:
            if (A.ok[i]) { v = static_cast<float>(A.d0[i]); has = true; }
            break;
        case kHeightRidge:
            if (A.vmask[i]) { v = A.f0[i] - A.val[i]; has = true; }
            break;
        case kDistRidge: v = static_cast<float>(A.d1[i] - A.d0[i]); has = true; break;
        case kDownstreamSum:
            if (!A.cmask[i]) { v = static_cast<float>(A.d0[i]); has = true; }
            break;
        case kUpslopeSum: v = static_cast<float>(A.d1[i]); has = true; break;
        case kUpslopeMean:
            if (A.i0[i] > 0) { v = static_cast<float>(A.d1[i] / static_cast<double>(A.i0[i])); has = true; }
            break;
        default: break;
        }
    }
    out[i] = v;
    out_mask[i] = has ? 1 : 0;
    if (donor_out) donor_out[i] = (kind == kHandMask && A.mask[i] && A.vmask[i]) ? A.i0[i] : -1;
}

// Levels above this many cells get a launch of their own; the rest run in
// the one-block tail.
constexpr std::uint32_t kTailCells = 2048;

cudaError_t sweep(const QArgs& A, int kind, bool forward, const std::uint32_t* order, const std::uint32_t* lstart_dev,
                  const std::vector<std::uint32_t>& lstart, int k0, int k1, cudaStream_t st)
{
    if (k1 < k0) return cudaSuccess;
    auto size_of = [&](int k) { return lstart[static_cast<std::size_t>(k) + 1] - lstart[static_cast<std::size_t>(k)]; };
    // The tail: the deepest levels from where every level is small.
    int split = k1 + 1;
    while (split > k0 && size_of(split - 1) <= kTailCells) --split;
    auto big = [&](int k) -> cudaError_t {
        const std::uint32_t sz = size_of(k);
        if (sz == 0) return cudaSuccess;
        q_level<<<grid_blocks(sz, 256), 256, 0, st>>>(A, kind, forward ? 1 : 0, order, lstart[k], lstart[k] + sz);
        return cudaGetLastError();
    };
    cudaError_t e = cudaSuccess;
    if (forward)
    {
        for (int k = k0; k < split && e == cudaSuccess; ++k) e = big(k);
        if (e == cudaSuccess && split <= k1) q_tail<<<1, 1024, 0, st>>>(A, kind, 1, order, lstart_dev, split, k1);
    }
    else
    {
        if (split <= k1) q_tail<<<1, 1024, 0, st>>>(A, kind, 0, order, lstart_dev, split, k1);
        for (int k = split - 1; k >= k0 && e == cudaSuccess; --k) e = big(k);
    }
    return e == cudaSuccess ? cudaGetLastError() : e;
}

}  // namespace
}  // namespace lsdtt_gb300

using namespace lsdtt_gb300;

extern "C" int lsdtt_gpu_flow_query(lsdtt_gpu_flow* f, int32_t kind, const float* values_dev,
                                    const std::uint8_t* value_mask_dev, const std::uint8_t* channel_mask_dev,
                                    int32_t threshold, int32_t include_self, float* out_dev,
                                    std::uint8_t* out_mask_dev, std::int64_t* donor_dev, void* stream)
{
    const char* who = "lsdtt_gpu_flow_query";
    if (!f || !out_dev || !out_mask_dev) return fail(LSDTT_GPU_EINVAL, std::string(who) + ": null argument");
    if (kind < 0 || kind >= kQueryKinds) return fail(LSDTT_GPU_EINVAL, std::string(who) + ": unknown query kind");
    if (!f->built) return fail(LSDTT_GPU_ESTATE, std::string(who) + ": the flow object is not built");
    if (!f->has_sv)
        return fail(LSDTT_GPU_ESTATE, "lsdtt_flowinfo: s_vector not built - set build_s_vector = true in "
                                      "lsdtt_flowinfo_options");
    const bool need_values = kind == kHandThreshold || kind == kHandMask || kind == kHeightRidge ||
                             kind == kDownstreamSum || kind == kUpslopeSum || kind == kUpslopeMean;
    const bool need_cmask = kind == kHandMask || kind == kDownstreamSum;
    if (need_values && (!values_dev || !value_mask_dev))
        return fail(LSDTT_GPU_EINVAL, std::string(who) + ": this query needs values and their validity mask");
    if (need_cmask && !channel_mask_dev)
        return fail(LSDTT_GPU_EINVAL, std::string(who) + ": this query needs a channel (or sink) mask");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const std::int64_t n = f->g.n;
    const unsigned nb = grid_blocks(n, 256);
    Scratch& ws = f->ws;
    const std::size_t mark = ws.used;
    std::uint32_t* count = ws.take<std::uint32_t>(static_cast<std::size_t>(n) + 2);
    std::uint32_t* lstart = ws.take<std::uint32_t>(static_cast<std::size_t>(n) + 2);
    std::uint32_t* order = ws.take<std::uint32_t>(static_cast<std::size_t>(n));
    std::uint32_t* maxd = ws.take<std::uint32_t>(1);
    QArgs A{};
    A.g = f->g;
    A.rec = f->receiver;
    A.dir = f->dir;
    A.mask = f->mask;
    A.size = f->sv_size;
    A.start = f->sv_start;
    A.val = values_dev;
    A.vmask = value_mask_dev;
    A.cmask = channel_mask_dev;
    A.thr = threshold;
    A.include_self = include_self ? 1 : 0;
    A.dx = f->g.cell;
    A.dxy = f->g.cell * 1.4142135623730950488;
    A.d0 = ws.take<double>(static_cast<std::size_t>(n));
    A.d1 = ws.take<double>(static_cast<std::size_t>(n));
    A.i0 = ws.take<std::int64_t>(static_cast<std::size_t>(n));
    A.f0 = ws.take<float>(static_cast<std::size_t>(n));
    A.ok = ws.take<std::uint8_t>(static_cast<std::size_t>(n));
    if (!count || !lstart || !order || !maxd || !A.d0 || !A.d1 || !A.i0 || !A.f0 || !A.ok)
    {
        ws.used = mark;
        return fail(LSDTT_GPU_ENOMEM, std::string(who) + ": the engine's workspace is too small");
    }
    // Depth order of the valid cells.
    cudaMemsetAsync(count, 0, sizeof(std::uint32_t) * (static_cast<std::size_t>(n) + 2), st);
    cudaMemsetAsync(maxd, 0, sizeof(std::uint32_t), st);
    q_depth_hist<<<nb, 256, 0, st>>>(n, f->mask, f->depth, count, maxd);
    std::uint32_t hmax = 0;
    cudaError_t e = cudaMemcpyAsync(&hmax, maxd, sizeof(hmax), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
    {
        ws.used = mark;
        return cuda_fail(e, who);
    }
    const std::int64_t levels = static_cast<std::int64_t>(hmax) + 1;
    e = exclusive_scan<std::uint32_t, std::uint32_t>(count, levels + 1, lstart, static_cast<std::uint32_t*>(nullptr),
                                                     ws, st);
    if (e == cudaSuccess)
    {
        // count doubles as the scatter cursors
        cudaMemsetAsync(count, 0, sizeof(std::uint32_t) * static_cast<std::size_t>(levels + 1), st);
        q_depth_scatter<<<nb, 256, 0, st>>>(n, f->mask, f->depth, lstart, count, order);
    }
    std::vector<std::uint32_t> hstart(static_cast<std::size_t>(levels) + 1);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(hstart.data(), lstart, sizeof(std::uint32_t) * hstart.size(), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
    {
        ws.used = mark;
        return cuda_fail(e, who);
    }
    const int kmax = static_cast<int>(hmax);
    q_init<<<nb, 256, 0, st>>>(A, kind);
    // Forward pass from depth 1 (depth 0 holds the outlets, which keep their
    // initial state); the reverse pass from the deepest level to depth 0.
    switch (kind)
    {
    case kUpslopeSum:
    case kUpslopeMean: e = sweep(A, kind, false, order, lstart, hstart, 0, kmax, st); break;
    case kHeightRidge:
    case kDistRidge:
        e = sweep(A, kind, true, order, lstart, hstart, 1, kmax, st);
        if (e == cudaSuccess)
        {
            q_ridge_seed<<<nb, 256, 0, st>>>(A, kind);
            e = sweep(A, kind, false, order, lstart, hstart, 0, kmax, st);
        }
        break;
    default:
        // HAND and the distance to a channel also decide at the outlets
        // (a channel outlet), so their forward pass starts at depth 0.
        e = sweep(A, kind, true, order, lstart, hstart, (kind == kDistOutlet) ? 1 : 0, kmax, st);
        break;
    }
    if (e == cudaSuccess)
    {
        q_output<<<nb, 256, 0, st>>>(A, kind, static_cast<float>(f->g.nodata), out_dev, out_mask_dev, donor_dev);
        e = cudaStreamSynchronize(st);
    }
    ws.used = mark;
    return e == cudaSuccess ? LSDTT_GPU_OK : cuda_fail(e, who);
}

namespace lsdtt_gb300
{
LSDTT_DEFINE_LAUNCH_READER(queries)
}  // namespace lsdtt_gb300
