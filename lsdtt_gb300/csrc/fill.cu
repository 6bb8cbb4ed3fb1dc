// fill.cu -- pit filling with an imposed minimum gradient (epsilon fill).
//
// Reference: fill_pits(raster, min_slope, bc) -> the improved priority-flood
// of Barnes et al. (2014) (src/cpu/lsdtt_raster_flow_preprocessing_cpu.cpp:
// 416-589, 707-782). Seeds are every valid cell on a non-periodic raster
// edge plus, when the interior holds any nodata, every valid cell with an
// in-bounds nodata neighbour. A cell first reached from a neighbour whose
// filled value is >= its own elevation is raised to
//     max(zeta + min_slope * d, nextafter(zeta, +inf)),   d = L or L*sqrt2 (float)
// and otherwise keeps its elevation.
//
// Two parts. The relaxation computes the value-ordered form of that rule:
// every cell's "discoverer" is its neighbour of lowest filled value (first
// in direction order N, NE, ..., NW on ties), the fixed point of
//     F(c) = z(c)                        if z(c) > m(c)
//          = raise(m(c), dir of m(c))    otherwise,   m(c) = min_nb F(nb)
// with seeds fixed at their elevation, solved by tile-local relaxation in
// shared memory (each CTA iterates its kT x kT tile to local convergence),
// repeated until no tile changes. With min_slope = 0 that fixed point is the
// reference's result (the epsilon-0 fill does not depend on the order). With
// min_slope > 0 the reference's FIFO takes raised cells in push order, not
// value order, so the fill is then rebuilt in the reference's own order by
// value windows (fill_window.cuh, fill_exact.cuh): the epsilon-0 fill fixes
// where every window starts and what it sees, the epsilon relaxation only
// estimates which window starts are worth replaying.

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>

#include "engine.cuh"
#include "fill_exact.cuh"
#include "fill_tile.cuh"

namespace lsdtt_gb300
{
namespace
{

__global__ void fill_interior_nodata(int nr, int nc, const float* __restrict__ z, const std::uint8_t* __restrict__ mask,
                                     double nodata, int* __restrict__ flag)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const std::int64_t n = static_cast<std::int64_t>(nr) * nc;
    if (i >= n) return;
    if (fill_interior_invalid(nr, nc, z, mask, nodata, i)) *flag = 1;
}

__global__ void fill_init(int nr, int nc, bool per_ns, bool per_ew, const float* __restrict__ z,
                          const std::uint8_t* __restrict__ mask, double nodata, const int* __restrict__ interior_nd,
                          float* __restrict__ F, std::uint8_t* __restrict__ kind)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const std::int64_t n = static_cast<std::int64_t>(nr) * nc;
    if (i >= n) return;
    fill_init_cell(nr, nc, per_ns, per_ew, z, mask, nodata, *interior_nd, F, kind, i);
}

// One colour of a gated pass over every tile (block (x, y) = tile (x, y));
// the other colours' blocks leave at once.
__global__ void __launch_bounds__(256) fill_relax(int nr, int nc, bool per_ns, bool per_ew, float L, float Ld,
                                                  float min_slope, const float* __restrict__ z,
                                                  const std::uint8_t* __restrict__ kind, float* __restrict__ F,
                                                  int* __restrict__ changed, const std::uint8_t* __restrict__ dirty_in,
                                                  std::uint8_t* __restrict__ dirty_out, int colour)
{
    LSDTT_COUNT();
    if (fill_colour(blockIdx.x, blockIdx.y, gridDim.x, gridDim.y, per_ns, per_ew) != colour) return;
    fill_relax_tile(nr, nc, per_ns, per_ew, L, Ld, min_slope, z, kind, F, changed, dirty_in, dirty_out, blockIdx.x,
                    blockIdx.y, gridDim.x, gridDim.y);
}

// Active tiles of a pass, one thread per tile: tile (tx, ty) is active when
// it or one of its eight neighbours (periodic axes wrap) changed in the
// previous pass. Clears dirty_out (an active tile's relaxation sets it
// again) and appends the active tiles to the list of their colour
// (list + colour * cap, warp-aggregated), counting them (cnt[colour]) and
// their cells (cnt[kFillColours]).
__global__ void fill_active(int nr, int nc, bool per_ns, bool per_ew, int ntx, int nty,
                            const std::uint8_t* __restrict__ din, std::uint8_t* __restrict__ dout,
                            std::int32_t* __restrict__ list, std::int64_t cap, unsigned long long* __restrict__ cnt)
{
    LSDTT_COUNT();
    const std::int32_t t = static_cast<std::int32_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    bool active = false;
    unsigned cells = 0;
    int colour = -1;
    if (t < ntx * nty)
    {
        const int tx = t % ntx, ty = t / ntx;
        for (int dy = -1; dy <= 1 && !active; ++dy)
            for (int dx = -1; dx <= 1; ++dx)
            {
                int yy = ty + dy, xx = tx + dx;
                if (per_ns) yy = (yy + nty) % nty;
                if (per_ew) xx = (xx + ntx) % ntx;
                if (yy < 0 || yy >= nty || xx < 0 || xx >= ntx) continue;
                if (din[yy * ntx + xx])
                {
                    active = true;
                    break;
                }
            }
        dout[t] = 0;
        if (active)
        {
            cells = static_cast<unsigned>(min(kT, nr - ty * kT)) * static_cast<unsigned>(min(kT, nc - tx * kT));
            colour = fill_colour(tx, ty, ntx, nty, per_ns, per_ew);
        }
    }
    const int lane = threadIdx.x & 31;
    const unsigned peers = __match_any_sync(0xffffffffu, colour);
    const int leader = __ffs(peers) - 1;
    unsigned long long base = 0;
    if (active && lane == leader) base = atomicAdd(&cnt[colour], static_cast<unsigned long long>(__popc(peers)));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (active) list[colour * cap + static_cast<std::int64_t>(base) + __popc(peers & ((1u << lane) - 1u))] = t;
    for (int o = 16; o > 0; o >>= 1) cells += __shfl_down_sync(0xffffffffu, cells, o);
    if (lane == 0 && cells) atomicAdd(&cnt[kFillColours], static_cast<unsigned long long>(cells));
}

// Relaxation of one colour's listed active tiles by a persistent grid (block
// w takes entries w, w + grid, ...), the tile gate skipped: one block per
// tile spent most of a late pass on inactive tiles reading their
// neighbours' flags.
__global__ void __launch_bounds__(256) fill_relax_list(int nr, int nc, bool per_ns, bool per_ew, float L, float Ld,
                                                       float min_slope, const float* __restrict__ z,
                                                       const std::uint8_t* __restrict__ kind, float* __restrict__ F,
                                                       int* __restrict__ changed,
                                                       const std::uint8_t* __restrict__ dirty_in,
                                                       std::uint8_t* __restrict__ dirty_out, int ntx, int nty,
                                                       const std::int32_t* __restrict__ list,
                                                       const unsigned long long* __restrict__ count)
{
    LSDTT_COUNT();
    const std::int64_t n = static_cast<std::int64_t>(*count);
    for (std::int64_t w = blockIdx.x; w < n; w += gridDim.x)
    {
        const int t = list[w];
        fill_relax_tile(nr, nc, per_ns, per_ew, L, Ld, min_slope, z, kind, F, changed, dirty_in, dirty_out, t % ntx,
                        t / ntx, ntx, nty, false);
        __syncthreads();  // the tile's shared arrays are staged again for the next tile
    }
}

}  // namespace
}  // namespace lsdtt_gb300

using namespace lsdtt_gb300;

namespace
{

// The relaxation from fill_init to its fixed point with raise step `eps`
// (0: the epsilon-0 fill) into F. Work buffers are the caller's.
cudaError_t relax_fill(int nr, int nc, bool per_ns, bool per_ew, float L, float Ld, float eps, const float* z_dev,
                       const std::uint8_t* mask_dev, double nodata, float* F, std::uint8_t* kind, int* flags,
                       int* hflag, std::uint8_t* dirty, std::int32_t* list, unsigned long long* cnt,
                       unsigned long long* hcnt, cudaStream_t st, bool* converged)
{
    *converged = false;
    const std::int64_t n = static_cast<std::int64_t>(nr) * nc;
    const std::int64_t ntiles = static_cast<std::int64_t>((nc + kT - 1) / kT) * ((nr + kT - 1) / kT);
    cudaError_t e = cudaMemsetAsync(flags, 0, sizeof(int) * 2, st);
    cudaMemsetAsync(dirty, 1, static_cast<std::size_t>(2 * ntiles), st);
    fill_interior_nodata<<<grid_blocks(n, 256), 256, 0, st>>>(nr, nc, z_dev, mask_dev, nodata, flags);
    fill_init<<<grid_blocks(n, 256), 256, 0, st>>>(nr, nc, per_ns, per_ew, z_dev, mask_dev, nodata, flags, F, kind);
    const dim3 block(32, 8);
    const dim3 tiles((nc + kT - 1) / kT, (nr + kT - 1) / kT);
    // Global passes until no tile changes; the change flag is read back every
    // few passes to keep the host out of the loop.
    const int kCheckEvery = 4;
    const long max_pass = 4L * (nr + nc) + 64;  // bound: any path crosses each tile row/column at most a few times
    const int ntx = static_cast<int>(tiles.x), nty = static_cast<int>(tiles.y);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const unsigned list_grid = static_cast<unsigned>(std::max(1, sms) * 8);
    const unsigned colours = fill_colour_mask(ntx, nty, per_ns, per_ew);
    long pass = 0;
    while (e == cudaSuccess)
    {
        cudaMemsetAsync(flags + 1, 0, sizeof(int), st);
        for (int k = 0; k < kCheckEvery && e == cudaSuccess; ++k, ++pass)
        {
            // Each pass lists its active tiles by colour, then relaxes each
            // colour's in turn. Algorithmic bytes per pass: z 4 + mask 1
            // in, filled value 4 out per relaxed cell (counted when
            // profiling).
            const std::uint8_t* din = dirty + (pass & 1) * ntiles;
            std::uint8_t* dout = dirty + ((pass + 1) & 1) * ntiles;
            cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * (kFillColours + 1), st);
            fill_active<<<grid_blocks(ntiles, 256), 256, 0, st>>>(nr, nc, per_ns, per_ew, ntx, nty, din, dout, list,
                                                                   ntiles, cnt);
            double bytes = 9.0 * static_cast<double>(n);
            if (profiling_enabled())
            {
                cudaMemcpyAsync(hcnt, cnt, sizeof(unsigned long long) * (kFillColours + 1), cudaMemcpyDeviceToHost,
                                st);
                e = cudaStreamSynchronize(st);
                bytes = 9.0 * static_cast<double>(hcnt[kFillColours]);
            }
            LSDTT_TIMED("fill_relax", bytes, st, ({
                            for (int c = 0; c < kFillColours; ++c)
                            {
                                if (!((colours >> c) & 1u)) continue;
                                fill_relax_list<<<list_grid, block, 0, st>>>(nr, nc, per_ns, per_ew, L, Ld, eps, z_dev,
                                                                             kind, F, flags + 1, din, dout, ntx, nty,
                                                                             list + c * ntiles, cnt + c);
                            }
                        }));
        }
        if (e != cudaSuccess) break;
        cudaMemcpyAsync(hflag, flags + 1, sizeof(int), cudaMemcpyDeviceToHost, st);
        e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) break;
        if (*hflag == 0)
        {
            *converged = true;
            break;
        }
        if (pass > max_pass) break;
    }
    return e;
}

// Bytes the exact-fill stages need for one nr x nc grid (beyond F0).
std::size_t exact_single_bytes(std::int64_t n)
{
    const std::int64_t N = (n + 255) / 256 * 256;
    std::int64_t fcap = 2;
    while (fcap < n) fcap <<= 1;
    return ex_round(sizeof(ExMember)) + ex_round(sizeof(std::uint16_t) * static_cast<std::size_t>(N / 256)) +
           ex_bytes(N, 1, fcap);
}

// The fill in the reference's order for one grid: the exact-fill stages with
// a single member, in the caller's buffer `buf` of exact_single_bytes(n)
// bytes. F holds the epsilon relaxation on entry. Allocates nothing.
cudaError_t exact_fill_single_in(int nr, int nc, bool per_ns, bool per_ew, float L, float Ld, float eps, float nodata,
                                 const float* z, const std::uint8_t* kind, const float* F0, float* F, char* buf,
                                 cudaStream_t st, unsigned* failure)
{
    *failure = 0;
    const std::int64_t n = static_cast<std::int64_t>(nr) * nc;
    const std::int64_t N = (n + 255) / 256 * 256;
    std::int64_t fcap = 2;
    while (fcap < n) fcap <<= 1;
    ExMember hm{};
    hm.base = 0;
    hm.fifo_base = 0;
    hm.fifo_cap = static_cast<std::uint32_t>(fcap);
    hm.nr = nr;
    hm.nc = nc;
    hm.L = L;
    hm.Ld = Ld;
    hm.eps = eps;
    hm.nodata = nodata;
    hm.per_ns = per_ns ? 1 : 0;
    hm.per_ew = per_ew ? 1 : 0;
    hm.on = 1;
    const std::size_t meta = ex_round(sizeof(ExMember)) + ex_round(sizeof(std::uint16_t) * static_cast<std::size_t>(N / 256));
    const std::size_t bytes = exact_single_bytes(n);
    ExMember* mem = reinterpret_cast<ExMember*>(buf);
    std::uint16_t* blk = reinterpret_cast<std::uint16_t*>(buf + ex_round(sizeof(ExMember)));
    Scratch ws{buf + meta, bytes - meta, 0};
    ExBuffers B{};
    cudaError_t e = cudaSuccess;
    if (!ex_carve(ws, N, 1, fcap, B)) e = cudaErrorMemoryAllocation;
    // the member table travels by a kernel argument-free path: a host-to-
    // device copy from pageable memory is synchronous and allocates nothing
    if (e == cudaSuccess) e = cudaMemcpyAsync(mem, &hm, sizeof(ExMember), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(blk, 0, sizeof(std::uint16_t) * static_cast<std::size_t>(N / 256), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.chain_order, 0, sizeof(std::int32_t), st);
    if (e == cudaSuccess) e = ex_setup();
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = ex_run(mem, blk, N, 1, 0, z, kind, F0, F, B, ws, std::max(sms, 1), st);
    unsigned hu[6] = {0, 0, 0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(hu, B.u, sizeof(hu), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) *failure = hu[5];
    return e;
}

// The same with its buffer allocated (stream-ordered) and released here.
cudaError_t exact_fill_single(int nr, int nc, bool per_ns, bool per_ew, float L, float Ld, float eps, float nodata,
                              const float* z, const std::uint8_t* kind, const float* F0, float* F, cudaStream_t st,
                              unsigned* failure)
{
    *failure = 0;
    char* buf = nullptr;
    cudaError_t e = cudaMallocAsync(&buf, exact_single_bytes(static_cast<std::int64_t>(nr) * nc), st);
    if (e != cudaSuccess) return e;
    e = exact_fill_single_in(nr, nc, per_ns, per_ew, L, Ld, eps, nodata, z, kind, F0, F, buf, st, failure);
    cudaFreeAsync(buf, st);
    return e;
}

}  // namespace

extern "C" int lsdtt_gpu_fill_pits(const lsdtt_gpu_grid* grid, const float* z_dev, const std::uint8_t* mask_dev,
                                   float min_slope, float* out_dev, void* stream)
{
    if (!grid || !z_dev || !mask_dev || !out_dev) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_fill_pits: null argument");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(LSDTT_GPU_ENODEV, "lsdtt_gpu_fill_pits: no CUDA device");
    if (!(grid->n_rows > 0 && grid->n_cols > 0 && grid->cell_size > 0.0))
        return fail(LSDTT_GPU_EINVAL, "lsdtt::fill_pits: invalid raster metadata");
    auto is_p = [&](int i) { return grid->boundary_conditions[i] == 'p' || grid->boundary_conditions[i] == 'P'; };
    const bool per_ns = is_p(0), per_ew = is_p(1);
    const std::string bc(grid->boundary_conditions, 4);
    if (per_ns != is_p(2))
        return fail(LSDTT_GPU_EINVAL,
                    "lsdtt::fill_pits: north and south periodic flags must match (boundary_conditions '" + bc + "')");
    if (per_ew != is_p(3))
        return fail(LSDTT_GPU_EINVAL,
                    "lsdtt::fill_pits: east and west periodic flags must match (boundary_conditions '" + bc + "')");
    if (per_ns && per_ew)
        return fail(LSDTT_GPU_EINVAL, "lsdtt::fill_pits: boundary_conditions '" + bc +
                                          "' is periodic in BOTH directions, so the grid has no drainage exit at all "
                                          "and every cell would fill to the global maximum. Leave one pair open.");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int nr = grid->n_rows, nc = grid->n_cols;
    const std::int64_t n = static_cast<std::int64_t>(nr) * nc;
    const float eps = min_slope > 0.0f ? min_slope : 0.0f;
    if (eps > 0.0f && n > (std::int64_t(1) << 31))
        return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_fill_pits: grids above 2^31 cells are not supported with min_slope > 0");
    std::uint8_t* kind = nullptr;
    int* flags = nullptr;   // [0] interior nodata, [1] changed
    int* hflag = nullptr;
    std::uint8_t* dirty = nullptr;  // two per-tile activity planes
    std::int32_t* list = nullptr;   // active tiles of the current pass, by colour
    unsigned long long* cnt = nullptr;  // their count and cells
    unsigned long long* hcnt = nullptr;
    float* F0 = nullptr;            // epsilon-0 fill (min_slope > 0 only)
    const std::int64_t ntiles = static_cast<std::int64_t>((nc + kT - 1) / kT) * ((nr + kT - 1) / kT);
    cudaError_t e = cudaMallocAsync(&kind, static_cast<std::size_t>(n), st);
    if (e == cudaSuccess) e = cudaMallocAsync(&dirty, static_cast<std::size_t>(2 * ntiles), st);
    if (e == cudaSuccess)
        e = cudaMallocAsync(&list, sizeof(std::int32_t) * kFillColours * static_cast<std::size_t>(ntiles), st);
    if (e == cudaSuccess) e = cudaMallocAsync(&cnt, sizeof(unsigned long long) * (kFillColours + 1), st);
    if (e == cudaSuccess) e = cudaMallocAsync(&flags, sizeof(int) * 2, st);
    if (e == cudaSuccess && eps > 0.0f) e = cudaMallocAsync(&F0, sizeof(float) * static_cast<std::size_t>(n), st);
    if (e == cudaSuccess) e = cudaMallocHost(&hflag, sizeof(int));
    if (e == cudaSuccess) e = cudaMallocHost(&hcnt, sizeof(unsigned long long) * (kFillColours + 1));
    const float L = static_cast<float>(grid->cell_size);
    const float Ld = L * static_cast<float>(1.4142135623730950488);
    bool converged = true;
    unsigned failure = 0;
    if (e == cudaSuccess)
        e = relax_fill(nr, nc, per_ns, per_ew, L, Ld, eps, z_dev, mask_dev, grid->no_data_value, out_dev, kind, flags,
                       hflag, dirty, list, cnt, hcnt, st, &converged);
    if (e == cudaSuccess && converged && eps > 0.0f)
    {
        e = relax_fill(nr, nc, per_ns, per_ew, L, Ld, 0.0f, z_dev, mask_dev, grid->no_data_value, F0, kind, flags,
                       hflag, dirty, list, cnt, hcnt, st, &converged);
        if (e == cudaSuccess && converged)
            e = exact_fill_single(nr, nc, per_ns, per_ew, L, Ld, eps, static_cast<float>(grid->no_data_value), z_dev,
                                  kind, F0, out_dev, st, &failure);
    }
    cudaFreeAsync(kind, st);
    cudaFreeAsync(dirty, st);
    cudaFreeAsync(list, st);
    cudaFreeAsync(cnt, st);
    cudaFreeAsync(flags, st);
    cudaFreeAsync(F0, st);
    cudaFreeHost(hflag);
    cudaFreeHost(hcnt);
    if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_fill_pits");
    if (!converged) return fail(LSDTT_GPU_ETIMEOUT, "lsdtt_gpu_fill_pits: relaxation did not converge");
    if (failure)
        return fail(LSDTT_GPU_EOVERFLOW, failure == 1 ? "lsdtt_gpu_fill_pits: a fill window outgrew its arrays"
                                                      : "lsdtt_gpu_fill_pits: the fill window chain did not advance");
    return LSDTT_GPU_OK;
}

namespace lsdtt_gb300
{
LSDTT_DEFINE_LAUNCH_READER(fill)
}  // namespace lsdtt_gb300

// ---------------------------------------------------------------------------
// lsdtt_gpu_fill_pits_noalloc -- the same fill with no device allocation.
//
// Some callers cannot let a library allocate device memory: a host framework
// whose caching allocator has already reserved the device's memory and
// budgets every byte itself, or a latency-critical loop where a
// cudaMallocAsync that has to grow its pool (or fails when the pool is
// exhausted) is not acceptable. For them this entry point takes its working
// memory -- the per-cell state plane, the two per-tile activity planes, the
// convergence flags and, with min_slope > 0, the epsilon-0 fill and the
// buffers of the window replays that put the raised cells in the
// reference's order -- from one fixed array that lives in this file:
//
//   * The array is a file-scope __device__ variable of kFillNoAllocBytes
//     (64 MiB + 64 KiB), allocated when the library is loaded and held by
//     every GPU that loads it until the process exits.
//   * With min_slope <= 0 it fits grids of up to about 67 million cells
//     (8192 x 8192); with min_slope > 0 the replays need about 240 bytes a
//     cell, so up to about 270,000 cells (520 x 520). Larger grids are
//     rejected with LSDTT_GPU_EINVAL before any work is queued.
//   * Host code cannot use the array's name as a device address, so the
//     first call in each CUDA context looks the address up with
//     cudaGetSymbolAddress (with that device current) and caches it under
//     the context's process-unique id; a context created after the last
//     lookup (for example after cudaDeviceReset tore the primary context
//     down, which unloads the module and may move the array) looks it up
//     again. Make the first call on a device before any stream capture.
//   * Every call reuses the same array and clears the parts that must start
//     from a known state. Calls whose work overlaps on the GPU (different
//     streams, or host threads without ordering) race on the array; keep
//     them on one stream or otherwise ordered.
// The caller still provides the input and output buffers.
// ---------------------------------------------------------------------------
static constexpr std::size_t kFillNoAllocBytes = (std::size_t(64) << 20) + (std::size_t(64) << 10);
static __device__ __align__(256) unsigned char g_fill_noalloc_scratch[kFillNoAllocBytes];

static std::mutex g_fill_noalloc_mu;
// Per device: the context the cached address belongs to (its
// process-unique id from cuCtxGetId, 0 = none yet) and the address.
static unsigned long long g_fill_noalloc_ctx[256] = {};
static void* g_fill_noalloc_addr[256] = {};

// Process-unique id of the calling thread's current context (the driver's
// cuCtxGetCurrent / cuCtxGetId, reached through the runtime's entry-point
// query so the library needs no link against the driver library).
static cudaError_t current_context_id(unsigned long long* id)
{
    using get_current_t = int (*)(void**);
    using get_id_t = int (*)(void*, unsigned long long*);
    static get_current_t get_current = nullptr;
    static get_id_t get_id = nullptr;
    if (!get_current || !get_id)
    {
        void* f0 = nullptr;
        void* f1 = nullptr;
        cudaDriverEntryPointQueryResult q0 = cudaDriverEntryPointSymbolNotFound, q1 = q0;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0);
        if (e == cudaSuccess) e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1);
        if (e != cudaSuccess) return e;
        if (q0 != cudaDriverEntryPointSuccess || q1 != cudaDriverEntryPointSuccess || !f0 || !f1)
            return cudaErrorNotSupported;
        get_current = reinterpret_cast<get_current_t>(f0);
        get_id = reinterpret_cast<get_id_t>(f1);
    }
    void* ctx = nullptr;
    if (get_current(&ctx) != 0 || !ctx) return cudaErrorDeviceUninitialized;
    if (get_id(ctx, id) != 0) return cudaErrorDeviceUninitialized;
    return cudaSuccess;
}

extern "C" int lsdtt_gpu_fill_pits_noalloc(const lsdtt_gpu_grid* grid, const float* z_dev,
                                           const std::uint8_t* mask_dev, float min_slope, float* out_dev,
                                           void* stream)
{
    if (!grid || !z_dev || !mask_dev || !out_dev)
        return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_fill_pits_noalloc: null argument");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(LSDTT_GPU_ENODEV, "lsdtt_gpu_fill_pits_noalloc: no CUDA device");
    {
        // every call reads flags back to the host between passes, which a
        // stream capture cannot hold: refuse before anything is enqueued
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(static_cast<cudaStream_t>(stream), &cs) != cudaSuccess)
            return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_fill_pits_noalloc: cannot query the stream's capture state");
        if (cs != cudaStreamCaptureStatusNone)
            return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_fill_pits_noalloc: the stream is capturing; this call waits on "
                                          "the host between passes and cannot be captured");
    }
    if (!(grid->n_rows > 0 && grid->n_cols > 0 && grid->cell_size > 0.0))
        return fail(LSDTT_GPU_EINVAL, "lsdtt::fill_pits: invalid raster metadata");
    auto is_p = [&](int i) { return grid->boundary_conditions[i] == 'p' || grid->boundary_conditions[i] == 'P'; };
    const bool per_ns = is_p(0), per_ew = is_p(1);
    const std::string bc(grid->boundary_conditions, 4);
    if (per_ns != is_p(2))
        return fail(LSDTT_GPU_EINVAL,
                    "lsdtt::fill_pits: north and south periodic flags must match (boundary_conditions '" + bc + "')");
    if (per_ew != is_p(3))
        return fail(LSDTT_GPU_EINVAL,
                    "lsdtt::fill_pits: east and west periodic flags must match (boundary_conditions '" + bc + "')");
    if (per_ns && per_ew)
        return fail(LSDTT_GPU_EINVAL, "lsdtt::fill_pits: boundary_conditions '" + bc +
                                          "' is periodic in BOTH directions, so the grid has no drainage exit at all "
                                          "and every cell would fill to the global maximum. Leave one pair open.");
    const int nr = grid->n_rows, nc = grid->n_cols;
    const std::int64_t n = static_cast<std::int64_t>(nr) * nc;
    const std::int64_t ntiles = static_cast<std::int64_t>((nc + kT - 1) / kT) * ((nr + kT - 1) / kT);
    const float eps = min_slope > 0.0f ? min_slope : 0.0f;
    // Layout inside the fixed array: flags (256 B), two activity planes
    // (rounded to 256 B), the per-cell state plane, then with min_slope > 0
    // the epsilon-0 fill and the window replays' buffers.
    const std::size_t dirty_bytes = (static_cast<std::size_t>(2 * ntiles) + 255) & ~std::size_t(255);
    const std::size_t kind_bytes = (static_cast<std::size_t>(n) + 255) & ~std::size_t(255);
    const std::size_t f0_bytes = eps > 0.0f ? (sizeof(float) * static_cast<std::size_t>(n) + 255) & ~std::size_t(255) : 0;
    const std::size_t need = 256 + dirty_bytes + kind_bytes + f0_bytes + (eps > 0.0f ? exact_single_bytes(n) : 0);
    if (need > kFillNoAllocBytes)
        return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_fill_pits_noalloc: a " + std::to_string(nr) + " x " +
                                          std::to_string(nc) + " grid needs " + std::to_string(need) +
                                          " bytes of scratch but the fixed scratch holds " +
                                          std::to_string(kFillNoAllocBytes) +
                                          " (about 8192 x 8192 cells at min_slope 0, 520 x 520 above); use "
                                          "lsdtt_gpu_fill_pits");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_fill_pits_noalloc");
    if (dev < 0 || dev >= 256) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_fill_pits_noalloc: device index out of range");
    // cudaSetDevice on the current device makes its primary context current
    // (it initialises the context when this thread has none yet), so the
    // context id below is the one the kernels will run in.
    e = cudaSetDevice(dev);
    if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_fill_pits_noalloc");
    unsigned long long ctx = 0;
    e = current_context_id(&ctx);
    if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_fill_pits_noalloc: current context");
    void* base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_fill_noalloc_mu);
        if (!g_fill_noalloc_addr[dev] || g_fill_noalloc_ctx[dev] != ctx)
        {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_fill_noalloc_scratch);
            if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_fill_pits_noalloc: cudaGetSymbolAddress");
            g_fill_noalloc_addr[dev] = p;
            g_fill_noalloc_ctx[dev] = ctx;
        }
        base = g_fill_noalloc_addr[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    char* cbase = static_cast<char*>(base);
    int* flags = reinterpret_cast<int*>(cbase);  // [0] interior nodata, [1] changed
    std::uint8_t* dirty = reinterpret_cast<std::uint8_t*>(cbase + 256);
    std::uint8_t* kind = reinterpret_cast<std::uint8_t*>(cbase + 256 + dirty_bytes);
    float* F0 = eps > 0.0f ? reinterpret_cast<float*>(cbase + 256 + dirty_bytes + kind_bytes) : nullptr;
    char* exbuf = cbase + 256 + dirty_bytes + kind_bytes + f0_bytes;
    const float L = static_cast<float>(grid->cell_size);
    const float Ld = L * static_cast<float>(1.4142135623730950488);
    const dim3 block(32, 8);
    const dim3 tiles((nc + kT - 1) / kT, (nr + kT - 1) / kT);
    const int kCheckEvery = 4;
    const long max_pass = 4L * (nr + nc) + 64;
    // one relaxation with raise step `step` into F; the previous call's
    // contents of the array are stale, so flags and activity are reset
    auto relax = [&](float step, float* F) -> int {
        cudaMemsetAsync(flags, 0, sizeof(int) * 2, st);
        cudaMemsetAsync(dirty, 1, static_cast<std::size_t>(2 * ntiles), st);
        fill_interior_nodata<<<grid_blocks(n, 256), 256, 0, st>>>(nr, nc, z_dev, mask_dev, grid->no_data_value, flags);
        fill_init<<<grid_blocks(n, 256), 256, 0, st>>>(nr, nc, per_ns, per_ew, z_dev, mask_dev, grid->no_data_value,
                                                      flags, F, kind);
        long pass = 0;
        int changed = 0;  // pageable host word: the read-back allocates nothing
        for (;;)
        {
            cudaMemsetAsync(flags + 1, 0, sizeof(int), st);
            const unsigned colours =
                fill_colour_mask(static_cast<int>(tiles.x), static_cast<int>(tiles.y), per_ns, per_ew);
            for (int k = 0; k < kCheckEvery; ++k, ++pass)
                for (int c = 0; c < kFillColours; ++c)
                {
                    if (!((colours >> c) & 1u)) continue;
                    fill_relax<<<tiles, block, 0, st>>>(nr, nc, per_ns, per_ew, L, Ld, step, z_dev, kind, F,
                                                        flags + 1, dirty + (pass & 1) * ntiles,
                                                        dirty + ((pass + 1) & 1) * ntiles, c);
                }
            cudaError_t re = cudaMemcpyAsync(&changed, flags + 1, sizeof(int), cudaMemcpyDeviceToHost, st);
            if (re == cudaSuccess) re = cudaStreamSynchronize(st);
            if (re != cudaSuccess) return cuda_fail(re, "lsdtt_gpu_fill_pits_noalloc");
            if (changed == 0) return LSDTT_GPU_OK;
            if (pass > max_pass)
                return fail(LSDTT_GPU_ETIMEOUT, "lsdtt_gpu_fill_pits_noalloc: relaxation did not converge");
        }
    };
    int s = relax(eps, out_dev);
    if (s != LSDTT_GPU_OK || eps <= 0.0f) return s;
    // min_slope > 0: the epsilon-0 fill, then the raised cells in the
    // reference's order (the replays' buffers carved from the same array)
    s = relax(0.0f, F0);
    if (s != LSDTT_GPU_OK) return s;
    unsigned failure = 0;
    e = exact_fill_single_in(nr, nc, per_ns, per_ew, L, Ld, eps, static_cast<float>(grid->no_data_value), z_dev, kind,
                             F0, out_dev, exbuf, st, &failure);
    if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_fill_pits_noalloc");
    if (failure)
        return fail(LSDTT_GPU_EOVERFLOW, failure == 1 ? "lsdtt_gpu_fill_pits_noalloc: a fill window outgrew its arrays"
                                                      : "lsdtt_gpu_fill_pits_noalloc: the fill window chain did not advance");
    return LSDTT_GPU_OK;
}
