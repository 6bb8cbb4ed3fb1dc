// d8.cu -- D8 steepest-descent receivers, donor counts and the outlet list.
//
// Receivers restate build_receiver_graph_d8 (src/cpu/lsdtt_flowinfo_cpu.cpp:
// 1077-1329): for each valid cell the steepest downhill neighbour, slope
// (double)z - (double)z_nb over dx or dx*sqrt(2) in double, strict '>' so the
// first of equal slopes in direction order 0..7 wins.
//
// GB300 note: this part has very little FP64 throughput, and a double
// division per neighbour would make the kernel FP64-bound many times over.
// The kernel therefore ranks neighbours without dividing: within a direction
// class (all cardinal or all diagonal) the quotients share a divisor, so the
// exact float drop orders them; between the two class winners a float screen
// or, near a tie, two double products decide (see the comment at the
// comparison). Cells whose drop is not exact in float, and exact cross-class
// ties, take the reference's own double division. The result is the
// reference's bit for bit.
//
// Donor counts restate build_donor_counts_and_outlets_d8 (:1359-1408) as a
// gather: cell c counts the neighbours d whose direction code points back
// at c. The outlet list is the row-major compaction of valid cells with no
// receiver.

#include <algorithm>

#include "engine.cuh"
#include "d8_cell.cuh"

namespace lsdtt_gb300
{
namespace
{

// Tile t of the grid: tiles across fastest.
struct GridTiles
{
    Grid g;
    const float* z;
    const std::uint8_t* mask;
    std::int64_t* receiver;
    std::uint8_t* dir;
    float inv_card, inv_diag;
    int ntx;
    __device__ D8Job operator()(int t) const
    {
        return D8Job{g, z, mask, receiver, dir, inv_card, inv_diag, t % ntx, t / ntx, 0};
    }
};

// Tile pass, one block per 128 x 32 tile (d8_receivers_tile).
__global__ void __launch_bounds__(256, 5) receivers_kernel(Grid g, const float* __restrict__ z,
                                                        const std::uint8_t* __restrict__ mask,
                                                        const std::uint8_t* __restrict__ forced,
                                                        int interior_nodata_is_outlet, int allow_pits, float inv_card,
                                                        float inv_diag, std::int64_t* __restrict__ receiver,
                                                        std::uint8_t* __restrict__ dir,
                                                        unsigned* __restrict__ undecided)
{
    LSDTT_COUNT();
    const GridTiles jobs{g, z, mask, receiver, dir, inv_card, inv_diag, (g.nc + kD8TileCols - 1) / kD8TileCols};
    d8_receivers_tile(jobs(static_cast<int>(blockIdx.x)), forced, interior_nodata_is_outlet, allow_pits, undecided);
}

// Fixup pass: every perimeter cell, then (only when the tile pass raised the
// flag) every cell it left undecided.
__global__ void __launch_bounds__(256) receivers_fixup(Grid g, const float* __restrict__ z,
                                                       const std::uint8_t* __restrict__ mask,
                                                       const std::uint8_t* __restrict__ forced,
                                                       int interior_nodata_is_outlet, int allow_pits, float inv_card,
                                                       float inv_diag, std::int64_t* __restrict__ receiver,
                                                       std::uint8_t* __restrict__ dir,
                                                       unsigned long long* __restrict__ err,
                                                       const unsigned* __restrict__ undecided)
{
    LSDTT_COUNT();
    const std::int64_t stride = static_cast<std::int64_t>(gridDim.x) * blockDim.x;
    const std::int64_t t0 = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const std::int64_t P = d8_perimeter(g.nr, g.nc);
    for (std::int64_t i = t0; i < P; i += stride)
    {
        int row, col;
        d8_perimeter_cell(g.nr, g.nc, i, row, col);
        d8_fixup_cell(g, z, mask, forced, interior_nodata_is_outlet, allow_pits, inv_card, inv_diag, receiver, dir,
                      err, row, col, 0, 0);
    }
    if (*undecided == 0u) return;
    for (std::int64_t i = t0; i < g.n; i += stride)
        if (dir[i] == kD8Undecided)
            d8_fixup_cell(g, z, mask, forced, interior_nodata_is_outlet, allow_pits, inv_card, inv_diag, receiver,
                          dir, err, static_cast<int>(i / g.nc), static_cast<int>(i % g.nc), 0, 0);
}

// Donor counts by gather (cell c counts neighbours d with dir(d) pointing to
// c; each donor matches exactly one direction, so no de-duplication is
// needed even when periodic wrap makes two directions reach one cell) and
// outlet flags for the ordered compaction.
__global__ void __launch_bounds__(256) donors_kernel(Grid g, const std::uint8_t* __restrict__ mask,
                                                     const std::uint8_t* __restrict__ dir,
                                                     std::uint8_t* __restrict__ donors,
                                                     std::uint8_t* __restrict__ outlet_flag)
{
    LSDTT_COUNT();
    const std::int64_t flat = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (flat >= g.n) return;
    const int row = static_cast<int>(flat / g.nc), col = static_cast<int>(flat % g.nc);
    std::uint8_t cnt = 0;
    const bool valid = mask[flat] != 0;
    if (valid)
    {
        if (is_interior(g, row, col))
        {
#pragma unroll
            for (int d = 0; d < 8; ++d)
            {
                const std::int64_t nf = flat + static_cast<std::int64_t>(d8_dr(d)) * g.nc + d8_dc(d);
                if (mask[nf] && dir[nf] == ((d + 4) & 7)) ++cnt;
            }
        }
        else
        {
            for (int d = 0; d < 8; ++d)
            {
                const Step s = resolve_step(g, row, col, d);
                if (s.kind != 1) continue;
                const std::int64_t nf = static_cast<std::int64_t>(s.r) * g.nc + s.c;
                if (nf == flat) continue;
                if (mask[nf] && dir[nf] == ((d + 4) & 7)) ++cnt;
            }
        }
    }
    donors[flat] = cnt;
    outlet_flag[flat] = (valid && dir[flat] == kNoDir) ? 1 : 0;
}

__global__ void scatter_flagged(const std::uint8_t* __restrict__ flag, const std::int64_t* __restrict__ pos,
                                std::int64_t n, std::int64_t* __restrict__ out)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n && flag[i]) out[pos[i]] = i;
}

__global__ void count_valid(const std::uint8_t* __restrict__ mask, std::int64_t n, unsigned long long* acc)
{
    LSDTT_COUNT();
    std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const std::int64_t stride = static_cast<std::int64_t>(gridDim.x) * blockDim.x;
    unsigned long long c = 0;
    for (; i < n; i += stride) c += mask[i] ? 1 : 0;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(acc, c);
}

}  // namespace

cudaError_t launch_receivers(lsdtt_gpu_flow* f, const float* z, const std::uint8_t* mask,
                             const std::uint8_t* forced_plane, int interior_nodata_is_outlet,
                             int allow_pits_as_outlets, cudaStream_t st)
{
    const std::int64_t tiles = static_cast<std::int64_t>((f->g.nc + kD8TileCols - 1) / kD8TileCols) *
                               ((f->g.nr + kD8TileRows - 1) / kD8TileRows);
    const float inv_card = static_cast<float>(1.0 / f->g.cell);
    const float inv_diag = static_cast<float>(1.0 / (f->g.cell * 1.4142135623730950488));
    cudaMemsetAsync(f->dundec, 0, sizeof(unsigned), st);
    // Algorithmic bytes: z 4 + mask 1 in, direction 1 + int64 receiver 8 out.
    LSDTT_TIMED("d8_receivers", 14.0 * static_cast<double>(f->g.n), st,
                (receivers_kernel<<<static_cast<unsigned>(tiles), 256, 0, st>>>(
                    f->g, z, mask, forced_plane, interior_nodata_is_outlet, allow_pits_as_outlets, inv_card, inv_diag,
                    f->receiver, f->dir, f->dundec)));
    const std::int64_t P = d8_perimeter(f->g.nr, f->g.nc);
    const unsigned fix_blocks = static_cast<unsigned>(std::max<std::int64_t>((P + 255) / 256, 152 * 4));
    receivers_fixup<<<fix_blocks, 256, 0, st>>>(f->g, z, mask, forced_plane, interior_nodata_is_outlet,
                                                allow_pits_as_outlets, inv_card, inv_diag, f->receiver, f->dir,
                                                f->derr, f->dundec);
    return cudaGetLastError();
}

cudaError_t launch_donors_outlets(lsdtt_gpu_flow* f, cudaStream_t st)
{
    const std::int64_t n = f->g.n;
    Scratch& ws = f->ws;
    const std::size_t mark = ws.used;
    std::uint8_t* flag = ws.take<std::uint8_t>(static_cast<std::size_t>(n));
    std::int64_t* pos = ws.take<std::int64_t>(static_cast<std::size_t>(n));
    if (!flag || !pos) return cudaErrorMemoryAllocation;
    // Algorithmic bytes: direction 1 in, donor count 1 out.
    LSDTT_TIMED("d8_donors", 2.0 * static_cast<double>(n), st,
                (donors_kernel<<<grid_blocks(n, 256), 256, 0, st>>>(f->g, f->mask, f->dir, f->donors, flag)));
    cudaError_t e = exclusive_scan<std::uint8_t, std::int64_t>(flag, n, pos, f->dscal + 1, ws, st);
    if (e != cudaSuccess) return e;
    scatter_flagged<<<grid_blocks(n, 256), 256, 0, st>>>(flag, pos, n, f->outlets);
    cudaMemsetAsync(f->dscal, 0, sizeof(std::int64_t), st);
    count_valid<<<152 * 4, 256, 0, st>>>(f->mask, n, reinterpret_cast<unsigned long long*>(f->dscal));
    ws.used = mark;
    return cudaGetLastError();
}

}  // namespace lsdtt_gb300

namespace lsdtt_gb300
{
LSDTT_DEFINE_LAUNCH_READER(d8)
}  // namespace lsdtt_gb300
