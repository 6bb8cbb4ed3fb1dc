// ensemble.cu -- batched LEM ensembles: many independent grids advanced
// together, one launch per stage over the packed cells of every member.
//
// Layout. Member k owns packed cells [base_k, base_k + nr_k*nc_k) in its own
// row-major order; bases are multiples of kPackAlign (256), so a 256-thread
// block belongs to exactly one member and finds it in blk_member. Fill tiles
// (kT x kT) are numbered member by member (tile_member). Receivers, outlets,
// the Euler tour and the stream-power level order use packed indices, so the
// members' receiver forests form one forest and the stack code runs on it
// unchanged.
//
// Step (per member, the single-grid lsdtt_gpu_lem_step):
//   fill (optional) -> D8 receivers -> outlets -> Euler-tour s-vector
//   (contributing counts, depth) -> area = count*dx^2 -> stream power swept
//   by depth level -> linear implicit hillslope by Jacobi-PCG, per-member
//   scalars and convergence -> uplift and boundary restore -> statistics.
// The per-cell arithmetic is the single-grid code's own (d8_cell.cuh,
// fill_tile.cuh, sp_node.cuh, hs_stencil.cuh, lem_cell.cuh).
//
// Schedule. The loops whose trip counts depend on the data (fill passes,
// depth levels, PCG iterations) are host-driven in an eager step, which
// records their counts. The step is then captured as one CUDA graph with
// those counts plus margin; every loop body is gated on the device (an
// inactive fill tile, an empty level or a converged member returns at
// once), and a loop that needs more than its captured count raises an
// overflow flag. After a replay the host reads the flags with the
// statistics; on overflow it restores the step's input surface (copied at
// the start of the step), reruns the step eagerly and captures again.
//
// Autotuner. The stream-power sweep runs the large depth levels as one
// launch each and the tail of small levels inside one block (levels-per-
// block: the block walks level after level with a barrier between them).
// The split level and the block size of the level launches are chosen by
// timing the candidate schedules on the first eager step.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include <cooperative_groups.h>
#include <cuda/atomic>

#include "engine.cuh"
#include "d8_cell.cuh"
#include "fill_exact.cuh"
#include "fill_tile.cuh"
#include "hs_stencil.cuh"
#include "lem_cell.cuh"
#include "sp_node.cuh"

namespace cg = cooperative_groups;

namespace lsdtt_gb300
{
namespace
{

// Per-member constants.
struct EnsParams
{
    SpParams sp;
    Hs hs;
    float inv_card, inv_diag;
    float fill_eps, L, Ld;
    float udz, bl;
    double dw;        // dx^2, the default accumulation weight
    double rel_tol;   // hillslope PCG relative residual
    float hs_invd[5]; // Jacobi inverse diagonal for 0..4 in-domain faces (FP64 division, rounded)
    float inv_dt_f, DA_f, U_f;
    int fill_on, per_ns, per_ew, hill_on, max_iter;
};

// Flags: [0] fill changed in the last pass, [1] fill overflow, [2] depth
// overflow, [3] PCG overflow, [4] PCG not converged within max_iter,
// [5] active PCG members (eager loop), [6] fill did not converge (eager),
// [7] stream-power sweep wait limit, [8] a fill window replay failed.
constexpr int kFlags = 9;

__device__ __forceinline__ int member_of(const Packed& P, std::int64_t i)
{
    return P.blk_member[i / kPackAlign];
}

// The member of the whole block, for kernels launched with kPackAlign-thread
// blocks over the packed buffer (members are kPackAlign-aligned, so such a
// block never spans two): a block-uniform index and loads.
__device__ __forceinline__ int block_member(const Packed& P)
{
    return P.blk_member[blockIdx.x];
}

// ---- fill ----------------------------------------------------------------
__global__ void ens_interior(Packed P, const EnsParams* __restrict__ prm, const float* __restrict__ z,
                             const std::uint8_t* __restrict__ mask, int* __restrict__ nd)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const int m = block_member(P);
    const PackedMember& M = P.m[m];
    const std::int64_t local = i - M.base;
    if (local >= static_cast<std::int64_t>(M.nr) * M.nc || !prm[m].fill_on) return;
    if (fill_interior_invalid(M.nr, M.nc, z + M.base, mask + M.base, M.nodata, local)) nd[m] = 1;
}

__global__ void ens_fill_init(Packed P, const EnsParams* __restrict__ prm, const float* __restrict__ z,
                              const std::uint8_t* __restrict__ mask, const int* __restrict__ nd, float* __restrict__ F,
                              std::uint8_t* __restrict__ kind)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const int m = block_member(P);
    const PackedMember& M = P.m[m];
    const EnsParams& q = prm[m];
    const std::int64_t local = i - M.base;
    if (local >= static_cast<std::int64_t>(M.nr) * M.nc)
    {
        F[i] = 0.0f;
        kind[i] = 0;
        return;
    }
    if (!q.fill_on)
    {
        F[i] = z[i];
        kind[i] = 0;
        return;
    }
    fill_init_cell(M.nr, M.nc, q.per_ns, q.per_ew, z + M.base, mask + M.base, M.nodata, nd[m], F + M.base,
                   kind + M.base, local);
}

__global__ void ens_dirty_init(std::int32_t T, const std::uint16_t* __restrict__ tile_member,
                               const EnsParams* __restrict__ prm, std::uint8_t* __restrict__ d0,
                               std::uint8_t* __restrict__ d1)
{
    LSDTT_COUNT();
    const std::int32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    const std::uint8_t v = prm[tile_member[t]].fill_on ? 1 : 0;
    d0[t] = v;
    d1[t] = v;
}

// Active tiles of a fill pass, one thread per tile: tile t is active when
// it or one of its eight neighbours in its member's tile grid (periodic axes
// wrap) changed in the previous pass. Clears dirty_out[t] (the relaxation
// of an active tile sets it again) and appends the active tiles to the list
// of their colour within their member (list + colour * T, warp-aggregated),
// counting them (cnt[colour]) and their cells (cnt[kFillColours]).
__global__ void ens_fill_active(Packed P, const EnsParams* __restrict__ prm,
                                const std::uint16_t* __restrict__ tile_member, std::int32_t T,
                                const std::uint8_t* __restrict__ din, std::uint8_t* __restrict__ dout,
                                std::int32_t* __restrict__ list, unsigned long long* __restrict__ cnt)
{
    LSDTT_COUNT();
    const std::int32_t t = static_cast<std::int32_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    bool active = false;
    unsigned cells = 0;
    int colour = -1;
    if (t < T)
    {
        const int m = tile_member[t];
        const PackedMember& M = P.m[m];
        const EnsParams& q = prm[m];
        const int local = t - M.tile_base, tx = local % M.ntx, ty = local / M.ntx;
        const std::uint8_t* d = din + M.tile_base;
        for (int dy = -1; dy <= 1 && !active; ++dy)
            for (int dx = -1; dx <= 1; ++dx)
            {
                int yy = ty + dy, xx = tx + dx;
                if (q.per_ns) yy = (yy + M.nty) % M.nty;
                if (q.per_ew) xx = (xx + M.ntx) % M.ntx;
                if (yy < 0 || yy >= M.nty || xx < 0 || xx >= M.ntx) continue;
                if (d[yy * M.ntx + xx])
                {
                    active = true;
                    break;
                }
            }
        dout[t] = 0;
        if (active)
        {
            cells = static_cast<unsigned>(min(kT, M.nr - ty * kT)) * static_cast<unsigned>(min(kT, M.nc - tx * kT));
            colour = fill_colour(tx, ty, M.ntx, M.nty, q.per_ns, q.per_ew);
        }
    }
    const int lane = threadIdx.x & 31;
    const unsigned peers = __match_any_sync(0xffffffffu, colour);
    const int leader = __ffs(peers) - 1;
    unsigned long long base = 0;
    if (active && lane == leader) base = atomicAdd(&cnt[colour], static_cast<unsigned long long>(__popc(peers)));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (active)
        list[static_cast<std::int64_t>(colour) * T + static_cast<std::int64_t>(base) +
             __popc(peers & ((1u << lane) - 1u))] = t;
    for (int o = 16; o > 0; o >>= 1) cells += __shfl_down_sync(0xffffffffu, cells, o);
    if (lane == 0 && cells) atomicAdd(&cnt[kFillColours], static_cast<unsigned long long>(cells));
}

// Fill relaxation over one colour's listed active tiles (with eps0 at raise
// step 0: the epsilon-0 fill): a persistent grid,
// block w relaxes tiles w, w + grid, ... of the list (fill_relax_tile with its gate
// skipped: a pass over every tile spent ~0.2 ms only on inactive tiles
// reading their neighbours' flags and leaving).
__global__ void __launch_bounds__(256) ens_fill_relax_list(Packed P, const EnsParams* __restrict__ prm,
                                                           const std::uint16_t* __restrict__ tile_member,
                                                           const float* __restrict__ z,
                                                           const std::uint8_t* __restrict__ kind,
                                                           float* __restrict__ F, int* __restrict__ changed,
                                                           const std::uint8_t* __restrict__ din,
                                                           std::uint8_t* __restrict__ dout,
                                                           const std::int32_t* __restrict__ list,
                                                           const unsigned long long* __restrict__ count, int eps0)
{
    LSDTT_COUNT();
    const std::int64_t n = static_cast<std::int64_t>(*count);
    for (std::int64_t w = blockIdx.x; w < n; w += gridDim.x)
    {
        const int t = list[w];
        const int m = tile_member[t];
        const PackedMember& M = P.m[m];
        const EnsParams& q = prm[m];
        const int local = t - M.tile_base;
        fill_relax_tile(M.nr, M.nc, q.per_ns, q.per_ew, q.L, q.Ld, eps0 ? 0.0f : q.fill_eps, z + M.base, kind + M.base,
                        F + M.base, changed, din + M.tile_base, dout + M.tile_base, local % M.ntx, local / M.ntx,
                        M.ntx, M.nty, false);
        __syncthreads();  // the tile's shared arrays are staged again for the next tile
    }
}

// Condition of the graph's fill loop (a conditional WHILE node whose body
// is two relaxation passes): go on while the second pass changed a tile; a
// loop that reaches max_pairs still changing raises the overflow flag.
__global__ void ens_fill_while(const int* __restrict__ changed, int* __restrict__ count, int max_pairs,
                               int* __restrict__ overflow, cudaGraphConditionalHandle h)
{
    LSDTT_COUNT();
    const int c = ++*count;
    const bool more = *changed != 0;
    if (more && c >= max_pairs) *overflow = 1;
    cudaGraphSetConditional(h, (more && c < max_pairs) ? 1u : 0u);
}

__global__ void ens_flag_copy(const int* __restrict__ src, int* __restrict__ dst)
{
    LSDTT_COUNT();
    if (*src) *dst = 1;
}

__global__ void ens_flag_copy_u(const unsigned* __restrict__ src, int* __restrict__ dst)
{
    LSDTT_COUNT();
    if (*src) *dst = 1;
}

// ---- D8, outlets, area -----------------------------------------------------
// Receiver tile t of the ensemble: a 128 x 32 tile of one member's grid,
// receivers written as packed indices.
struct MemberTiles
{
    Packed P;
    const EnsParams* prm;
    const std::uint16_t* rtile_member;
    const float* zf;
    const std::uint8_t* mask;
    std::int64_t* receiver;
    std::uint8_t* dir;
    __device__ D8Job operator()(int t) const
    {
        const int m = rtile_member[t];
        const PackedMember& M = P.m[m];
        const EnsParams& q = prm[m];
        const int local = t - M.rtile_base;
        return D8Job{member_grid(M), zf + M.base, mask + M.base, receiver + M.base, dir + M.base,
                     q.inv_card,      q.inv_diag,  local % M.nrx, local / M.nrx,    M.base};
    }
};

// D8 receivers, tile pass: one block per member tile (d8_receivers_tile). The
// LEM's engine: interior nodata drains, pits are outlets.
__global__ void __launch_bounds__(256, 5) ens_receivers(Packed P, const EnsParams* __restrict__ prm,
                                                     const std::uint16_t* __restrict__ rtile_member,
                                                     const float* __restrict__ zf,
                                                     const std::uint8_t* __restrict__ mask,
                                                     std::int64_t* __restrict__ receiver,
                                                     std::uint8_t* __restrict__ dir, unsigned* __restrict__ undecided)
{
    LSDTT_COUNT();
    const MemberTiles jobs{P, prm, rtile_member, zf, mask, receiver, dir};
    d8_receivers_tile(jobs(static_cast<int>(blockIdx.x)), nullptr, 1, 1, undecided);
}

// D8 receivers, fixup pass: every member's perimeter cells, then (only when
// the tile pass raised the flag) every cell it left undecided.
__global__ void __launch_bounds__(256) ens_receivers_fixup(Packed P, const EnsParams* __restrict__ prm,
                                                           std::int64_t perim, const float* __restrict__ zf,
                                                           const std::uint8_t* __restrict__ mask,
                                                           std::int64_t* __restrict__ receiver,
                                                           std::uint8_t* __restrict__ dir,
                                                           unsigned long long* __restrict__ err,
                                                           const unsigned* __restrict__ undecided)
{
    LSDTT_COUNT();
    const std::int64_t stride = static_cast<std::int64_t>(gridDim.x) * blockDim.x;
    const std::int64_t t0 = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    for (std::int64_t i = t0; i < perim; i += stride)
    {
        int lo = 0, hi = P.n_members - 1;  // last member with perim_base <= i
        while (lo < hi)
        {
            const int mid = (lo + hi + 1) >> 1;
            if (P.m[mid].perim_base <= i) lo = mid;
            else hi = mid - 1;
        }
        const PackedMember& M = P.m[lo];
        const EnsParams& q = prm[lo];
        int row, col;
        d8_perimeter_cell(M.nr, M.nc, i - M.perim_base, row, col);
        d8_fixup_cell(member_grid(M), zf + M.base, mask + M.base, nullptr, 1, 1, q.inv_card, q.inv_diag,
                      receiver + M.base, dir + M.base, err, row, col, M.base, M.base);
    }
    if (*undecided == 0u) return;
    for (std::int64_t i = t0; i < P.n; i += stride)
    {
        if (dir[i] != kD8Undecided) continue;
        const int m = P.blk_member[i / kPackAlign];
        const PackedMember& M = P.m[m];
        const EnsParams& q = prm[m];
        const std::int64_t local = i - M.base;
        d8_fixup_cell(member_grid(M), zf + M.base, mask + M.base, nullptr, 1, 1, q.inv_card, q.inv_diag,
                      receiver + M.base, dir + M.base, err, static_cast<int>(local / M.nc),
                      static_cast<int>(local % M.nc), M.base, M.base);
    }
}

__global__ void ens_outlet_flag(std::int64_t n, const std::uint8_t* __restrict__ mask,
                                const std::uint8_t* __restrict__ dir, std::uint8_t* __restrict__ flag)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) flag[i] = (mask[i] && dir[i] == kNoDir) ? 1 : 0;
}

__global__ void ens_scatter(const std::uint8_t* __restrict__ flag, const std::int64_t* __restrict__ pos,
                            std::int64_t n, std::int64_t* __restrict__ out)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n && flag[i]) out[pos[i]] = i;
}

// K * A^m per node ahead of the sweep, fully parallel (the level-ordered
// sweep then only solves each node's implicit update). A = count * dx^2
// (divided by dx when the member says so) is exact when n_valid * m < 2^53
// for dx^2 = m * 2^e (checked per member on the host): the reference's
// accumulate() total in any order (stack.cu, accumulate). Counts below
// kKamTab take a per-member table built once with the same arithmetic.
constexpr int kKamTab = 4096;

__global__ void ens_kam_table(Packed P, const EnsParams* __restrict__ prm, double* __restrict__ tab)
{
    LSDTT_COUNT();
    const std::int64_t t = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= static_cast<std::int64_t>(P.n_members) * kKamTab) return;
    const int m = static_cast<int>(t / kKamTab), c = static_cast<int>(t % kKamTab);
    const EnsParams& q = prm[m];
    tab[t] = sp_kam(q.sp, static_cast<double>(c) * q.dw, q.sp.K);
}

// Table lookups in place; nodes with larger counts (a few percent, spread
// so that about half of all warps would hold one) are appended to a compact
// list with warp-aggregated slots and done densely by ens_kam_big, so no
// warp idles through the FP64 pow for one lane.
__global__ void ens_kam(Packed P, const EnsParams* __restrict__ prm, const std::uint8_t* __restrict__ mask,
                        const std::uint8_t* __restrict__ dir, const std::uint64_t* __restrict__ size,
                        const double* __restrict__ tab, double* __restrict__ kam, std::uint32_t* __restrict__ big,
                        std::uint32_t* __restrict__ n_big)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    bool need = false;
    if (i < P.n && mask[i] && dir[i] != kNoDir)  // a valid cell with a receiver
    {
        const int m = block_member(P);
        const std::uint64_t c = size[i];
        if (c < static_cast<std::uint64_t>(kKamTab))
            kam[i] = tab[static_cast<std::int64_t>(m) * kKamTab + static_cast<std::int64_t>(c)];
        else
            need = true;
    }
    const unsigned bal = __ballot_sync(0xffffffffu, need);
    if (!bal) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(bal) - 1;
    std::uint32_t base = 0;
    if (lane == leader) base = atomicAdd(n_big, static_cast<unsigned>(__popc(bal)));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (need) big[base + __popc(bal & ((1u << lane) - 1u))] = static_cast<std::uint32_t>(i);
}

__global__ void ens_kam_big(Packed P, const EnsParams* __restrict__ prm, const std::uint64_t* __restrict__ size,
                            const std::uint32_t* __restrict__ big, const std::uint32_t* __restrict__ n_big,
                            double* __restrict__ kam)
{
    LSDTT_COUNT();
    const std::uint32_t nb = *n_big;
    for (std::uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nb; k += gridDim.x * blockDim.x)
    {
        const std::uint32_t i = big[k];
        const EnsParams& q = prm[member_of(P, i)];
        kam[i] = sp_kam(q.sp, static_cast<double>(size[i]) * q.dw, q.sp.K);
    }
}

// ---- depth levels and the stream-power sweep -------------------------------
// Depth histogram and scatter with warp-aggregated atomics: lanes of a warp
// holding the same depth (neighbouring cells mostly do) share one atomic.
__global__ void ens_depth_hist(std::int64_t n, const std::uint8_t* __restrict__ mask,
                               const std::int32_t* __restrict__ depth, std::uint32_t cap,
                               std::uint32_t* __restrict__ count, std::uint32_t* __restrict__ maxd,
                               int* __restrict__ overflow)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    int key = -1;
    if (i < n && mask[i])
    {
        const std::int32_t d = depth[i];
        if (d >= 0 && static_cast<std::uint32_t>(d) >= cap) *overflow = 1;
        else if (d >= 0) key = d;
    }
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int lane = threadIdx.x & 31;
    if (key >= 0 && lane == __ffs(peers) - 1)
    {
        atomicAdd(&count[key], static_cast<unsigned>(__popc(peers)));
        atomicMax(maxd, static_cast<std::uint32_t>(key));
    }
}

__global__ void ens_depth_scatter(std::int64_t n, const std::uint8_t* __restrict__ mask,
                                  const std::int32_t* __restrict__ depth, std::uint32_t cap,
                                  const std::uint32_t* __restrict__ start, std::uint32_t* __restrict__ fillc,
                                  std::uint32_t* __restrict__ order)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    int key = -1;
    if (i < n && mask[i])
    {
        const std::int32_t d = depth[i];
        if (d >= 0 && static_cast<std::uint32_t>(d) < cap) key = d;
    }
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    std::uint32_t base = 0;
    if (key >= 0 && lane == leader) base = atomicAdd(&fillc[key], static_cast<unsigned>(__popc(peers)));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (key >= 0)
    {
        const unsigned rank = __popc(peers & ((1u << lane) - 1u));
        order[start[key] + base + rank] = static_cast<std::uint32_t>(i);
    }
}

// Member-major depth order: the bucket of a valid cell is its member's
// packed base plus its depth (a member's depths are below its cell count, so
// members' bucket ranges do not overlap and the packed length bounds them).
// Also the deepest level of each member.
__global__ void ens_mdepth_hist(Packed P, const std::uint8_t* __restrict__ mask, const std::int32_t* __restrict__ depth,
                                std::uint32_t* __restrict__ count, std::uint32_t* __restrict__ mmax)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    long long key = -1;
    int m = 0;
    std::int32_t d = 0;
    if (i < P.n && mask[i])
    {
        d = depth[i];
        if (d >= 0)
        {
            m = member_of(P, i);
            key = P.m[m].base + d;
        }
    }
    const unsigned peers = __match_any_sync(0xffffffffu, static_cast<unsigned long long>(key));
    const int lane = threadIdx.x & 31;
    if (key >= 0 && lane == __ffs(peers) - 1)
    {
        atomicAdd(&count[key], static_cast<unsigned>(__popc(peers)));
        if (static_cast<std::uint32_t>(d) > mmax[m]) atomicMax(&mmax[m], static_cast<std::uint32_t>(d));
    }
}

__global__ void ens_mdepth_scatter(Packed P, const std::uint8_t* __restrict__ mask,
                                   const std::int32_t* __restrict__ depth, const std::uint32_t* __restrict__ start,
                                   std::uint32_t* __restrict__ fillc, std::uint32_t* __restrict__ order)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    long long key = -1;
    if (i < P.n && mask[i])
    {
        const std::int32_t d = depth[i];
        if (d >= 0) key = P.m[member_of(P, i)].base + d;
    }
    const unsigned peers = __match_any_sync(0xffffffffu, static_cast<unsigned long long>(key));
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    std::uint32_t base = 0;
    if (key >= 0 && lane == leader) base = atomicAdd(&fillc[key], static_cast<unsigned>(__popc(peers)));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (key >= 0)
    {
        const unsigned rank = __popc(peers & ((1u << lane) - 1u));
        order[start[key] + base + rank] = static_cast<std::uint32_t>(i);
    }
}

// Member-major depth order, one CTA per member (blockIdx.x = m): a
// shared-memory histogram of the member's depths (bins 0 .. cap-1), its
// exclusive scan, bucket starts start[base + d] = base + (the member's
// cells above depth d) for d = 0 .. deepest + 1, then the scatter through
// shared-memory cursors, so member m's nodes sit at order[base ..] level by
// level (within a level in no fixed order: its nodes are independent). The
// sweep reads start[base + 1 .. base + deepest + 1] and the ranges between
// them, as with the global counting sort, which needs a scan over every
// bucket of the packed grid. A depth at or beyond `cap` raises *overflow
// (the host reruns the step eagerly and captures with a larger cap).
constexpr int kMdSortThreads = 1024;
constexpr std::size_t kMdSortMaxSmem = 200 * 1024;  // bins for depths up to ~51,000 levels

__global__ void __launch_bounds__(kMdSortThreads) ens_mdepth_sort(Packed P, const std::uint8_t* __restrict__ mask,
                                                                  const std::int32_t* __restrict__ depth,
                                                                  std::uint32_t cap, std::uint32_t* __restrict__ start,
                                                                  std::uint32_t* __restrict__ order,
                                                                  std::uint32_t* __restrict__ mmax,
                                                                  int* __restrict__ overflow)
{
    LSDTT_COUNT();
    extern __shared__ std::uint32_t md_hist[];  // cap + 1 bins
    __shared__ std::uint32_t s_max, s_warp[kMdSortThreads / 32];
    __shared__ int s_over;
    const int m = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const PackedMember& M = P.m[m];
    const std::int64_t base = M.base, n = static_cast<std::int64_t>(M.nr) * M.nc;
    for (std::uint32_t k = tid; k <= cap; k += blockDim.x) md_hist[k] = 0;
    if (tid == 0)
    {
        s_max = 0;
        s_over = 0;
    }
    __syncthreads();
    std::uint32_t dmax = 0;
    for (std::int64_t l = tid; l < n; l += blockDim.x)
    {
        const std::int64_t i = base + l;
        if (!mask[i]) continue;
        const std::int32_t d = depth[i];
        if (d < 0) continue;
        if (static_cast<std::uint32_t>(d) >= cap)
        {
            s_over = 1;
            continue;
        }
        atomicAdd(&md_hist[d], 1u);
        dmax = max(dmax, static_cast<std::uint32_t>(d));
    }
    for (int o = 16; o > 0; o >>= 1) dmax = max(dmax, __shfl_down_sync(0xffffffffu, dmax, o));
    if (lane == 0) atomicMax(&s_max, dmax);
    __syncthreads();
    if (s_over)  // block-uniform
    {
        if (tid == 0) *overflow = 1;
        return;
    }
    // exclusive scan of bins 0 .. D+1 (bin D+1 is empty: the end of level D)
    const std::uint32_t D = s_max, nbins = D + 2;
    const std::uint32_t per = (nbins + blockDim.x - 1) / blockDim.x;
    const std::uint32_t lo = min(nbins, tid * per), hi = min(nbins, lo + per);
    std::uint32_t sum = 0;
    for (std::uint32_t k = lo; k < hi; ++k) sum += md_hist[k];
    std::uint32_t incl = sum;
    for (int o = 1; o < 32; o <<= 1)
    {
        const std::uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0)
    {
        const int nw = static_cast<int>(blockDim.x >> 5);
        std::uint32_t w = lane < nw ? s_warp[lane] : 0u, wi = w;
        for (int o = 1; o < 32; o <<= 1)
        {
            const std::uint32_t v = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += v;
        }
        if (lane < nw) s_warp[lane] = wi - w;  // exclusive prefix of the warps
    }
    __syncthreads();
    std::uint32_t run = s_warp[warp] + incl - sum;
    for (std::uint32_t k = lo; k < hi; ++k)
    {
        const std::uint32_t c = md_hist[k];
        md_hist[k] = run;
        start[base + k] = static_cast<std::uint32_t>(base) + run;
        run += c;
    }
    if (tid == 0) mmax[m] = D;
    __syncthreads();
    for (std::int64_t l = tid; l < n; l += blockDim.x)
    {
        const std::int64_t i = base + l;
        if (!mask[i]) continue;
        const std::int32_t d = depth[i];
        if (d < 0) continue;
        const std::uint32_t pos = atomicAdd(&md_hist[d], 1u);
        order[base + pos] = static_cast<std::uint32_t>(i);
    }
}

// The deepest level over all members.
__global__ void ens_mdepth_max(int n_members, const std::uint32_t* __restrict__ mmax, std::uint32_t* __restrict__ maxd)
{
    LSDTT_COUNT();
    std::uint32_t v = 0;
    for (int m = threadIdx.x; m < n_members; m += blockDim.x) v = max(v, mmax[m]);
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_down_sync(0xffffffffu, v, o));
    __shared__ std::uint32_t w[32];
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        std::uint32_t r = 0;
        for (int k = 0; k < static_cast<int>(blockDim.x >> 5); ++k) r = max(r, w[k]);
        *maxd = r;
    }
}

__global__ void ens_copy(const float* __restrict__ a, float* __restrict__ b, std::int64_t n)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) b[i] = a[i];
}

struct SweepArgs
{
    Packed P;
    const EnsParams* prm;
    const std::uint32_t* order;
    const std::uint32_t* start;   // level offsets, [cap + 1]
    const std::uint32_t* maxd;    // deepest level present
    const std::int64_t* receiver;
    const std::uint8_t* dir;
    const double* kam;
    const float* z_old;
    float* z;
};

__device__ __forceinline__ void sweep_node(const SweepArgs& A, std::uint32_t flat)
{
    sp_node_kam(A.prm[member_of(A.P, flat)].sp, A.P.n, flat, A.receiver, A.dir, A.kam[flat], A.z_old, A.z);
}

// One depth level (offsets read on the device; grid-stride over the level).
__global__ void ens_sp_level(SweepArgs A, int k)
{
    LSDTT_COUNT();
    const std::uint32_t lo = A.start[k], hi = A.start[k + 1];
    for (std::uint32_t j = lo + blockIdx.x * blockDim.x + threadIdx.x; j < hi; j += gridDim.x * blockDim.x)
        sweep_node(A, A.order[j]);
}

// Levels k0 .. maxd in one block: a barrier between levels orders each
// level's writes before the next level's reads.
__global__ void __launch_bounds__(1024) ens_sp_tail(SweepArgs A, int k0)
{
    LSDTT_COUNT();
    const int kmax = static_cast<int>(*A.maxd);
    for (int k = k0; k <= kmax; ++k)
    {
        const std::uint32_t lo = A.start[k], hi = A.start[k + 1];
        for (std::uint32_t j = lo + threadIdx.x; j < hi; j += blockDim.x) sweep_node(A, A.order[j]);
        __syncthreads();
    }
}

// Cooperative level sweep: one launch of co-resident blocks runs levels
// 1 .. split-1 with a grid barrier between levels, then block 0 alone runs
// the small levels split .. maxd with block barriers (as ens_sp_tail). The
// barrier is a counter plus a generation word; its wait is bounded and a
// wait that runs out sets the abort flag, which ends every other wait.
// Receiver elevations are read from L2 (other SMs wrote them).
constexpr int kBarrierSpinLimit = 1 << 22;

__device__ __forceinline__ bool ens_grid_barrier(unsigned* bar, unsigned nblocks, int* abort_flag,
                                                 int spin_limit = kBarrierSpinLimit)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        cuda::atomic_ref<unsigned, cuda::thread_scope_device> count(bar[0]), gen(bar[1]);
        cuda::atomic_ref<int, cuda::thread_scope_device> ab(*abort_flag);
        const unsigned g = gen.load(cuda::memory_order_relaxed);
        int good = 1;
        __threadfence();
        if (count.fetch_add(1u, cuda::memory_order_acq_rel) == nblocks - 1u)
        {
            count.store(0u, cuda::memory_order_relaxed);
            gen.store(g + 1u, cuda::memory_order_release);
        }
        else
        {
            int spins = 0;
            while (gen.load(cuda::memory_order_acquire) == g)
            {
                if (++spins > spin_limit || ab.load(cuda::memory_order_relaxed) != 0)
                {
                    ab.store(1, cuda::memory_order_relaxed);
                    good = 0;
                    break;
                }
            }
        }
        __threadfence();
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

__global__ void __launch_bounds__(512) ens_sp_coop(SweepArgs A, int split, unsigned* __restrict__ bar,
                                                   int* __restrict__ abort_flag)
{
    LSDTT_COUNT();
    const int kmax = static_cast<int>(*A.maxd);
    const int kend = min(split, kmax + 1);
    const std::uint32_t stride = gridDim.x * blockDim.x;
    for (int k = 1; k < kend; ++k)
    {
        const std::uint32_t lo = A.start[k], hi = A.start[k + 1];
        for (std::uint32_t j = lo + blockIdx.x * blockDim.x + threadIdx.x; j < hi; j += stride)
        {
            const std::uint32_t flat = A.order[j];
            sp_node_kam<true>(A.prm[member_of(A.P, flat)].sp, A.P.n, flat, A.receiver, A.dir, A.kam[flat], A.z_old,
                              A.z);
        }
        if (!ens_grid_barrier(bar, gridDim.x, abort_flag)) return;
    }
    if (blockIdx.x != 0) return;
    for (int k = max(kend, 1); k <= kmax; ++k)
    {
        const std::uint32_t lo = A.start[k], hi = A.start[k + 1];
        for (std::uint32_t j = lo + threadIdx.x; j < hi; j += blockDim.x)
        {
            const std::uint32_t flat = A.order[j];
            sp_node_kam<true>(A.prm[member_of(A.P, flat)].sp, A.P.n, flat, A.receiver, A.dir, A.kam[flat], A.z_old,
                              A.z);
        }
        __syncthreads();
    }
}

// Failure-detection self-test of the bounded grid barrier: one block
// arrives at a barrier that expects two arrivals, so nothing ever releases
// its wait; the wait gives up after spin_limit polls, raises the abort flag
// and the kernel reports it. bar[0..1] and *abort_flag start at zero.
__global__ void ens_barrier_selftest(unsigned* __restrict__ bar, int* __restrict__ abort_flag,
                                     int* __restrict__ released, int spin_limit)
{
    LSDTT_COUNT();
    const bool ok = ens_grid_barrier(bar, 2u, abort_flag, spin_limit);
    if (threadIdx.x == 0) *released = ok ? 1 : 0;
}

constexpr unsigned kSweepClusterBlock = 256;  // largest block of the member-cluster sweep

// One node of the member-cluster sweep with its independent loads done.
struct SweepNode
{
    std::int64_t recv;  // < 0: nothing to do
    double kam;
    std::uint32_t flat;
    float zo;
    bool diag;
};

__device__ __forceinline__ SweepNode sweep_fetch(const SweepArgs& A, std::uint32_t j, std::uint32_t hi)
{
    SweepNode v{-1, -1.0, 0u, 0.0f, false};
    if (j < hi)
    {
        v.flat = A.order[j];
        v.recv = A.receiver[v.flat];
        v.kam = A.kam[v.flat];
        v.zo = A.z_old[v.flat];
        v.diag = (A.dir[v.flat] & 1u) != 0;
        if (v.recv >= A.P.n || v.kam < 0.0) v.recv = -1;  // outlets, nodata, below threshold
    }
    return v;
}

__device__ __forceinline__ void sweep_solve(const SweepArgs& A, const SpParams& sp, const SweepNode& v)
{
    if (v.recv < 0) return;
    A.z[v.flat] = sp_solve(sp, v.diag, v.kam, v.zo, __ldcg(A.z + v.recv));
}

// Member-cluster sweep: one cluster of CTAs per member (largest members
// first), walking the member's own depth levels from the member-major order
// with the hardware cluster barrier between levels. Members do not wait on
// one another, a member's nodes of one level are spread over the cluster's
// SMs (the FP64 Newton work of a large member is not confined to one SM), and
// a level costs a cluster barrier instead of a launch or a grid barrier. Only
// the receiver's new elevation depends on the previous level: each thread
// fetches its first two nodes of level k+1 (order, receiver, K*A^m, old
// elevation, direction) between its arrival at the cluster barrier and its
// wait there, so a level up to twice the cluster's width costs one L2 load,
// the solves and the barrier.
__global__ void __launch_bounds__(kSweepClusterBlock, 2) ens_sp_clusters(SweepArgs A,
                                                                      const std::uint16_t* __restrict__ perm,
                                                                      const std::uint32_t* __restrict__ mmax)
{
    LSDTT_COUNT();
    cg::cluster_group cluster = cg::this_cluster();
    const unsigned C = cluster.num_blocks(), rank = cluster.block_rank();
    const int m = perm[blockIdx.x / C];
    const std::int64_t base = A.P.m[m].base;
    const SpParams sp = A.prm[m].sp;
    const std::uint32_t kmax = mmax[m];
    const std::uint32_t stride = C * blockDim.x, off = rank * blockDim.x + threadIdx.x;
    if (kmax == 0) return;  // whole clusters: kmax is the member's
    // every CTA of the cluster is running before any arrives at its barrier
    cluster.sync();
    std::uint32_t lo = A.start[base + 1], hi = A.start[base + 2];
    SweepNode cur0 = sweep_fetch(A, lo + off, hi), cur1 = sweep_fetch(A, lo + off + stride, hi);
    std::uint32_t nhi = kmax > 1 ? A.start[base + 3] : hi;  // end of level 2
    for (std::uint32_t k = 1; k <= kmax; ++k)
    {
        // this thread's first two nodes of the level (independent solves),
        // then any further ones (levels wider than twice the cluster)
        sweep_solve(A, sp, cur0);
        sweep_solve(A, sp, cur1);
        for (std::uint32_t j = lo + off + 2 * stride; j < hi; j += stride) sweep_solve(A, sp, sweep_fetch(A, j, hi));
        // Arrive (release: this level's elevations), then fetch the next
        // level's independent data while the cluster catches up, then wait
        // (acquire) before any receiver elevation of it is read.
        __syncwarp();  // the .aligned barrier wants converged warps
        asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
        const std::uint32_t nlo = hi;
        cur0 = sweep_fetch(A, nlo + off, nhi);
        cur1 = sweep_fetch(A, nlo + off + stride, nhi);
        const std::uint32_t nnhi = k + 1 < kmax ? A.start[base + k + 3] : nhi;
        asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
        lo = nlo;
        hi = nhi;
        nhi = nnhi;
    }
}

// In-order dataflow sweep (no level barriers). Persistent warps claim
// 64-node chunks of the level-ordered list with an atomic counter; each node
// waits until its receiver's word zg[] carries this sweep's generation,
// solves its update and publishes its own word. A word is {generation (high
// 32 bits), float bits of z (low 32)}: value and flag travel in one aligned
// 64-bit store, so neither side needs a fence. Chunks are claimed in list
// order and a receiver always precedes its donors in the list, so every
// wait is on a node already held by a running warp (or finished); within a
// chunk each lane takes its nodes in list order. Waits are bounded; a wait
// that runs out sets the abort flag, which ends every other wait at once,
// and the host reports the step as failed.
constexpr int kSpinLimit = 1 << 22;
constexpr std::uint32_t kDfChunk = 64;

__device__ __forceinline__ unsigned long long df_word(std::uint32_t gen, float z)
{
    return (static_cast<unsigned long long>(gen) << 32) | __float_as_uint(z);
}

__global__ void ens_gen_bump(std::uint32_t* __restrict__ gen)
{
    LSDTT_COUNT();
    *gen += 1u;
}

// Level 0 (outlets: not eroded) is final from the start.
__global__ void ens_mark_roots(SweepArgs A, const std::uint32_t* __restrict__ gen,
                               unsigned long long* __restrict__ zg)
{
    LSDTT_COUNT();
    const std::uint32_t g = *gen;
    const std::uint32_t lo = A.start[0], hi = A.start[1];
    for (std::uint32_t j = lo + blockIdx.x * blockDim.x + threadIdx.x; j < hi; j += gridDim.x * blockDim.x)
    {
        const std::uint32_t flat = A.order[j];
        cuda::atomic_ref<unsigned long long, cuda::thread_scope_device>(zg[flat])
            .store(df_word(g, A.z_old[flat]), cuda::memory_order_relaxed);
    }
}

__global__ void __launch_bounds__(256) ens_sp_dataflow(SweepArgs A, const std::uint32_t* __restrict__ gen,
                                                       std::uint32_t* __restrict__ next,
                                                       unsigned long long* __restrict__ zg,
                                                       int* __restrict__ abort_flag)
{
    LSDTT_COUNT();
    const std::uint32_t g = *gen;
    const std::uint32_t lo = A.start[1];
    const std::uint32_t hi = A.start[*A.maxd + 1];
    const int lane = threadIdx.x & 31;
    for (;;)
    {
        std::uint32_t c = 0;
        if (lane == 0) c = atomicAdd(next, kDfChunk);
        c = __shfl_sync(0xffffffffu, c, 0);
        if (lo + c >= hi) break;
        for (std::uint32_t k = static_cast<std::uint32_t>(lane); k < kDfChunk; k += 32)
        {
            const std::uint32_t j = lo + c + k;
            if (j >= hi) break;
            const std::uint32_t flat = A.order[j];
            const std::int64_t recv = A.receiver[flat];
            const float zo = A.z_old[flat];
            float zn = zo;
            if (recv >= 0)
            {
                cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> wr(zg[recv]);
                unsigned long long w = wr.load(cuda::memory_order_relaxed);
                int spins = 0;
                bool ok = true;
                while (static_cast<std::uint32_t>(w >> 32) != g)
                {
                    if (++spins > kSpinLimit || *reinterpret_cast<volatile int*>(abort_flag))
                    {
                        atomicExch(abort_flag, 1);
                        ok = false;
                        break;
                    }
                    __nanosleep(32);
                    w = wr.load(cuda::memory_order_relaxed);
                }
                const double kam = A.kam[flat];
                if (ok && kam >= 0.0)
                    zn = sp_solve(A.prm[member_of(A.P, flat)].sp, (A.dir[flat] & 1u) != 0, kam, zo,
                                  __uint_as_float(static_cast<std::uint32_t>(w)));
            }
            cuda::atomic_ref<unsigned long long, cuda::thread_scope_device>(zg[flat])
                .store(df_word(g, zn), cuda::memory_order_relaxed);
        }
    }
}

// The swept elevations back into z (cells this sweep did not reach keep
// theirs).
__global__ void ens_sp_extract(std::int64_t n, const std::uint32_t* __restrict__ gen,
                               const unsigned long long* __restrict__ zg, float* __restrict__ z)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long w = zg[i];
    if (static_cast<std::uint32_t>(w >> 32) == *gen) z[i] = __uint_as_float(static_cast<std::uint32_t>(w));
}

// ---- hillslope: Jacobi-PCG with per-member scalars -----------------------
// Reduction slots: slot s (s = iteration + 1; slot 0 holds r.z of the start)
// has 4 doubles per member: [0] p.Ap, [1] r.z, [2] r.r.
constexpr int kHsSlot = 4;

// Reductions are deterministic and atomic-free: each 256-cell block (one
// member's) writes its partial to part[q * nblk + block], and
// ens_member_reduce sums a member's partials in a fixed order. (FP64 atomics
// into one slot per member serialise at well under a nanosecond each and
// dominated the kernels that used them.)
// Block partial of a float quantity: summed in FP32 within each warp
// (32 terms), in FP64 across the warps of the block and across blocks.
// The FP64 stage carries the cancellation-prone part of a grid-wide dot
// product; per-thread FP64 arithmetic, scarce on this part, is avoided.
__device__ __forceinline__ void block_partial_f(float v, bool is_max, double* __restrict__ part, std::int64_t nblk,
                                                int q, std::int64_t blk = -1)
{
    if (blk < 0) blk = blockIdx.x;  // the partial's index: the block, or the block a list mapped it to
    __shared__ double shf[32];
    for (int o = 16; o > 0; o >>= 1)
    {
        const float w = __shfl_down_sync(0xffffffffu, v, o);
        v = is_max ? fmaxf(v, w) : v + w;
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) shf[threadIdx.x >> 5] = static_cast<double>(v);
    __syncthreads();
    if (threadIdx.x < 32)
    {
        // the warp partials as a shuffle tree: every FP64 instruction of a
        // warp holds this part's narrow FP64 pipe for many cycles, whatever
        // the number of active lanes
        const int nw = static_cast<int>(blockDim.x >> 5);
        double t = threadIdx.x < nw ? shf[threadIdx.x] : (is_max ? -INFINITY : 0.0);
        for (int o = 16; o > 0; o >>= 1)
        {
            if (o >= nw) continue;
            const double w = __shfl_down_sync(0xffffffffu, t, o);
            t = is_max ? fmax(t, w) : t + w;
        }
        if (threadIdx.x == 0) part[q * nblk + blk] = t;
    }
}

// block_partial_f for NQ quantities at once (NQ divides 32; bit q of
// max_mask: maximum, else sum): FP32 within each warp, then warp 0 gives
// each lane one quantity and a group of warps, sums the group in FP64 and
// combines the groups with xor shuffles: one barrier and a handful of FP64
// instructions per block for all NQ. Call once per kernel.
template <int NQ>
__device__ __forceinline__ void block_partials_f(const float (&v)[NQ], unsigned max_mask, double* __restrict__ part,
                                                 std::int64_t nblk, std::int64_t blk = -1)
{
    if (blk < 0) blk = blockIdx.x;
    static_assert(32 % NQ == 0, "NQ must divide the warp");
    __shared__ float sw[32][NQ];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = static_cast<int>(blockDim.x >> 5);
#pragma unroll
    for (int q = 0; q < NQ; ++q)
    {
        const bool is_max = (max_mask >> q) & 1u;
        float x = v[q];
        for (int o = 16; o > 0; o >>= 1)
        {
            const float y = __shfl_down_sync(0xffffffffu, x, o);
            x = is_max ? fmaxf(x, y) : x + y;
        }
        if (lane == 0) sw[wid][q] = x;
    }
    __syncthreads();
    if (wid == 0)
    {
        constexpr int G = 32 / NQ;
        const int q = lane % NQ, g = lane / NQ;
        const bool is_max = (max_mask >> q) & 1u;
        double t = is_max ? -INFINITY : 0.0;
        for (int k = g; k < nw; k += G)
        {
            const double x = static_cast<double>(sw[k][q]);
            t = is_max ? fmax(t, x) : t + x;
        }
        for (int o = NQ; o < 32; o <<= 1)
        {
            const double y = __shfl_xor_sync(0xffffffffu, t, o);
            t = is_max ? fmax(t, y) : t + y;
        }
        if (g == 0) part[q * nblk + blk] = t;
    }
}

// dst[m * stride + off + q] = reduction of member m's block partials of
// quantity q (bit q of max_mask: maximum, else sum); one warp per (m, q).
// Members with done[m] set are skipped. With shift, dst moves by
// *shift * shift_step (a device-side iteration's slot). With tile_partials
// the partials are per 128 x 32 member tile (ens_hs_apply_tiled).
__global__ void ens_member_reduce(Packed P, int nq, unsigned max_mask, const double* __restrict__ part,
                                  std::int64_t nblk, const int* __restrict__ done, double* __restrict__ dst, int stride,
                                  int off, const int* __restrict__ shift = nullptr, std::int64_t shift_step = 0,
                                  int tile_partials = 0)
{
    LSDTT_COUNT();
    if (shift) dst += static_cast<std::int64_t>(*shift) * shift_step;
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int m = w / nq, q = w % nq;
    if (m >= P.n_members) return;
    if (done && done[m]) return;
    const PackedMember& M = P.m[m];
    const bool is_max = (max_mask >> q) & 1u;
    // partials per kPackAlign block of the member, or per 128 x 32 tile
    const std::int64_t b0 = tile_partials ? M.rtile_base : M.base / kPackAlign;
    const std::int64_t nb = tile_partials ? static_cast<std::int64_t>(M.nrx) * M.nry
                                          : (static_cast<std::int64_t>(M.nr) * M.nc + kPackAlign - 1) / kPackAlign;
    double s = is_max ? -INFINITY : 0.0;
    for (std::int64_t b = b0 + lane; b < b0 + nb; b += 32)
    {
        const double v = part[q * nblk + b];
        s = is_max ? fmax(s, v) : s + v;
    }
    for (int o = 16; o > 0; o >>= 1)
    {
        const double v = __shfl_down_sync(0xffffffffu, s, o);
        s = is_max ? fmax(s, v) : s + v;
    }
    if (lane == 0) dst[m * stride + off + q] = s;
}

// hs_setup (hillslope.cu) for every member at once: DOF flags, Jacobi
// inverse diagonal, b = -F of the linear law at z = z^n (the time term is
// zero there), in FP32: the face differences z_nb - z_P are formed first,
// so no large term cancels. Block partials of ||b||^2.
__global__ void ens_hs_setup(Packed P, const EnsParams* __restrict__ prm, const std::uint8_t* __restrict__ mask,
                             const float* __restrict__ z, std::uint8_t* __restrict__ dof, float* __restrict__ inv_diag,
                             float* __restrict__ b, double* __restrict__ part,
                             const std::int32_t* __restrict__ blist = nullptr)
{
    LSDTT_COUNT();
    // the block: this one, or (a member group's solve) its list entry
    const std::int64_t blk = blist ? blist[blockIdx.x] : static_cast<std::int64_t>(blockIdx.x);
    const std::int64_t i = blk * blockDim.x + threadIdx.x;
    const int m = P.blk_member[blk];
    const PackedMember& M = P.m[m];
    const EnsParams& q = prm[m];
    const Hs& H = q.hs;
    float bb = 0.0f;
    if (i < P.n)
    {
        const std::int64_t local = i - M.base;
        bool is_dof = false, fast = false;
        if (local < static_cast<std::int64_t>(M.nr) * M.nc && q.hill_on)
        {
            const int l = static_cast<int>(local);
            const int r = l / M.nc, c = l - r * M.nc;
            const std::uint8_t* mk = mask + M.base;
            is_dof = mk[l] && !hs_dirichlet_edge(H, r, c);
            if (is_dof)
            {
                // Fast cell (dof = 3): interior, and all four neighbours
                // in-grid, valid and themselves DOFs (not on a Dirichlet
                // edge), so the stencil needs no boundary rules.
                if (r > 1 && r < M.nr - 2 && c > 1 && c < M.nc - 2 && mk[l - M.nc] && mk[l + 1] && mk[l + M.nc] &&
                    mk[l - 1])
                    fast = true;
                const float* zm = z + M.base;
                const float zp = zm[l];
                float flux = 0.0f;
                int nf = 0;
                if (fast)
                {
                    // the four in-grid neighbours, in the general path's order (N, E, S, W)
                    flux = (((zm[l - M.nc] - zp) + (zm[l + 1] - zp)) + (zm[l + M.nc] - zp)) + (zm[l - 1] - zp);
                    nf = 4;
                }
                else
                {
#pragma unroll
                    for (int f = 0; f < 4; ++f)
                    {
                        const std::int64_t j = hs_nb(H, mk, r, c, kDr[f], kDc[f]);
                        flux += zm[j] - zp;
                        nf += (j != l) ? 1 : 0;
                    }
                }
                const float F = -q.U_f - q.DA_f * flux;
                b[i] = -F;
                inv_diag[i] = q.hs_invd[nf];
                bb = F * F;
            }
        }
        dof[i] = is_dof ? (fast ? 3 : 1) : 0;
        if (!is_dof)
        {
            b[i] = 0.0f;
            inv_diag[i] = 0.0f;
        }
    }
    block_partial_f(bb, false, part, P.n / kPackAlign, 0, blk);
}

// Start from x0 (the previous step's increment; zero at non-DOF cells):
// r = b - A x0 (A x0 in Ax0), p = M^-1 r; block partials of r.z.
__global__ void ens_hs_init(Packed P, const float* __restrict__ b, const float* __restrict__ inv_diag,
                            const std::uint8_t* __restrict__ dof, const float* __restrict__ Ax0,
                            float* __restrict__ x, float* __restrict__ r, float* __restrict__ p,
                            double* __restrict__ part, const std::int32_t* __restrict__ blist = nullptr)
{
    LSDTT_COUNT();
    const std::int64_t blk = blist ? blist[blockIdx.x] : static_cast<std::int64_t>(blockIdx.x);
    const std::int64_t i = blk * blockDim.x + threadIdx.x;
    float rz = 0.0f;
    if (i < P.n)
    {
        const bool d = dof[i] != 0;
        const float ri = d ? b[i] - Ax0[i] : 0.0f;
        const float zi = ri * inv_diag[i];
        if (!d) x[i] = 0.0f;
        r[i] = ri;
        p[i] = zi;
        rz = ri * zi;
    }
    block_partial_f(rz, false, part, P.n / kPackAlign, 0, blk);
}

// done[m] = no hillslope or nothing to solve; iters[m] = 0
__global__ void ens_hs_start(int M, const EnsParams* __restrict__ prm, const double* __restrict__ hs_bb,
                             int* __restrict__ done, int* __restrict__ iters, const std::uint8_t* __restrict__ grp,
                             int g)
{
    LSDTT_COUNT();
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    if (grp && grp[m] != g) return;  // another member group's solve: stays done here
    done[m] = (!prm[m].hill_on || hs_bb[m] == 0.0) ? 1 : 0;
    iters[m] = 0;
}

// done[m] = 1 for the members outside group g (grp = null: every member
// takes part), so the solve's reductions and PCG kernels skip them.
__global__ void ens_group_done(int M, const std::uint8_t* __restrict__ grp, int g, int* __restrict__ done)
{
    LSDTT_COUNT();
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m < M) done[m] = (grp && grp[m] != g) ? 1 : 0;
}

// Ap = A p in the difference form inv_dt p_P + (D/h^2) sum_f (p_P - [nb DOF]
// p_nb) (faces to the cell itself carry no flux), FP32; block partials of
// p.Ap. A converged member's blocks return at once.
// Fused with the CG direction update of the previous iteration: with `fuse`,
// p = z + beta p_src is formed on the fly at the cell and its neighbours
// (beta = r.z / r_old.z_old of this member) and written to
// p_dst, the buffer the update then reads; without it p_dst already holds p.
// beta_m holds each member's beta (ens_pcg_ratio); with it_dev (a
// device-side loop) the direction update is fused whenever *it_dev > 0.
//
// The apply over the members' 128 x 32 tiles (the receiver tiles), one
// 256-thread block per tile: p (formed as z + beta p_src when fused) for the
// tile and a one-cell halo is staged in shared memory by coalesced rows, and
// fast cells (dof 3) read their four neighbours there, in the order of the
// general path's sum (N, E, S, W); other DOF cells take the general path from
// global memory. Each lane handles columns lane, lane + 32, ... of four rows,
// so every load and store of a warp is contiguous. One p.Ap partial per tile.
template <bool kFuse>
__device__ __forceinline__ void hs_apply_tile(float (&sp)[kD8TileRows + 2][132], const PackedMember& M,
                                              const EnsParams& q, int tile, int tx, int ty,
                                              const std::uint8_t* __restrict__ mask,
                                              const std::uint8_t* __restrict__ dof, float beta,
                                              const float* __restrict__ zz, const float* __restrict__ p_src,
                                              float* __restrict__ p_dst, float* __restrict__ Ap,
                                              double* __restrict__ part, std::int64_t nblk)
{
    // sp: column c0 - 1 + k at index k
    const int c0 = tx * kD8TileCols, r0 = ty * kD8TileRows;
    const int nr = M.nr, nc = M.nc;
    const std::int64_t base = M.base;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    auto pv = [&](std::int64_t k) { return kFuse ? zz[k] + beta * p_src[k] : p_dst[k]; };
    for (int lr = w; lr < kD8TileRows + 2; lr += 8)
    {
        const int r = r0 - 1 + lr;
        const bool row_in = r >= 0 && r < nr;
        const std::int64_t rb = base + static_cast<std::int64_t>(r) * nc;
#pragma unroll
        for (int k = 0; k < 5; ++k)
        {
            const int col = 32 * k + lane;  // 0 .. 159: columns c0 - 1 .. c0 + 128 are used
            if (col >= 130) continue;
            const int c = c0 - 1 + col;
            sp[lr][col] = (row_in && c >= 0 && c < nc) ? pv(rb + c) : 0.0f;
        }
    }
    __syncthreads();
    float pap = 0.0f;
#pragma unroll
    for (int qr = 0; qr < 4; ++qr)
    {
        const int lr = 1 + w * 4 + qr, r = r0 + lr - 1;
        if (r >= nr) continue;
        const std::int64_t rb = base + static_cast<std::int64_t>(r) * nc;
#pragma unroll
        for (int k = 0; k < 4; ++k)
        {
            const int lc = 1 + 32 * k + lane, c = c0 + lc - 1;
            if (c >= nc) continue;
            const std::int64_t i = rb + c;
            const std::uint8_t kd = dof[i];
            const float pi = sp[lr][lc];
            if (kFuse) p_dst[i] = pi;
            float v = 0.0f;
            if (kd == 3)
            {
                const float s = (((pi - sp[lr - 1][lc]) + (pi - sp[lr][lc + 1])) + (pi - sp[lr + 1][lc])) +
                                (pi - sp[lr][lc - 1]);
                v = q.inv_dt_f * pi + q.DA_f * s;
            }
            else if (kd)
            {
                const int l = r * nc + c;
                const std::uint8_t* mk = mask + base;
                const std::uint8_t* dm = dof + base;
                float s = 0.0f;
                if (r > 0 && r < nr - 1 && c > 0 && c < nc - 1)
                {
                    // interior: the in-grid neighbour, or the cell itself when masked
                    const int nbr[4] = {l - nc, l + 1, l + nc, l - 1};
#pragma unroll
                    for (int f = 0; f < 4; ++f)
                    {
                        const int j = nbr[f];
                        if (!mk[j]) continue;
                        s += pi - (dm[j] ? pv(base + j) : 0.0f);
                    }
                }
                else
                {
#pragma unroll
                    for (int f = 0; f < 4; ++f)
                    {
                        const std::int64_t j = hs_nb(q.hs, mk, r, c, kDr[f], kDc[f]);
                        if (j == l) continue;
                        s += pi - (dm[j] ? pv(base + j) : 0.0f);
                    }
                }
                v = q.inv_dt_f * pi + q.DA_f * s;
            }
            pap += pi * v;
            Ap[i] = v;
        }
    }
    block_partial_f(pap, false, part, nblk, 0, tile);
}

__global__ void __launch_bounds__(256, 4) ens_hs_apply_tiled(Packed P, const EnsParams* __restrict__ prm,
                                                          const std::uint16_t* __restrict__ rtile_member,
                                                          const std::uint8_t* __restrict__ mask,
                                                          const std::uint8_t* __restrict__ dof,
                                                          const int* __restrict__ done, int fuse,
                                                          const float* __restrict__ beta_m,
                                                          const int* __restrict__ it_dev,
                                                          const float* __restrict__ zz,
                                                          const float* __restrict__ p_src, float* __restrict__ p_dst,
                                                          float* __restrict__ Ap, double* __restrict__ part,
                                                          const std::int32_t* __restrict__ tlist = nullptr)
{
    LSDTT_COUNT();
    // the receiver tile: this block's, or (a member group's solve) the
    // tile its list entry names
    const int tile = tlist ? tlist[blockIdx.x] : static_cast<int>(blockIdx.x);
    const int m = rtile_member[tile];
    if (done[m]) return;
    if (it_dev && *it_dev > 0) fuse = 1;
    const PackedMember& M = P.m[m];
    const EnsParams& q = prm[m];
    const int local = tile - M.rtile_base;
    const std::int64_t nblk = P.n / kPackAlign;
    __shared__ float sp[kD8TileRows + 2][132];
    if (fuse)
        hs_apply_tile<true>(sp, M, q, tile, local % M.nrx, local / M.nrx, mask, dof, beta_m[m], zz, p_src, p_dst, Ap,
                            part, nblk);
    else
        hs_apply_tile<false>(sp, M, q, tile, local % M.nrx, local / M.nrx, mask, dof, 0.0f, zz, p_src, p_dst, Ap,
                             part, nblk);
}

// x += alpha p; r -= alpha Ap; z = M^-1 r (alpha_m: each member's
// r.z / p.Ap, from ens_pcg_ratio); block partials of r.z and r.r.
__global__ void ens_hs_update(Packed P, const int* __restrict__ done, const float* __restrict__ alpha_m,
                              const float* __restrict__ inv_diag, const float* __restrict__ p,
                              const float* __restrict__ Ap, float* __restrict__ x, float* __restrict__ r,
                              float* __restrict__ zz, double* __restrict__ part,
                              const std::int32_t* __restrict__ blist = nullptr)
{
    LSDTT_COUNT();
    const std::int64_t blk = blist ? blist[blockIdx.x] : static_cast<std::int64_t>(blockIdx.x);
    const std::int64_t i = blk * blockDim.x + threadIdx.x;
    const int m = P.blk_member[blk];  // kPackAlign-cell blocks: one member each
    if (done[m]) return;
    const float alpha = alpha_m[m];
    float rz = 0.0f, rr = 0.0f;
    if (i < P.n)
    {
        x[i] += alpha * p[i];
        const float ri = r[i] - alpha * Ap[i];
        r[i] = ri;
        const float zi = ri * inv_diag[i];
        zz[i] = zi;
        rz = ri * zi;
        rr = ri * ri;
    }
    const float rv[2] = {rz, rr};
    block_partials_f<2>(rv, 0u, part, P.n / kPackAlign, blk);
}

// After iteration `it` (0-based, it + 1 a multiple of 4 or the last one):
// the single-grid convergence test per member. flags[5] counts the members
// still iterating; flags[4] marks a member that reached max_iter. With
// it_dev, `it` and the slot `cur` move by *it_dev iterations.
__global__ void ens_hs_check(int M, const EnsParams* __restrict__ prm, int it, const double* __restrict__ cur,
                             const double* __restrict__ hs_bb, int* __restrict__ done, int* __restrict__ iters,
                             int* __restrict__ flags, const int* __restrict__ it_dev = nullptr)
{
    LSDTT_COUNT();
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M || done[m]) return;
    if (it_dev)
    {
        it += *it_dev;
        cur += static_cast<std::int64_t>(*it_dev) * kHsSlot * M;
    }
    const EnsParams& q = prm[m];
    const double rel = sqrt(cur[m * kHsSlot + 2]) / sqrt(hs_bb[m]);
    iters[m] = it + 1;
    if (rel <= q.rel_tol)
        done[m] = 1;
    else if (it + 1 >= q.max_iter)
    {
        done[m] = 1;
        flags[4] = 1;
    }
    else
        atomicAdd(&flags[5], 1);
}

// After the captured iterations: a member still iterating overflows.
__global__ void ens_hs_overflow(int M, const int* __restrict__ done, int* __restrict__ flags)
{
    LSDTT_COUNT();
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m < M && !done[m]) flags[3] = 1;
}

// A PCG scalar per member, out[m] = num / den in double rounded to float
// (0 when den <= 0): alpha = r.z / p.Ap after the apply's reduction, beta =
// r.z / r_old.z_old after the update's. num and den are entries of
// iteration slots of acc (kHsSlot * M doubles each); with it_dev both slots
// move by *it_dev.
__global__ void ens_pcg_ratio(int M, const int* __restrict__ done, const double* __restrict__ acc, int slot_num,
                              int off_num, int slot_den, int off_den, const int* __restrict__ it_dev,
                              float* __restrict__ out)
{
    LSDTT_COUNT();
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M || done[m]) return;
    const std::int64_t sh = it_dev ? *it_dev : 0;
    const std::int64_t slot = static_cast<std::int64_t>(kHsSlot) * M;
    const double num = acc[slot * (slot_num + sh) + m * kHsSlot + off_num];
    const double den = acc[slot * (slot_den + sh) + m * kHsSlot + off_den];
    out[m] = den > 0.0 ? static_cast<float>(num / den) : 0.0f;
}

// Condition of the graph's PCG loop (a conditional WHILE node whose body is
// two iterations and the convergence test): advance the iteration counter,
// go on while a member is still iterating; a member still iterating at
// itmax raises the PCG overflow flag.
__global__ void ens_pcg_while(int* __restrict__ it_dev, int itmax, int* __restrict__ flags,
                              cudaGraphConditionalHandle h)
{
    LSDTT_COUNT();
    const int it = (*it_dev += 2);
    const int active = flags[5];
    flags[5] = 0;
    if (active > 0 && it >= itmax) flags[3] = 1;
    cudaGraphSetConditional(h, (active > 0 && it < itmax) ? 1u : 0u);
}

// ---- uplift, boundary restore, statistics ----------------------------------
__global__ void ens_boundary_flag(Packed P, const std::uint8_t* __restrict__ mask, std::uint8_t* __restrict__ flag)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const PackedMember& M = P.m[block_member(P)];
    const std::int64_t local = i - M.base;
    flag[i] = (local < static_cast<std::int64_t>(M.nr) * M.nc &&
               boundary_flat_cell(M.nr, M.nc, M.bc, mask + M.base, local))
                  ? 1
                  : 0;
}

// The end of a step in one pass: the hillslope increment added in double
// (z = zsp + x on DOFs, zsp elsewhere), uplift on valid cells, the boundary
// restore (z = z_before - bl on flagged cells), then lem_stats (lem.cu) per
// member as block partials (zb = the surface before the step, za = after):
// [0] sum of (after - before), [1] unused, [2] erosion sum, [3] valid count,
// [4..7] maxima (before, after, |dz|, erosion). Differences are formed per
// cell (exact for nearby elevations) before any sum, so FP32 warp sums
// suffice.
__global__ void ens_step_finish(Packed P, const EnsParams* __restrict__ prm, const std::uint8_t* __restrict__ mask,
                                const std::uint8_t* __restrict__ bflag, const std::uint8_t* __restrict__ dof,
                                const float* __restrict__ zsp, const float* __restrict__ x,
                                const float* __restrict__ zb, float* __restrict__ z, double* __restrict__ part)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int m = P.blk_member[blockIdx.x];  // kPackAlign-cell blocks: one member each
    const EnsParams& q = prm[m];
    float v[8] = {0.0f, 0.0f, 0.0f, 0.0f, -1e30f, -1e30f, 0.0f, 0.0f};
    if (i < P.n)
    {
        const float s = zsp[i];
        float a = dof[i] ? static_cast<float>(static_cast<double>(s) + static_cast<double>(x[i])) : s;
        const bool valid = mask[i] != 0;
        if (valid) a = __fadd_rn(a, q.udz);
        if (bflag[i]) a = __fsub_rn(zb[i], q.bl);
        z[i] = a;
        if (valid)
        {
            const float b = zb[i];
            v[0] = a - b;
            v[4] = b;
            v[5] = a;
            v[6] = fabsf(a - b);
            const float ero = (b - a) + q.udz;
            if (ero > 0.0f) { v[2] = ero; v[7] = ero; }
            v[3] = 1.0f;
        }
    }
    block_partials_f<8>(v, 0xf0u, part, P.n / kPackAlign);
}

bool exact_area(double dw, std::int64_t nv)
{
    if (!(dw > 0.0) || !std::isfinite(dw)) return false;
    int e = 0;
    const double fr = std::frexp(dw, &e);
    std::uint64_t m = static_cast<std::uint64_t>(std::ldexp(fr, 53));
    while (m && !(m & 1)) m >>= 1;
    return static_cast<long double>(m) * static_cast<long double>(nv) < 9007199254740992.0L;
}

}  // namespace
}  // namespace lsdtt_gb300

using namespace lsdtt_gb300;

struct lsdtt_gpu_ensemble
{
    int M = 0;
    std::vector<lsdtt_gpu_member> members;
    std::vector<PackedMember> pm;
    std::vector<EnsParams> prm_h;
    std::int64_t N = 0, member_cells = 0;
    std::int32_t T = 0;
    std::int32_t S = 0;      // receiver tiles (128 x 32 cells)
    std::int64_t perim = 0;  // perimeter cells of all members
    PackedMember* d_pm = nullptr;
    EnsParams* d_prm = nullptr;
    std::uint16_t* blk_member = nullptr;
    std::uint16_t* tile_member = nullptr;
    std::uint16_t* strip_member = nullptr;  // [S]: member of each 128 x 32 receiver tile
    unsigned* undecided = nullptr;          // receivers tile pass left undecided cells
    Packed P{};
    // state and stage buffers
    float *z = nullptr, *zf = nullptr, *zsp = nullptr, *zpre = nullptr;
    // The epsilon fill in the reference's order (fill_exact.cuh): the
    // epsilon-0 fill, the member table and the buffers of the replay.
    float* zf0 = nullptr;
    ExMember* d_exm = nullptr;
    char* exbuf = nullptr;
    Scratch exws{};
    ExBuffers exB{};
    int ex_mbits = 0;
    bool ex_any = false;  // some member fills with min_slope > 0
    int ex_on = 0;        // members that fill with min_slope > 0
    int sms = 152;
    std::uint8_t *mask = nullptr, *kind = nullptr, *bflag = nullptr, *dirty = nullptr, *oflag = nullptr;
    std::int32_t* flist = nullptr;           // [kFillColours][T] active fill tiles of the current pass
    unsigned long long* fcnt = nullptr;      // [kFillColours + 1] their counts by colour, then their cells
    unsigned long long* h_fcnt = nullptr;    // pinned copy (eager steps)
    unsigned fill_grid = 0;                  // persistent grid of the listed relaxation
    unsigned fill_colours = 0;               // tile colours some member can hold (fill_colour_mask)
    std::int64_t* pos = nullptr;
    int* nd = nullptr;
    lsdtt_gpu_flow* f = nullptr;
    double* area = nullptr;
    std::uint32_t *order = nullptr, *lstart = nullptr, *lcount = nullptr, *lfill = nullptr, *maxd = nullptr;
    std::uint8_t* dof = nullptr;
    float *invd = nullptr, *b = nullptr, *x = nullptr, *r = nullptr, *p = nullptr, *zz = nullptr, *Ap = nullptr;
    float* p2 = nullptr;  // second CG direction buffer (the fused direction update alternates)
    double *hs_bb = nullptr, *hs_acc = nullptr;
    int *done = nullptr, *iters = nullptr;
    double* stats_acc = nullptr;
    double* part = nullptr;  // block partials [8][packed / 256]
    double* kam_tab = nullptr;  // [n_members][kKamTab]
    int* flags = nullptr;
    // pinned host mirrors
    double* h_stats = nullptr;
    int* h_flags = nullptr;
    int* h_iters = nullptr;
    std::uint32_t* h_maxd = nullptr;
    unsigned long long* h_err = nullptr;
    int max_iter_all = 1000;
    int max_pass_all = 64;
    // schedule
    bool use_graph = true, captured = false, tuned = false;
    int fill_cap = 0, depth_cap = 0, split = 1, sweep_block = 256, it_cap = 0;
    std::vector<unsigned> level_blocks;  // grid of each captured level launch
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t own = nullptr;  // private stream: the legacy default stream cannot be captured
    cudaStream_t own2 = nullptr;  // captures the bodies of the graph's device-side loops
    cudaStream_t own3 = nullptr;  // the deep member group's sweep (captured steps)
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // Member groups of captured steps: the deep group (members deeper than
    // half the deepest, a prefix of perm) sweeps on own3 while the shallow
    // group sweeps and solves its hillslope on the main stream; the deep
    // group's solve follows the join. Block / receiver-tile lists per group.
    int n_deep = 0;
    bool groups_on = false;                 // lsdtt_gpu_ensemble_set_member_groups (off: measured slower
                                            // on the bench ensemble, 62.1 vs 59.9 ms a step)
    std::vector<std::uint32_t> depth_last;  // members' deepest levels of the last eager step
    std::uint16_t* perm_cap = nullptr;      // the member order the captured graph's sweeps use
    std::int32_t* glist = nullptr;   // [blocks of group 0][blocks of group 1][tiles of 0][tiles of 1]
    std::int64_t gcount[4] = {0, 0, 0, 0};
    std::uint8_t* grp = nullptr;     // [M] 1 = deep group
    bool use_while = true;        // device-side loops (conditional WHILE nodes) in the graph
    int* loopc = nullptr;         // [2] their trip counters (fill pass pairs, PCG iterations)
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;  // order the private stream after/before the caller's
    std::uint32_t tail = 0;      // tuned: levels of at most `tail` cells run in one block (0: none)
    int sweep_mode = 0;          // tuned: 0 level launches (+ tail), 1 in-order dataflow, 2 cooperative levels,
                                 // 3 member clusters
    bool forced_mode = false;    // sweep_mode set by the caller, not the autotuner
    int df_grid = 0;             // persistent blocks of the dataflow sweep
    int coop_grid = 0;           // co-resident blocks of the cooperative level sweep
    std::uint32_t* morder = nullptr;  // [N] member-major depth order (member-cluster sweep)
    std::uint32_t* mstart = nullptr;  // [N + 2] its bucket offsets (member base + depth)
    std::uint32_t* mmax = nullptr;    // [M] deepest level of each member
    std::uint16_t* perm = nullptr;    // [M] members by decreasing cell count
    float* pcg_scal = nullptr;        // [2M] each member's PCG alpha, then beta
    std::vector<std::uint16_t> perm_h;
    int sweep_cluster = 8;            // CTAs per member cluster (tuned: 4, 8 or 16)
    unsigned* bar = nullptr;     // its grid barrier: {count, generation}
    unsigned long long* zg = nullptr;  // dataflow {generation, z} word per cell
    std::uint32_t* dfc = nullptr;    // [0] generation, [1] chunk counter
    int ov_fill = 0, ov_it = 0;  // one-shot schedule override for the next capture
    lsdtt_gpu_ensemble_info info{};
    bool ready = false;  // every member set at least once
    std::vector<char> member_set;
};

namespace
{

struct StepRecord
{
    int fill_passes = 0;
    int max_depth = 0;
    int pcg_iters = 0;
    std::vector<std::uint32_t> level_size;  // [max_depth + 1]
};

void free_ensemble(lsdtt_gpu_ensemble* E)
{
    if (E->exec) cudaGraphExecDestroy(E->exec);
    if (E->graph) cudaGraphDestroy(E->graph);
    void* bufs[] = {E->d_pm, E->d_prm, E->blk_member, E->tile_member, E->strip_member, E->undecided, E->bar, E->loopc, E->pcg_scal, E->morder, E->mstart, E->mmax, E->perm, E->z, E->zf, E->zsp, E->zpre, E->kind, E->bflag, E->dirty, E->oflag, E->pos, E->nd, E->area, E->order, E->lstart, E->lcount,
                    E->lfill, E->maxd, E->dof, E->invd, E->b, E->x, E->r, E->p, E->p2, E->zz, E->Ap, E->hs_bb, E->hs_acc,
                    E->done, E->iters, E->stats_acc, E->part, E->kam_tab, E->flags, E->zg, E->dfc, E->flist, E->fcnt, E->glist, E->grp, E->perm_cap, E->zf0, E->d_exm, E->exbuf};
    for (void* q : bufs) cudaFree(q);
    void* hb[] = {E->h_stats, E->h_flags, E->h_iters, E->h_maxd, E->h_err, E->h_fcnt};
    for (void* q : hb) cudaFreeHost(q);
    if (E->f) lsdtt_gpu_flow_destroy(E->f);
    if (E->own) cudaStreamDestroy(E->own);
    if (E->own2) cudaStreamDestroy(E->own2);
    if (E->own3) cudaStreamDestroy(E->own3);
    if (E->ev_fork) cudaEventDestroy(E->ev_fork);
    if (E->ev_join) cudaEventDestroy(E->ev_join);
    if (E->ev_in) cudaEventDestroy(E->ev_in);
    if (E->ev_out) cudaEventDestroy(E->ev_out);
    delete E;
}

// Member groups of a captured graph, set right before the capture from the
// last eager step's member order (perm_h, deepest first) and depths: the
// deep group is the prefix of that order deeper than 3/4 of the deepest
// member; its sweep runs beside the shallow group's sweep and hillslope
// solve. The graph keeps its own copy of the order (perm_cap), so eager
// steps that re-sort perm (a profiled step) leave the graph's groups, lists
// and order consistent. Any grouping gives the same result (each group's
// sweep precedes its own solve); only the overlap depends on it. No groups
// when the deepest member is shallow (the sweep is short) or one group
// would be empty.
constexpr std::uint32_t kSplitMinDepth = 64;

cudaError_t set_member_groups(lsdtt_gpu_ensemble* E, const std::vector<std::uint32_t>& depth_h, cudaStream_t st)
{
    const int M = E->M;
    if (depth_h.size() != static_cast<std::size_t>(M))
    {
        E->n_deep = 0;
        return cudaSuccess;
    }
    const std::uint32_t dmax = depth_h[E->perm_h[0]];
    int nd = 0;
    while (nd < M && 4ull * depth_h[E->perm_h[static_cast<std::size_t>(nd)]] > 3ull * dmax) ++nd;
    E->n_deep = (nd > 0 && nd < M && dmax >= kSplitMinDepth) ? nd : 0;
    std::vector<std::uint8_t> g(static_cast<std::size_t>(M), 0);
    for (int k = 0; k < E->n_deep; ++k) g[E->perm_h[static_cast<std::size_t>(k)]] = 1;
    std::vector<std::int32_t> lists[4];
    for (int m = 0; m < M; ++m)
    {
        const PackedMember& Pm = E->pm[static_cast<std::size_t>(m)];
        const std::int64_t b0 = Pm.base / kPackAlign;
        const std::int64_t nbm = (static_cast<std::int64_t>(Pm.nr) * Pm.nc + kPackAlign - 1) / kPackAlign;
        const int gm = g[static_cast<std::size_t>(m)];
        for (std::int64_t b = b0; b < b0 + nbm; ++b) lists[gm].push_back(static_cast<std::int32_t>(b));
        for (std::int32_t t = Pm.rtile_base; t < Pm.rtile_base + Pm.nrx * Pm.nry; ++t) lists[2 + gm].push_back(t);
    }
    std::vector<std::int32_t> all;
    for (int k = 0; k < 4; ++k)
    {
        E->gcount[k] = static_cast<std::int64_t>(lists[k].size());
        all.insert(all.end(), lists[k].begin(), lists[k].end());
    }
    cudaMemcpyAsync(E->glist, all.data(), sizeof(std::int32_t) * all.size(), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(E->grp, g.data(), static_cast<std::size_t>(M), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(E->perm_cap, E->perm_h.data(), sizeof(std::uint16_t) * M, cudaMemcpyHostToDevice, st);
    return cudaStreamSynchronize(st);
}

// Sweep launches for levels 1 .. split-1 (one launch each), then the tail.
cudaError_t enqueue_sweep(lsdtt_gpu_ensemble* E, const SweepArgs& A, int split, int block,
                          const std::vector<unsigned>& blocks, cudaStream_t st, int mode, int perm_off = 0,
                          int perm_count = -1, const std::uint16_t* perm = nullptr)
{
    if (!perm) perm = E->perm;
    if (mode == 3)
    {
        // member clusters for perm[perm_off .. perm_off + perm_count)
        if (perm_count < 0) perm_count = E->M - perm_off;
        if (perm_count == 0) return cudaSuccess;
        SweepArgs B = A;
        B.order = E->morder;
        B.start = E->mstart;
        cudaLaunchConfig_t cfg{};
        const unsigned cl = static_cast<unsigned>(E->sweep_cluster);
        cfg.gridDim = dim3(static_cast<unsigned>(perm_count) * cl);
        cfg.blockDim = dim3(static_cast<unsigned>(std::min(block, static_cast<int>(kSweepClusterBlock))));
        cfg.stream = st;
        cudaLaunchAttribute attr{};
        attr.id = cudaLaunchAttributeClusterDimension;
        attr.val.clusterDim.x = cl;
        attr.val.clusterDim.y = 1;
        attr.val.clusterDim.z = 1;
        cfg.attrs = &attr;
        cfg.numAttrs = 1;
        return cudaLaunchKernelEx(&cfg, ens_sp_clusters, B, static_cast<const std::uint16_t*>(perm + perm_off),
                                  static_cast<const std::uint32_t*>(E->mmax));
    }
    if (mode == 2)
    {
        cudaMemsetAsync(E->bar, 0, sizeof(unsigned) * 2, st);
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3(static_cast<unsigned>(E->coop_grid));
        cfg.blockDim = dim3(512);
        cfg.stream = st;
        cudaLaunchAttribute attr{};
        attr.id = cudaLaunchAttributeCooperative;
        attr.val.cooperative = 1;
        cfg.attrs = &attr;
        cfg.numAttrs = 1;
        return cudaLaunchKernelEx(&cfg, ens_sp_coop, A, split, E->bar, E->flags + 7);
    }
    if (mode == 1)
    {
        ens_gen_bump<<<1, 1, 0, st>>>(E->dfc);
        ens_mark_roots<<<152 * 4, 256, 0, st>>>(A, E->dfc, E->zg);
        cudaMemsetAsync(E->dfc + 1, 0, sizeof(std::uint32_t), st);
        ens_sp_dataflow<<<E->df_grid, 256, 0, st>>>(A, E->dfc, E->dfc + 1, E->zg, E->flags + 7);
        ens_sp_extract<<<grid_blocks(E->N, 256), 256, 0, st>>>(E->N, E->dfc, E->zg, A.z);
        return cudaSuccess;
    }
    for (int k = 1; k < split; ++k)
        ens_sp_level<<<blocks[static_cast<std::size_t>(k)], block, 0, st>>>(A, k);
    ens_sp_tail<<<1, 1024, 0, st>>>(A, split);
    return cudaSuccess;
}

// Blocks of each level launch for a level-size profile.
std::vector<unsigned> level_grid(const std::vector<std::uint32_t>& size, int split, int block, double margin)
{
    std::vector<unsigned> g(static_cast<std::size_t>(std::max(split, 1)), 1u);
    for (int k = 1; k < split; ++k)
    {
        const double s = k < static_cast<int>(size.size()) ? size[static_cast<std::size_t>(k)] : 0.0;
        const double want = std::ceil(s * margin / block) + 1.0;
        g[static_cast<std::size_t>(k)] = static_cast<unsigned>(std::min(want, 152.0 * 16.0));
    }
    return g;
}

// First level from which every level holds at most `tail` cells.
int split_for(const std::vector<std::uint32_t>& size, std::uint32_t tail)
{
    int k = static_cast<int>(size.size());
    while (k > 1 && size[static_cast<std::size_t>(k - 1)] <= tail) --k;
    return std::max(k, 1);
}

// One step. eager: host-driven loops (records the schedule in *rec and
// autotunes the sweep on the first call); otherwise the captured schedule.
// Appends a conditional WHILE node to the graph being captured on st (after
// the work captured so far) and captures body(st2, handle) as its body; the
// body's last kernel sets the condition with cudaGraphSetConditional. Work
// captured on st afterwards depends on the node.
template <class Body>
cudaError_t capture_while(cudaStream_t st, cudaStream_t st2, const Body& body)
{
    cudaStreamCaptureStatus status = cudaStreamCaptureStatusNone;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    std::size_t ndeps = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(st, &status, nullptr, &g, &deps, nullptr, &ndeps);
    if (e != cudaSuccess) return e;
    if (status != cudaStreamCaptureStatusActive) return cudaErrorStreamCaptureInvalidated;
    cudaGraphConditionalHandle h = 0;
    e = cudaGraphConditionalHandleCreate(&h, g, 1u, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) return e;
    cudaGraphNodeParams np{};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    e = cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &np);
    if (e != cudaSuccess) return e;
    e = cudaStreamBeginCaptureToGraph(st2, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                      cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    body(st2, h);
    cudaGraph_t done = nullptr;
    e = cudaStreamEndCapture(st2, &done);
    if (e != cudaSuccess) return e;
    return cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
}

cudaError_t run_step(lsdtt_gpu_ensemble* E, cudaStream_t st, bool eager, StepRecord* rec)
{
    const std::int64_t N = E->N;
    const unsigned nb = grid_blocks(N, 256);
    const int M = E->M;
    const unsigned mb = static_cast<unsigned>((M + 127) / 128);
    cudaError_t e = cudaSuccess;
    cudaMemcpyAsync(E->zpre, E->z, sizeof(float) * N, cudaMemcpyDeviceToDevice, st);
    cudaMemsetAsync(E->flags, 0, sizeof(int) * kFlags, st);
    // 0. fill: the value-ordered relaxation (the fill itself where min_slope
    // is 0; the estimate otherwise), then, for members with min_slope > 0,
    // the epsilon-0 relaxation and the fill in the reference's order
    cudaMemsetAsync(E->nd, 0, sizeof(int) * M, st);
    LSDTT_TIMED("ens_interior", 0.0, st, (ens_interior<<<nb, 256, 0, st>>>(E->P, E->d_prm, E->z, E->mask, E->nd)));
    const dim3 fblock(32, 8);
    const double cells = static_cast<double>(E->member_cells);
    const unsigned tb = static_cast<unsigned>((E->T + 255) / 256);
    auto relax_all = [&](float* F, int eps0, const char* name) -> cudaError_t {
        LSDTT_TIMED("ens_fill_init", 0.0, st,
                    (ens_fill_init<<<nb, 256, 0, st>>>(E->P, E->d_prm, E->z, E->mask, E->nd, F, E->kind)));
        LSDTT_TIMED("ens_dirty_init", 0.0, st,
                    (ens_dirty_init<<<grid_blocks(E->T, 256), 256, 0, st>>>(E->T, E->tile_member, E->d_prm, E->dirty,
                                                                            E->dirty + E->T)));
        // One pass: list the active tiles, then relax only those. In eager
        // steps the listed cells are read back, so the pass's algorithmic
        // bytes (z 4 + mask 1 in, filled value 4 out per cell of an active
        // tile) are those of the work done.
        auto pass_on = [&](int pass, cudaStream_t s, bool timed) -> cudaError_t {
            const std::uint8_t* din = E->dirty + (pass & 1) * E->T;
            std::uint8_t* dout = E->dirty + ((pass + 1) & 1) * E->T;
            cudaMemsetAsync(E->fcnt, 0, sizeof(unsigned long long) * (kFillColours + 1), s);
            if (timed)
                LSDTT_TIMED("ens_fill_active", 0.0, s,
                            (ens_fill_active<<<tb, 256, 0, s>>>(E->P, E->d_prm, E->tile_member, E->T, din, dout,
                                                                E->flist, E->fcnt)));
            else
                ens_fill_active<<<tb, 256, 0, s>>>(E->P, E->d_prm, E->tile_member, E->T, din, dout, E->flist,
                                                   E->fcnt);
            double bytes = 9.0 * cells;
            if (timed && profiling_enabled())
            {
                cudaMemcpyAsync(E->h_fcnt, E->fcnt, sizeof(unsigned long long) * (kFillColours + 1),
                                cudaMemcpyDeviceToHost, s);
                const cudaError_t pe = cudaStreamSynchronize(s);
                if (pe != cudaSuccess) return pe;
                bytes = 9.0 * static_cast<double>(E->h_fcnt[kFillColours]);
            }
            // the colours in turn: a tile reads its neighbours settled
            LSDTT_TIMED(name, bytes, s, ({
                            for (int c = 0; c < kFillColours; ++c)
                            {
                                if (!((E->fill_colours >> c) & 1u)) continue;
                                ens_fill_relax_list<<<E->fill_grid, fblock, 0, s>>>(
                                    E->P, E->d_prm, E->tile_member, E->z, E->kind, F, E->flags, din, dout,
                                    E->flist + static_cast<std::int64_t>(c) * E->T, E->fcnt + c, eps0);
                            }
                        }));
            return cudaSuccess;
        };
        cudaError_t re = cudaSuccess;
        int passes = 0;
        if (eager)
        {
            for (;;)
            {
                cudaMemsetAsync(E->flags, 0, sizeof(int), st);
                for (int k = 0; k < 4 && re == cudaSuccess; ++k, ++passes) re = pass_on(passes, st, true);
                if (re != cudaSuccess) return re;
                cudaMemcpyAsync(E->h_flags, E->flags, sizeof(int), cudaMemcpyDeviceToHost, st);
                re = cudaStreamSynchronize(st);
                if (re != cudaSuccess) return re;
                if (E->h_flags[0] == 0) break;
                if (passes > E->max_pass_all) return cudaErrorLaunchTimeout;
            }
            rec->fill_passes = std::max(rec->fill_passes, passes);
        }
        else if (E->use_while)
        {
            // Device-side loop: pairs of passes until the second of a pair
            // changes nothing (a fixed point), at most max_pass_all passes.
            cudaMemsetAsync(E->loopc, 0, sizeof(int), st);
            const int max_pairs = (E->max_pass_all + 1) / 2;
            re = capture_while(st, E->own2, [&](cudaStream_t s2, cudaGraphConditionalHandle h) {
                for (int k = 0; k < 2; ++k)
                {
                    if (k == 1) cudaMemsetAsync(E->flags, 0, sizeof(int), s2);
                    pass_on(k, s2, false);
                }
                ens_fill_while<<<1, 1, 0, s2>>>(E->flags, E->loopc, max_pairs, E->flags + 1, h);
            });
        }
        else
        {
            for (int k = 0; k < E->fill_cap; ++k)
            {
                if (k == E->fill_cap - 1) cudaMemsetAsync(E->flags, 0, sizeof(int), st);
                pass_on(k, st, false);
            }
            ens_flag_copy<<<1, 1, 0, st>>>(E->flags, E->flags + 1);
        }
        return re;
    };
    if (eager) rec->fill_passes = 0;
    e = relax_all(E->zf, 0, "ens_fill_relax");
    if (e != cudaSuccess) return e;
    if (E->ex_any)
    {
        e = relax_all(E->zf0, 1, "ens_fill_relax_eps0");
        if (e != cudaSuccess) return e;
        // (each stage is timed inside, as ens_fill_exact_*)
        e = ex_run(E->d_exm, E->blk_member, N, M, E->ex_mbits, E->z, E->kind, E->zf0, E->zf, E->exB, E->exws, E->sms,
                   st, true, E->ex_on);
        if (e != cudaSuccess) return e;
        ens_flag_copy_u<<<1, 1, 0, st>>>(E->exB.u + 5, E->flags + 8);
    }
    // 1. D8 receivers, outlets, s-vector (contributing counts, depth)
    lsdtt_gpu_flow* f = E->f;
    cudaMemsetAsync(f->derr, 0, sizeof(unsigned long long) * 4, st);
    // Algorithmic bytes: z 4 + mask 1 in, direction 1 + int64 receiver 8 out.
    cudaMemsetAsync(E->undecided, 0, sizeof(unsigned), st);
    LSDTT_TIMED("ens_d8_receivers", 14.0 * cells, st,
                (ens_receivers<<<E->S, 256, 0, st>>>(E->P, E->d_prm, E->strip_member, E->zf, E->mask, f->receiver,
                                                     f->dir, E->undecided)));
    // one thread per perimeter cell (each looks its member up by a binary search)
    LSDTT_TIMED("ens_d8_receivers_fixup", 0.0, st,
                (ens_receivers_fixup<<<static_cast<unsigned>(std::max<std::int64_t>((E->perim + 255) / 256, 152 * 4)),
                                       256, 0, st>>>(E->P, E->d_prm, E->perim, E->zf, E->mask, f->receiver, f->dir,
                                                     f->derr, E->undecided)));
    LSDTT_TIMED("ens_outlet_flag", 0.0, st, (ens_outlet_flag<<<nb, 256, 0, st>>>(N, E->mask, f->dir, E->oflag)));
    f->ws.used = 0;
    LSDTT_TIMED("ens_outlet_scan", 0.0, st,
                (e = exclusive_scan<std::uint8_t, std::int64_t>(E->oflag, N, E->pos, f->dscal + 1, f->ws, st)));
    if (e != cudaSuccess) return e;
    LSDTT_TIMED("ens_outlet_scatter", 0.0, st, (ens_scatter<<<nb, 256, 0, st>>>(E->oflag, E->pos, N, f->outlets)));
    f->ws.used = 0;
    // The s-vector stage (Euler tour, ruling-set list ranking): contributing
    // counts and depths; timed as a whole (its ruler walk also on its own).
    // Algorithmic bytes per cell: direction 1 + donor 1 in, int64 count 8
    // out (10).
    LSDTT_TIMED("ens_stack_counts", 10.0 * cells, st, (e = build_stack(f, false, st, &E->P)));
    if (e != cudaSuccess) return e;
    cudaMemsetAsync(E->dfc + 1, 0, sizeof(std::uint32_t), st);  // count of large-count nodes
    LSDTT_TIMED("ens_kam", 0.0, st,
                (ens_kam<<<nb, 256, 0, st>>>(E->P, E->d_prm, E->mask, f->dir, f->sv_size, E->kam_tab, E->area,
                                             E->lfill, E->dfc + 1)));
    LSDTT_TIMED("ens_kam_big", 0.0, st,
                (ens_kam_big<<<152 * 8, 256, 0, st>>>(E->P, E->d_prm, f->sv_size, E->lfill, E->dfc + 1, E->area)));
    // 2. depth levels: the global level order (level launches, the
    // cooperative and dataflow sweeps, and every eager step's record) and
    // the member-major order (member-cluster sweep, and the autotuner)
    const bool global_order = eager || E->sweep_mode != 3;
    const bool member_order = E->sweep_mode == 3 || (eager && !E->tuned);
    if (global_order)
    {
        const std::uint32_t cap =
            eager ? static_cast<std::uint32_t>(N + 1) : static_cast<std::uint32_t>(E->depth_cap);
        cudaMemsetAsync(E->maxd, 0, sizeof(std::uint32_t), st);
        cudaMemsetAsync(E->lcount, 0, sizeof(std::uint32_t) * (static_cast<std::size_t>(cap) + 2), st);
        LSDTT_TIMED("ens_depth_hist", 0.0, st,
                    (ens_depth_hist<<<nb, 256, 0, st>>>(N, E->mask, f->depth, cap, E->lcount, E->maxd, E->flags + 2)));
        std::uint32_t scan_len = cap + 1;
        if (eager)
        {
            cudaMemcpyAsync(E->h_maxd, E->maxd, sizeof(std::uint32_t), cudaMemcpyDeviceToHost, st);
            e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) return e;
            scan_len = *E->h_maxd + 2;
        }
        f->ws.used = 0;
        e = exclusive_scan<std::uint32_t, std::uint32_t>(E->lcount, scan_len, E->lstart,
                                                         static_cast<std::uint32_t*>(nullptr), f->ws, st);
        if (e != cudaSuccess) return e;
        cudaMemsetAsync(E->lfill, 0, sizeof(std::uint32_t) * scan_len, st);
        LSDTT_TIMED("ens_depth_scatter", 0.0, st,
                    (ens_depth_scatter<<<nb, 256, 0, st>>>(N, E->mask, f->depth, cap, E->lstart, E->lfill, E->order)));
    }
    if (member_order)
    {
        // one CTA per member while the depth histogram fits shared memory
        // (eager steps know the deepest level; captured steps use the cap)
        const std::uint32_t mcap =
            eager ? *E->h_maxd + 1 : static_cast<std::uint32_t>(std::min<std::int64_t>(E->depth_cap, N + 1));
        const std::size_t md_smem = sizeof(std::uint32_t) * (static_cast<std::size_t>(mcap) + 1);
        if (md_smem <= kMdSortMaxSmem)
        {
            LSDTT_TIMED("ens_member_depth_sort", 9.0 * static_cast<double>(N), st,
                        (ens_mdepth_sort<<<static_cast<unsigned>(M), kMdSortThreads, md_smem, st>>>(
                            E->P, E->mask, f->depth, mcap, E->mstart, E->morder, E->mmax, E->flags + 2)));
        }
        else
        {
            cudaMemsetAsync(E->mmax, 0, sizeof(std::uint32_t) * M, st);
            cudaMemsetAsync(E->lcount, 0, sizeof(std::uint32_t) * (static_cast<std::size_t>(N) + 1), st);
            ens_mdepth_hist<<<nb, 256, 0, st>>>(E->P, E->mask, f->depth, E->lcount, E->mmax);
            f->ws.used = 0;
            e = exclusive_scan<std::uint32_t, std::uint32_t>(E->lcount, N + 1, E->mstart,
                                                             static_cast<std::uint32_t*>(nullptr), f->ws, st);
            if (e != cudaSuccess) return e;
            cudaMemsetAsync(E->lfill, 0, sizeof(std::uint32_t) * (static_cast<std::size_t>(N) + 1), st);
            ens_mdepth_scatter<<<nb, 256, 0, st>>>(E->P, E->mask, f->depth, E->mstart, E->lfill, E->morder);
        }
        if (!global_order) ens_mdepth_max<<<1, 256, 0, st>>>(M, E->mmax, E->maxd);
        if (eager)
        {
            // Clusters start in member order: deepest members first (the
            // sweep's critical path is a member's depth), then larger ones.
            std::vector<std::uint32_t> depth_h(static_cast<std::size_t>(M));
            cudaMemcpyAsync(depth_h.data(), E->mmax, sizeof(std::uint32_t) * M, cudaMemcpyDeviceToHost, st);
            e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) return e;
            std::stable_sort(E->perm_h.begin(), E->perm_h.end(), [&](std::uint16_t a, std::uint16_t b) {
                if (depth_h[a] != depth_h[b]) return depth_h[a] > depth_h[b];
                const PackedMember &A = E->pm[a], &B = E->pm[b];
                return static_cast<std::int64_t>(A.nr) * A.nc > static_cast<std::int64_t>(B.nr) * B.nc;
            });
            cudaMemcpyAsync(E->perm, E->perm_h.data(), sizeof(std::uint16_t) * M, cudaMemcpyHostToDevice, st);
            e = cudaStreamSynchronize(st);  // perm_h is updated again by the next eager step
            if (e != cudaSuccess) return e;
            E->depth_last = depth_h;  // member groups are set at the next capture
        }
    }
    // 3. stream power, swept by depth level
    LSDTT_TIMED("ens_copy", 0.0, st, (ens_copy<<<nb, 256, 0, st>>>(E->zf, E->zsp, N)));
    SweepArgs A{E->P, E->d_prm, E->order, E->lstart, E->maxd, f->receiver, f->dir, E->area, E->zf, E->zsp};
    if (eager)
    {
        const std::uint32_t D = *E->h_maxd;
        std::vector<std::uint32_t> start(static_cast<std::size_t>(D) + 2);
        cudaMemcpyAsync(start.data(), E->lstart, sizeof(std::uint32_t) * (D + 2), cudaMemcpyDeviceToHost, st);
        e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return e;
        rec->max_depth = static_cast<int>(D);
        rec->level_size.assign(static_cast<std::size_t>(D) + 1, 0u);
        for (std::uint32_t k = 0; k <= D; ++k) rec->level_size[k] = start[k + 1] - start[k];
        if (!E->tuned)
        {
            // Autotune the levels-per-block split and the level block size:
            // time each candidate schedule on this step's levels.
            const std::uint32_t tails[] = {0u, 256u, 1024u, 4096u, 16384u};
            const int blocks[] = {128, 256, 512};
            cudaEvent_t t0, t1;
            cudaEventCreate(&t0);
            cudaEventCreate(&t1);
            double best = 1e30, one_per_level = 0.0;
            int best_cluster = 0;
            std::uint32_t best_tail = 0;
            int best_block = 256;
            int best_mode = 0;
            // candidate schedules {tail threshold, block, mode}: level
            // launches with each tail threshold and block size, the
            // cooperative level sweep with each tail threshold, then the
            // dataflow sweep
            struct Cand
            {
                std::uint32_t tail;
                int blk, mode, cluster;
            };
            std::vector<Cand> cands;
            for (std::uint32_t tail : tails)
                for (int blk : blocks) cands.push_back({tail, blk, 0, 0});
            for (std::uint32_t tail : tails) cands.push_back({tail, 512, 2, 0});
            cands.push_back({0u, 256, 1, 0});
            // clusters of 16 CTAs are the non-portable size (allowed at
            // creation; a launch the device refuses is no candidate)
            for (int cl : {4, 8, 16})
                for (int blk : {64, 128, 256}) cands.push_back({0u, blk, 3, cl});
            for (const auto& cand : cands)
                {
                    const std::uint32_t tail = cand.tail;
                    const int blk = cand.blk;
                    const int mode = cand.mode;
                    if (mode == 3) E->sweep_cluster = cand.cluster;
                    const int sp = (tail == 0 || mode == 1) ? static_cast<int>(D) + 1
                                                            : split_for(rec->level_size, tail);
                    const auto g = level_grid(rec->level_size, sp, blk, 1.0);
                    float ms_best = 1e30f;
                    for (int rep = 0; rep < 2; ++rep)
                    {
                        ens_copy<<<nb, 256, 0, st>>>(E->zf, E->zsp, N);
                        cudaEventRecord(t0, st);
                        if (enqueue_sweep(E, A, sp, blk, g, st, mode) != cudaSuccess)
                        {
                            cudaGetLastError();  // a launch refused (not a fault): not a candidate
                            ms_best = 1e30f;
                            cudaEventRecord(t1, st);
                            cudaEventSynchronize(t1);
                            break;
                        }
                        cudaEventRecord(t1, st);
                        e = cudaEventSynchronize(t1);
                        if (e != cudaSuccess) break;
                        float ms = 0.0f;
                        cudaEventElapsedTime(&ms, t0, t1);
                        ms_best = std::min(ms_best, ms);
                    }
                    if (e != cudaSuccess) break;
                    if (mode == 0 && tail == 0 && blk == 256) one_per_level = ms_best;
                    if (mode == 1) E->info.dataflow_sweep_ms = ms_best;
                    if (mode == 3)
                        E->info.cluster_sweep_ms = E->info.cluster_sweep_ms > 0.0
                                                       ? std::min<double>(E->info.cluster_sweep_ms, ms_best)
                                                       : ms_best;
                    if (mode == 2)
                        E->info.coop_sweep_ms =
                            E->info.coop_sweep_ms > 0.0 ? std::min<double>(E->info.coop_sweep_ms, ms_best) : ms_best;
                    // a run that hit its wait limit is not a candidate
                    if (mode != 0)
                    {
                        int ab = 0;
                        cudaMemcpy(&ab, E->flags + 7, sizeof(int), cudaMemcpyDeviceToHost);
                        if (ab) { cudaMemset(E->flags + 7, 0, sizeof(int)); continue; }
                    }
                    if (ms_best < best)
                    {
                        best = ms_best;
                        best_tail = mode == 1 ? 0u : tail;
                        best_block = blk;
                        best_mode = mode;
                        best_cluster = cand.cluster;
                    }
                }
            cudaEventDestroy(t0);
            cudaEventDestroy(t1);
            if (e != cudaSuccess) return e;
            // Keep the tail threshold, not the level index: the split is
            // recomputed from each recorded profile.
            E->tail = best_tail;
            E->sweep_block = best_block;
            if (best_cluster > 0) E->sweep_cluster = best_cluster;
            if (!E->forced_mode) E->sweep_mode = best_mode;
            E->info.tuned_sweep_ms = best;
            E->info.untuned_sweep_ms = one_per_level;
            E->tuned = true;
            ens_copy<<<nb, 256, 0, st>>>(E->zf, E->zsp, N);
        }
        const int sp = E->tail == 0 ? static_cast<int>(D) + 1 : split_for(rec->level_size, E->tail);
        E->split = sp;
        // Algorithmic bytes per cell: z_old 4 + direction 1 + count 8 +
        // receiver z 4 in, z 4 out (21).
        static const char* const kSweepName[4] = {"ens_sp_levels", "ens_sp_dataflow", "ens_sp_coop", "ens_sp_clusters"};
        LSDTT_TIMED(kSweepName[E->sweep_mode & 3], 21.0 * cells, st,
                    (e = enqueue_sweep(E, A, sp, E->sweep_block, level_grid(rec->level_size, sp, E->sweep_block, 1.0),
                                       st, E->sweep_mode)));
        if (e != cudaSuccess) return e;
    }
    const bool split_groups = !eager && E->sweep_mode == 3 && E->n_deep > 0 && E->n_deep < M;
    if (!eager && split_groups)
    {
        // the deep group's clusters on own3, the shallow group's here
        cudaEventRecord(E->ev_fork, st);
        cudaStreamWaitEvent(E->own3, E->ev_fork, 0);
        e = enqueue_sweep(E, A, E->split, E->sweep_block, E->level_blocks, E->own3, 3, 0, E->n_deep, E->perm_cap);
        cudaEventRecord(E->ev_join, E->own3);
        if (e != cudaSuccess) return e;
        e = enqueue_sweep(E, A, E->split, E->sweep_block, E->level_blocks, st, 3, E->n_deep, M - E->n_deep,
                          E->perm_cap);
        if (e != cudaSuccess) return e;
    }
    else if (!eager)
    {
        e = enqueue_sweep(E, A, E->split, E->sweep_block, E->level_blocks, st, E->sweep_mode);
        if (e != cudaSuccess) return e;
    }
    // 4. hillslope: Jacobi-PCG per member, for every member at once or for
    // one member group (block / receiver-tile lists; the others stay done)
    const std::size_t slot_bytes = sizeof(double) * kHsSlot * M;
    const std::int64_t slot_len = static_cast<std::int64_t>(kHsSlot) * M;
    const bool device_loop = !eager && E->use_while;
    const int itmax = (eager || device_loop) ? E->max_iter_all : E->it_cap;
    const std::int64_t nblk = N / kPackAlign;
    auto reduce = [&](cudaStream_t s2, int nq, unsigned max_mask, const int* dn, double* dst, int stride, int off,
                      const int* shift, int tile_partials = 0) {
        const unsigned warps = static_cast<unsigned>(M * nq);
        LSDTT_TIMED("ens_member_reduce", 0.0, s2,
                    (ens_member_reduce<<<(warps + 3) / 4, 128, 0, s2>>>(E->P, nq, max_mask, E->part, nblk, dn, dst,
                                                                        stride, off, shift, slot_len, tile_partials)));
    };
    struct HsGroup
    {
        const std::int32_t* blist;  // null: every block
        unsigned nblk;
        const std::int32_t* tlist;  // null: every receiver tile
        unsigned ntile;
        const std::uint8_t* grp;    // null: every member
        int g;
    };
    auto hillslope_stage = [&](cudaStream_t hs, const HsGroup& G) -> cudaError_t {
        cudaMemsetAsync(E->hs_acc, 0, slot_bytes * (static_cast<std::size_t>(itmax) + 1), hs);
        ens_group_done<<<mb, 128, 0, hs>>>(M, G.grp, G.g, E->done);
        LSDTT_TIMED("ens_hs_setup", 0.0, hs,
                    (ens_hs_setup<<<G.nblk, 256, 0, hs>>>(E->P, E->d_prm, E->mask, E->zsp, E->dof, E->invd, E->b,
                                                          E->part, G.blist)));
        reduce(hs, 1, 0u, E->done, E->hs_bb, 1, 0, nullptr);
        // Warm start: the previous step's increment x (zero at the first step)
        // as the initial guess; A x0 by one plain apply (p_dst = x).
        LSDTT_TIMED("ens_hs_warm_apply", 0.0, hs,
                    (ens_hs_apply_tiled<<<G.ntile, 256, 0, hs>>>(E->P, E->d_prm, E->strip_member, E->mask, E->dof,
                                                                 E->done, 0, E->pcg_scal, nullptr, E->zz, E->p2, E->x,
                                                                 E->Ap, E->part, G.tlist)));
        LSDTT_TIMED("ens_hs_init", 0.0, hs,
                    (ens_hs_init<<<G.nblk, 256, 0, hs>>>(E->P, E->b, E->invd, E->dof, E->Ap, E->x, E->r, E->p, E->part,
                                                         G.blist)));
        reduce(hs, 1, 0u, E->done, E->hs_acc, kHsSlot, 1, nullptr);
        ens_hs_start<<<mb, 128, 0, hs>>>(M, E->d_prm, E->hs_bb, E->done, E->iters, G.grp, G.g);
        // One iteration whose slots are it / it + 1 (it_dev: plus the device-side
        // counter); p_it lives in pbuf[it % 2] and every iteration but the first
        // forms it inside the apply.
        auto iteration = [&](cudaStream_t s2, int it, const int* it_dev, bool timed) {
            float* p_it = (it & 1) ? E->p2 : E->p;
            const float* p_prev = (it & 1) ? E->p : E->p2;
            double* cur = E->hs_acc + slot_len * (it + 1);
            float* alpha = E->pcg_scal;
            float* beta = E->pcg_scal + M;
            if (timed)
            {
                // Algorithmic bytes: p 4 in (+ z 4 when fused), Ap 4 out (+ p 4 when fused).
                LSDTT_TIMED("ens_hillslope_apply", (it ? 16.0 : 8.0) * cells, s2,
                            (ens_hs_apply_tiled<<<G.ntile, 256, 0, s2>>>(E->P, E->d_prm, E->strip_member, E->mask,
                                                                         E->dof, E->done, it ? 1 : 0, beta, it_dev, E->zz,
                                                                         p_prev, p_it, E->Ap, E->part, G.tlist)));
            }
            else
                ens_hs_apply_tiled<<<G.ntile, 256, 0, s2>>>(E->P, E->d_prm, E->strip_member, E->mask, E->dof, E->done,
                                                            it ? 1 : 0, beta, it_dev, E->zz, p_prev, p_it, E->Ap, E->part,
                                                            G.tlist);
            reduce(s2, 1, 0u, E->done, cur, kHsSlot, 0, it_dev, 1);
            // alpha = r.z (slot it) / p.Ap (slot it + 1)
            LSDTT_TIMED("ens_pcg_ratio", 0.0, s2,
                        (ens_pcg_ratio<<<mb, 128, 0, s2>>>(M, E->done, E->hs_acc, it, 1, it + 1, 0, it_dev, alpha)));
            if (timed)
            {
                // Algorithmic bytes: the update 24 B/cell.
                LSDTT_TIMED("ens_hillslope_update", 24.0 * cells, s2,
                            (ens_hs_update<<<G.nblk, 256, 0, s2>>>(E->P, E->done, alpha, E->invd, p_it, E->Ap, E->x,
                                                                   E->r, E->zz, E->part, G.blist)));
            }
            else
                ens_hs_update<<<G.nblk, 256, 0, s2>>>(E->P, E->done, alpha, E->invd, p_it, E->Ap, E->x, E->r, E->zz,
                                                      E->part, G.blist);
            reduce(s2, 2, 0u, E->done, cur, kHsSlot, 1, it_dev);
            // beta for the next iteration = r.z (slot it + 1) / r.z (slot it)
            LSDTT_TIMED("ens_pcg_ratio", 0.0, s2,
                        (ens_pcg_ratio<<<mb, 128, 0, s2>>>(M, E->done, E->hs_acc, it + 1, 1, it, 1, it_dev, beta)));
        };
        if (device_loop)
        {
            // Device-side loop: two iterations and the convergence test per trip,
            // until no member is iterating (each member stops at its own
            // max_iter; all of them by max_iter_all).
            cudaMemsetAsync(E->loopc + 1, 0, sizeof(int), hs);
            cudaMemsetAsync(E->flags + 5, 0, sizeof(int), hs);
            e = capture_while(hs, E->own2, [&](cudaStream_t s2, cudaGraphConditionalHandle h) {
                iteration(s2, 0, E->loopc + 1, false);
                iteration(s2, 1, E->loopc + 1, false);
                ens_hs_check<<<mb, 128, 0, s2>>>(M, E->d_prm, 1, E->hs_acc + slot_len * 2, E->hs_bb, E->done, E->iters,
                                                 E->flags, E->loopc + 1);
                ens_pcg_while<<<1, 1, 0, s2>>>(E->loopc + 1, itmax, E->flags, h);
            });
            if (e != cudaSuccess) return e;
        }
        else
        {
            int it = 0;
            for (; it < itmax;)
            {
                const int batch = std::min(4, itmax - it);
                for (int k = 0; k < batch; ++k, ++it) iteration(hs, it, nullptr, true);
                if (eager) cudaMemsetAsync(E->flags + 5, 0, sizeof(int), hs);
                ens_hs_check<<<mb, 128, 0, hs>>>(M, E->d_prm, it - 1,
                                                E->hs_acc + static_cast<std::size_t>(kHsSlot) * M * it, E->hs_bb,
                                                E->done, E->iters, E->flags);
                if (eager)
                {
                    cudaMemcpyAsync(E->h_flags + 5, E->flags + 5, sizeof(int), cudaMemcpyDeviceToHost, hs);
                    e = cudaStreamSynchronize(hs);
                    if (e != cudaSuccess) return e;
                    if (E->h_flags[5] == 0) break;
                }
            }
            if (eager) rec->pcg_iters = it;
            else ens_hs_overflow<<<mb, 128, 0, hs>>>(M, E->done, E->flags);
        }
        return cudaSuccess;
    };
    if (split_groups)
    {
        // shallow group beside the deep group's sweep, then the deep group
        const std::int32_t* L = E->glist;
        const HsGroup shallow{L, static_cast<unsigned>(E->gcount[0]),
                              L + E->gcount[0] + E->gcount[1], static_cast<unsigned>(E->gcount[2]), E->grp, 0};
        const HsGroup deep{L + E->gcount[0], static_cast<unsigned>(E->gcount[1]),
                           L + E->gcount[0] + E->gcount[1] + E->gcount[2], static_cast<unsigned>(E->gcount[3]),
                           E->grp, 1};
        e = hillslope_stage(st, shallow);
        if (e != cudaSuccess) return e;
        cudaStreamWaitEvent(st, E->ev_join, 0);
        e = hillslope_stage(st, deep);
    }
    else
        e = hillslope_stage(st, HsGroup{nullptr, nb, nullptr, static_cast<unsigned>(E->S), nullptr, 0});
    if (e != cudaSuccess) return e;
    // 5. the increment, uplift + boundary restore and the statistics in one
    // pass; flags to the host
    // Algorithmic bytes per cell (uplift + restore + statistics): 12.
    LSDTT_TIMED("ens_step_finish", 12.0 * cells, st,
                (ens_step_finish<<<nb, 256, 0, st>>>(E->P, E->d_prm, E->mask, E->bflag, E->dof, E->zsp, E->x, E->zf,
                                                     E->z, E->part)));
    reduce(st, 8, 0xf0u, nullptr, E->stats_acc, 8, 0, nullptr);
    cudaMemcpyAsync(E->h_stats, E->stats_acc, sizeof(double) * 8 * M, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(E->h_flags, E->flags, sizeof(int) * kFlags, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(E->h_iters, E->iters, sizeof(int) * M, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(E->h_err, f->derr, sizeof(unsigned long long) * 4, cudaMemcpyDeviceToHost, st);
    return cudaGetLastError();
}

// Capture one step with the schedule derived from the record.
cudaError_t capture(lsdtt_gpu_ensemble* E, const StepRecord& rec, cudaStream_t st)
{
    if (E->exec) cudaGraphExecDestroy(E->exec);
    if (E->graph) cudaGraphDestroy(E->graph);
    E->exec = nullptr;
    E->graph = nullptr;
    E->fill_cap = std::max(8, ((rec.fill_passes + std::max(8, rec.fill_passes / 4)) + 3) / 4 * 4);
    E->depth_cap = std::max(rec.max_depth * 2, rec.max_depth + 256) + 2;
    E->depth_cap = static_cast<int>(std::min<std::int64_t>(E->depth_cap, E->N + 1));
    E->it_cap = std::min(E->max_iter_all, std::max(8, (rec.pcg_iters + std::max(8, rec.pcg_iters / 2) + 3) / 4 * 4));
    // A one-shot override of the caps captures the capped loops (which can
    // overflow: the recovery path), the device-side loops otherwise.
    const bool capped = E->ov_fill > 0 || E->ov_it > 0;
    const bool use_while = E->use_while;
    if (capped) E->use_while = false;
    if (E->ov_fill > 0) E->fill_cap = E->ov_fill;
    if (E->ov_it > 0) E->it_cap = E->ov_it;
    E->ov_fill = E->ov_it = 0;
    // levels of this profile above the tuned tail threshold get a launch each
    E->split = E->tail == 0 ? rec.max_depth + 1 : split_for(rec.level_size, E->tail);
    E->level_blocks = level_grid(rec.level_size, E->split, E->sweep_block, 1.5);
    cudaError_t e = (E->sweep_mode == 3 && E->groups_on) ? set_member_groups(E, E->depth_last, st) : cudaSuccess;
    if (e != cudaSuccess) return e;
    if (E->sweep_mode != 3 || !E->groups_on) E->n_deep = 0;
    cudaGraph_t g = nullptr;
    for (int attempt = 0; attempt < 2; ++attempt)
    {
        e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return e;
        StepRecord dummy;
        cudaError_t e_run = run_step(E, st, false, &dummy);
        g = nullptr;
        e = cudaStreamEndCapture(st, &g);
        if (e_run != cudaSuccess) e = e_run;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&E->exec, g, 0);
        if (e == cudaSuccess) break;
        if (g) cudaGraphDestroy(g);
        g = nullptr;
        // A driver without conditional nodes: capture the capped loops.
        if (!E->use_while)
        {
            if (capped) E->use_while = use_while;
            return e;
        }
        cudaGetLastError();
        E->use_while = false;
    }
    if (capped && e == cudaSuccess) E->use_while = use_while;
    E->graph = g;
    E->captured = true;
    ++E->info.graph_captures;
    return cudaSuccess;
}

void fill_stats(const lsdtt_gpu_ensemble* E, lsdtt_gpu_lem_stats* stats)
{
    for (int m = 0; m < E->M; ++m)
    {
        const double* A = E->h_stats + 8 * m;
        const lsdtt_gpu_lem_options& o = E->members[static_cast<std::size_t>(m)].options;
        const double nv = A[3];
        const double inv_dt = 1.0 / static_cast<double>(o.timestep);
        const double inv_n = nv > 0 ? 1.0 / nv : 0.0;
        lsdtt_gpu_lem_stats& s = stats[m];
        s.delta_max_elevation = static_cast<float>(std::fabs(A[5] - A[4]));
        s.delta_mean_elevation = static_cast<float>(std::fabs(A[0] * inv_n));
        s.max_local_elevation_change = static_cast<float>(A[6]);
        const double me = A[7];
        s.mean_erosion_rate = static_cast<float>(A[2] * inv_n * inv_dt);
        s.max_erosion_rate = static_cast<float>((me > 0 ? me : 0.0) * inv_dt);
        s.hillslope_iterations = E->h_iters[m];
        s.p999_local_elevation_change = 0.0f;
        s.reserved = 0;
    }
}

}  // namespace

extern "C" {

int lsdtt_gpu_ensemble_create(const lsdtt_gpu_member* members, int32_t n_members, int32_t use_graph,
                              lsdtt_gpu_ensemble** out, void* stream)
{
    const char* who = "lsdtt_gpu_ensemble_create";
    if (!members || !out || n_members <= 0) return fail(LSDTT_GPU_EINVAL, std::string(who) + ": bad argument");
    *out = nullptr;
    if (n_members > 65535) return fail(LSDTT_GPU_EINVAL, std::string(who) + ": at most 65535 members");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(LSDTT_GPU_ENODEV, std::string(who) + ": no CUDA device");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaFuncSetAttribute(ens_mdepth_sort, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(kMdSortMaxSmem)) != cudaSuccess)
        return cuda_fail(cudaGetLastError(), "lsdtt_gpu_ensemble_create: shared memory of the member depth sort");
    if (cudaFuncSetAttribute(ens_sp_clusters, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
        cudaGetLastError();  // without it the 16-CTA clusters are refused and not chosen
    auto* E = new lsdtt_gpu_ensemble();
    E->M = n_members;
    E->use_graph = use_graph != 0;
    E->members.assign(members, members + n_members);
    E->member_set.assign(static_cast<std::size_t>(n_members), 0);
    std::int64_t base = 0;
    std::int32_t tiles = 0;
    std::int32_t strips = 0;     // 128 x 32 receiver tiles
    std::int64_t perim = 0;      // perimeter cells of all members
    for (int k = 0; k < n_members; ++k)
    {
        const lsdtt_gpu_grid& g = members[k].grid;
        const lsdtt_gpu_lem_options& o = members[k].options;
        const std::string mk = std::string(who) + ": member " + std::to_string(k);
        if (!(g.n_rows > 0 && g.n_cols > 0 && g.cell_size > 0.0) ||
            static_cast<std::int64_t>(g.n_rows) * g.n_cols >= (std::int64_t(1) << 31))
        {
            free_ensemble(E);
            return fail(LSDTT_GPU_EINVAL, mk + ": raster metadata is invalid");
        }
        if (!(o.timestep > 0.0f))
        {
            free_ensemble(E);
            return fail(LSDTT_GPU_EINVAL, mk + ": timestep must be positive");
        }
        if (o.enable_hillslope && o.hillslope_nonlinear)
        {
            free_ensemble(E);
            return fail(LSDTT_GPU_EINVAL, mk + ": ensembles run the linear hillslope law");
        }
        auto is_p = [&](int i) { return g.boundary_conditions[i] == 'p' || g.boundary_conditions[i] == 'P'; };
        if (is_p(0) != is_p(2) || is_p(1) != is_p(3) || (is_p(0) && is_p(1)))
        {
            free_ensemble(E);
            return fail(LSDTT_GPU_EINVAL, mk + ": periodic boundary flags must pair up and leave one axis open");
        }
        const std::int64_t n = static_cast<std::int64_t>(g.n_rows) * g.n_cols;
        if (!exact_area(g.cell_size * g.cell_size, n))
        {
            free_ensemble(E);
            return fail(LSDTT_GPU_EINVAL, mk + ": cell_size^2 * cells is not exact in double; the packed "
                                               "accumulation needs the exact contributing-area path");
        }
        PackedMember P{};
        P.base = base;
        P.nr = g.n_rows;
        P.nc = g.n_cols;
        P.cell = g.cell_size;
        P.nodata = g.no_data_value;
        std::memcpy(P.bc, g.boundary_conditions, 4);
        P.tile_base = tiles;
        P.ntx = (g.n_cols + kT - 1) / kT;
        P.nty = (g.n_rows + kT - 1) / kT;
        tiles += P.ntx * P.nty;
        P.rtile_base = strips;
        P.nrx = (g.n_cols + kD8TileCols - 1) / kD8TileCols;
        P.nry = (g.n_rows + kD8TileRows - 1) / kD8TileRows;
        strips += P.nrx * P.nry;
        P.perim_base = perim;
        perim += d8_perimeter(g.n_rows, g.n_cols);
        base += (n + kPackAlign - 1) / kPackAlign * kPackAlign;
        E->member_cells += n;
        E->pm.push_back(P);
        EnsParams q{};
        q.sp.K = o.erodibility;
        q.sp.m = o.m_exponent;
        q.sp.n = o.n_exponent;
        q.sp.dt = o.timestep;
        q.sp.threshold = 0.0f;
        q.sp.slope_clamp = o.slope_clamp;
        q.sp.dx = static_cast<float>(g.cell_size);
        q.sp.dx_diag = q.sp.dx * static_cast<float>(1.4142135623730950488);
        q.sp.divide_by_dx = o.divide_area_by_dx;
        q.sp.n_is_one = std::fabs(o.n_exponent - 1.0f) < 1e-6f ? 1 : 0;
        q.hs.nr = g.n_rows;
        q.hs.nc = g.n_cols;
        q.hs.bn = g.boundary_conditions[0];
        q.hs.be = g.boundary_conditions[1];
        q.hs.bs = g.boundary_conditions[2];
        q.hs.bw = g.boundary_conditions[3];
        q.hs.DA = static_cast<double>(o.hillslope_diffusivity) / (g.cell_size * g.cell_size);
        q.hs.inv_dt = 1.0 / static_cast<double>(o.timestep);
        q.hs.U = 0.0;
        for (int k = 0; k < 5; ++k) q.hs_invd[k] = static_cast<float>(1.0 / (q.hs.inv_dt + q.hs.DA * k));
        q.inv_dt_f = static_cast<float>(q.hs.inv_dt);
        q.DA_f = static_cast<float>(q.hs.DA);
        q.U_f = 0.0f;
        q.inv_card = static_cast<float>(1.0 / g.cell_size);
        q.inv_diag = static_cast<float>(1.0 / (g.cell_size * 1.4142135623730950488));
        q.fill_on = o.fill_min_slope > 0.0f ? 1 : 0;
        q.fill_eps = o.fill_min_slope > 0.0f ? o.fill_min_slope : 0.0f;
        q.L = static_cast<float>(g.cell_size);
        q.Ld = q.L * static_cast<float>(1.4142135623730950488);
        q.per_ns = is_p(0);
        q.per_ew = is_p(1);
        q.udz = o.uplift_rate * o.timestep;
        q.bl = o.baselevel_fall_rate * o.timestep;
        q.dw = g.cell_size * g.cell_size;
        q.hill_on = o.enable_hillslope ? 1 : 0;
        q.rel_tol = o.hillslope_rel_tol > 0 ? o.hillslope_rel_tol : 1e-8;
        q.max_iter = o.hillslope_max_iter > 0 ? o.hillslope_max_iter : 1000;
        E->prm_h.push_back(q);
        E->max_iter_all = std::max(E->max_iter_all, q.max_iter);
        E->max_pass_all = std::max<int>(E->max_pass_all, 4 * (g.n_rows + g.n_cols) + 64);
    }
    E->N = base;
    E->T = tiles;
    E->S = strips;
    E->perim = perim;
    const std::int64_t N = E->N;
    if (2 * N >= (std::int64_t(1) << 32))
    {
        free_ensemble(E);
        return fail(LSDTT_GPU_EINVAL, std::string(who) + ": the packed ensemble exceeds 2^31 cells");
    }
    std::vector<std::uint16_t> blk(static_cast<std::size_t>(N / kPackAlign));
    std::vector<std::uint16_t> tm(static_cast<std::size_t>(tiles));
    std::vector<std::uint16_t> sm(static_cast<std::size_t>(strips));
    for (int k = 0; k < n_members; ++k)
    {
        const PackedMember& P = E->pm[static_cast<std::size_t>(k)];
        const std::int64_t n = static_cast<std::int64_t>(P.nr) * P.nc;
        const std::int64_t nblk = (n + kPackAlign - 1) / kPackAlign;
        for (std::int64_t b = 0; b < nblk; ++b) blk[static_cast<std::size_t>(P.base / kPackAlign + b)] = k;
        for (int t = 0; t < P.ntx * P.nty; ++t) tm[static_cast<std::size_t>(P.tile_base + t)] = k;
        for (int t = 0; t < P.nrx * P.nry; ++t) sm[static_cast<std::size_t>(P.rtile_base + t)] = k;
    }
    // The stack runs on the packed forest: one flow engine over N cells.
    lsdtt_gpu_grid fg{};
    fg.n_rows = 1;
    fg.n_cols = static_cast<std::int32_t>(N);
    fg.cell_size = 1.0;
    fg.no_data_value = -9999.0;
    std::memcpy(fg.boundary_conditions, "oooo", 4);
    int s = lsdtt_gpu_flow_create(&fg, &E->f);
    if (s != LSDTT_GPU_OK)
    {
        free_ensemble(E);
        return s;
    }
    E->mask = E->f->mask;  // the stack reads the engine's mask
    int lo_prio = 0, hi_prio = 0;  // the deep group's sweep is the step's critical path
    cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio);
    if (cudaStreamCreateWithFlags(&E->own, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&E->own2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithPriority(&E->own3, cudaStreamNonBlocking, hi_prio) != cudaSuccess ||
        cudaEventCreateWithFlags(&E->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&E->ev_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&E->ev_in, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&E->ev_out, cudaEventDisableTiming) != cudaSuccess)
    {
        free_ensemble(E);
        return fail(LSDTT_GPU_ECUDA, std::string(who) + ": stream creation failed");
    }
    cudaError_t e = cudaSuccess;
    auto alloc = [&](auto** p, std::size_t count) {
        if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(p), sizeof(**p) * (count ? count : 1));
    };
    const std::size_t n = static_cast<std::size_t>(N);
    alloc(&E->d_pm, static_cast<std::size_t>(n_members));
    alloc(&E->d_prm, static_cast<std::size_t>(n_members));
    alloc(&E->blk_member, blk.size());
    alloc(&E->tile_member, tm.size());
    alloc(&E->strip_member, sm.size());
    alloc(&E->undecided, 1);
    alloc(&E->z, n);
    alloc(&E->zf, n);
    alloc(&E->zsp, n);
    alloc(&E->zpre, n);
    alloc(&E->kind, n);
    alloc(&E->bflag, n);
    alloc(&E->dirty, 2 * static_cast<std::size_t>(tiles));
    alloc(&E->flist, kFillColours * static_cast<std::size_t>(tiles));
    alloc(&E->glist, static_cast<std::size_t>(n / kPackAlign) + static_cast<std::size_t>(strips));
    alloc(&E->grp, static_cast<std::size_t>(n_members));
    alloc(&E->perm_cap, static_cast<std::size_t>(n_members));
    alloc(&E->fcnt, kFillColours + 1);
    alloc(&E->oflag, n);
    alloc(&E->pos, n);
    alloc(&E->nd, static_cast<std::size_t>(n_members));
    alloc(&E->area, n);
    alloc(&E->order, n);
    alloc(&E->lstart, n + 3);
    alloc(&E->lcount, n + 3);
    alloc(&E->lfill, n + 3);
    alloc(&E->maxd, 1);
    alloc(&E->dof, n);
    alloc(&E->invd, n);
    alloc(&E->b, n);
    alloc(&E->x, n);
    alloc(&E->r, n);
    alloc(&E->p, n);
    alloc(&E->p2, n);
    alloc(&E->zz, n);
    alloc(&E->Ap, n);
    alloc(&E->hs_bb, static_cast<std::size_t>(n_members));
    alloc(&E->hs_acc, static_cast<std::size_t>(kHsSlot) * n_members * (static_cast<std::size_t>(E->max_iter_all) + 2));
    alloc(&E->done, static_cast<std::size_t>(n_members));
    alloc(&E->iters, static_cast<std::size_t>(n_members));
    alloc(&E->stats_acc, 8 * static_cast<std::size_t>(n_members));
    alloc(&E->part, 8 * (n / kPackAlign));
    alloc(&E->kam_tab, static_cast<std::size_t>(n_members) * kKamTab);
    alloc(&E->zg, n);
    alloc(&E->dfc, 2);
    alloc(&E->flags, kFlags);
    alloc(&E->bar, 2);
    alloc(&E->loopc, 2);
    alloc(&E->pcg_scal, 2 * static_cast<std::size_t>(n_members));
    alloc(&E->morder, n);
    alloc(&E->mstart, n + 2);
    alloc(&E->mmax, static_cast<std::size_t>(n_members));
    alloc(&E->perm, static_cast<std::size_t>(n_members));
    if (e == cudaSuccess) e = cudaMallocHost(&E->h_stats, sizeof(double) * 8 * n_members);
    if (e == cudaSuccess) e = cudaMallocHost(&E->h_flags, sizeof(int) * kFlags);
    if (e == cudaSuccess) e = cudaMallocHost(&E->h_iters, sizeof(int) * n_members);
    if (e == cudaSuccess) e = cudaMallocHost(&E->h_maxd, sizeof(std::uint32_t));
    if (e == cudaSuccess) e = cudaMallocHost(&E->h_err, sizeof(unsigned long long) * 4);
    if (e == cudaSuccess) e = cudaMallocHost(&E->h_fcnt, sizeof(unsigned long long) * (kFillColours + 1));
    // The epsilon fill in the reference's order: member table, FIFO rings
    // of the global-memory replay (a power of two of entries per member)
    // and the replay's buffers.
    std::vector<ExMember> exm(static_cast<std::size_t>(n_members));
    {
        std::int64_t fifo_total = 0;
        for (int k = 0; k < n_members; ++k)
        {
            const PackedMember& Pm = E->pm[static_cast<std::size_t>(k)];
            const EnsParams& q = E->prm_h[static_cast<std::size_t>(k)];
            ExMember& x = exm[static_cast<std::size_t>(k)];
            const std::int64_t cells_k = static_cast<std::int64_t>(Pm.nr) * Pm.nc;
            std::int64_t cap = 2;
            while (cap < cells_k) cap <<= 1;
            x.base = Pm.base;
            x.fifo_base = fifo_total;
            x.fifo_cap = static_cast<std::uint32_t>(cap);
            x.nr = Pm.nr;
            x.nc = Pm.nc;
            x.L = q.L;
            x.Ld = q.Ld;
            x.eps = q.fill_eps;
            x.nodata = static_cast<float>(Pm.nodata);
            x.per_ns = q.per_ns;
            x.per_ew = q.per_ew;
            x.on = (q.fill_on && q.fill_eps > 0.0f) ? 1 : 0;
            if (x.on)
            {
                E->ex_any = true;
                ++E->ex_on;
            }
            fifo_total += cap;
        }
        while ((1 << E->ex_mbits) < n_members) ++E->ex_mbits;
        if (E->ex_any)
        {
            alloc(&E->zf0, n);
            alloc(&E->d_exm, static_cast<std::size_t>(n_members));
            const std::size_t exb = ex_bytes(N, n_members, fifo_total);
            alloc(&E->exbuf, exb);
            if (e == cudaSuccess)
            {
                E->exws = Scratch{E->exbuf, exb, 0};
                if (!ex_carve(E->exws, N, n_members, fifo_total, E->exB)) e = cudaErrorMemoryAllocation;
            }
            if (e == cudaSuccess) e = ex_setup();
        }
    }
    {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        // One wave of resident blocks: with more, the blocks that are not
        // resident start their share of the tiles only when a resident one
        // has finished all of its own.
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ens_fill_relax_list, kFillThreads, 0) !=
                cudaSuccess ||
            per_sm < 1 || per_sm > 8)
        {
            cudaGetLastError();
            per_sm = 8;
        }
        E->fill_grid = static_cast<unsigned>(std::max(1, sms) * per_sm);
        E->sms = std::max(1, sms);
        for (const PackedMember& Pm : E->pm)
        {
            const lsdtt_gpu_grid& g = E->members[&Pm - E->pm.data()].grid;
            auto per = [&](int i) { return g.boundary_conditions[i] == 'p' || g.boundary_conditions[i] == 'P'; };
            E->fill_colours |= fill_colour_mask(Pm.ntx, Pm.nty, per(0), per(1));
        }
    }
    if (e != cudaSuccess)
    {
        free_ensemble(E);
        return cuda_fail(e, who);
    }
    cudaMemcpyAsync(E->d_pm, E->pm.data(), sizeof(PackedMember) * n_members, cudaMemcpyHostToDevice, st);
    std::vector<std::int32_t> chain_order(static_cast<std::size_t>(n_members));
    if (E->d_exm)
    {
        cudaMemcpyAsync(E->d_exm, exm.data(), sizeof(ExMember) * n_members, cudaMemcpyHostToDevice, st);
        // the exact fill's chain blocks, largest members first (their long
        // episodes set the fill's time; the rest finish around them)
        for (int k = 0; k < n_members; ++k) chain_order[static_cast<std::size_t>(k)] = k;
        std::stable_sort(chain_order.begin(), chain_order.end(), [&](std::int32_t a, std::int32_t b) {
            const PackedMember &A = E->pm[static_cast<std::size_t>(a)], &Bm = E->pm[static_cast<std::size_t>(b)];
            return static_cast<std::int64_t>(A.nr) * A.nc > static_cast<std::int64_t>(Bm.nr) * Bm.nc;
        });
        cudaMemcpyAsync(E->exB.chain_order, chain_order.data(), sizeof(std::int32_t) * n_members,
                        cudaMemcpyHostToDevice, st);
        cudaStreamSynchronize(st);  // chain_order is a local vector
    }
    cudaMemcpyAsync(E->d_prm, E->prm_h.data(), sizeof(EnsParams) * n_members, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(E->blk_member, blk.data(), sizeof(std::uint16_t) * blk.size(), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(E->tile_member, tm.data(), sizeof(std::uint16_t) * tm.size(), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(E->strip_member, sm.data(), sizeof(std::uint16_t) * sm.size(), cudaMemcpyHostToDevice, st);
    {
        std::vector<std::uint16_t> perm(static_cast<std::size_t>(n_members));
        for (int k = 0; k < n_members; ++k) perm[static_cast<std::size_t>(k)] = static_cast<std::uint16_t>(k);
        std::stable_sort(perm.begin(), perm.end(), [&](std::uint16_t a, std::uint16_t b) {
            const PackedMember &A = E->pm[a], &B = E->pm[b];
            return static_cast<std::int64_t>(A.nr) * A.nc > static_cast<std::int64_t>(B.nr) * B.nc;
        });
        E->perm_h = perm;
    }
    cudaMemcpyAsync(E->perm, E->perm_h.data(), sizeof(std::uint16_t) * E->perm_h.size(), cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(E->z, 0, sizeof(float) * n, st);
    cudaMemsetAsync(E->mask, 0, n, st);
    // the PCG's padding cells (between members) stay zero: the tiled apply
    // covers member cells only
    cudaMemsetAsync(E->p, 0, sizeof(float) * n, st);
    cudaMemsetAsync(E->p2, 0, sizeof(float) * n, st);
    cudaMemsetAsync(E->Ap, 0, sizeof(float) * n, st);
    cudaMemsetAsync(E->x, 0, sizeof(float) * n, st);  // the first step's PCG starts from zero
    cudaMemsetAsync(E->zg, 0, sizeof(unsigned long long) * n, st);
    // padding cells between members: no receiver, no direction, ever
    cudaMemsetAsync(E->f->receiver, 0xFF, sizeof(std::int64_t) * n, st);
    cudaMemsetAsync(E->f->dir, 0xFF, n, st);
    cudaMemsetAsync(E->dfc, 0, sizeof(std::uint32_t) * 2, st);
    {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ens_sp_dataflow, 256, 0);
        E->df_grid = std::max(1, sms * std::max(1, per_sm));
        per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ens_sp_coop, 512, 0);
        E->coop_grid = std::max(1, sms * std::max(1, std::min(per_sm, 2)));
    }
    E->P.m = E->d_pm;
    E->P.blk_member = E->blk_member;
    E->P.n = N;
    E->P.n_members = n_members;
    ens_kam_table<<<grid_blocks(static_cast<std::int64_t>(n_members) * kKamTab, 256), 256, 0, st>>>(E->P, E->d_prm,
                                                                                                   E->kam_tab);
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
    {
        free_ensemble(E);
        return cuda_fail(e, who);
    }
    E->info.packed_cells = N;
    E->info.member_cells = E->member_cells;
    E->info.graph_enabled = E->use_graph ? 1 : 0;
    *out = E;
    return LSDTT_GPU_OK;
}

int lsdtt_gpu_ensemble_destroy(lsdtt_gpu_ensemble* E)
{
    if (E) free_ensemble(E);
    return LSDTT_GPU_OK;
}

int lsdtt_gpu_ensemble_offsets(const lsdtt_gpu_ensemble* E, int64_t* offsets)
{
    if (!E || !offsets) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_ensemble_offsets: null argument");
    for (int k = 0; k < E->M; ++k) offsets[k] = E->pm[static_cast<std::size_t>(k)].base;
    offsets[E->M] = E->N;
    return LSDTT_GPU_OK;
}

int lsdtt_gpu_ensemble_set_member(lsdtt_gpu_ensemble* E, int32_t k, const float* z_dev, const uint8_t* mask_dev,
                                  void* stream)
{
    if (!E || !z_dev || !mask_dev || k < 0 || k >= E->M)
        return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_ensemble_set_member: bad argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const PackedMember& P = E->pm[static_cast<std::size_t>(k)];
    const std::size_t n = static_cast<std::size_t>(P.nr) * P.nc;
    cudaMemcpyAsync(E->z + P.base, z_dev, sizeof(float) * n, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(E->mask + P.base, mask_dev, n, cudaMemcpyDeviceToDevice, st);
    ens_boundary_flag<<<grid_blocks(E->N, 256), 256, 0, st>>>(E->P, E->mask, E->bflag);
    // Mask changes alter the valid count the stack checks against.
    E->member_set[static_cast<std::size_t>(k)] = 1;
    E->ready = std::all_of(E->member_set.begin(), E->member_set.end(), [](char c) { return c != 0; });
    E->captured = false;  // the valid count (a captured constant) may have changed
    const cudaError_t e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? LSDTT_GPU_OK : cuda_fail(e, "lsdtt_gpu_ensemble_set_member");
}

int lsdtt_gpu_ensemble_set_surface(lsdtt_gpu_ensemble* E, int32_t k, const float* z_dev, void* stream)
{
    if (!E || !z_dev || k < 0 || k >= E->M) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_ensemble_set_surface: bad argument");
    if (!E->member_set[static_cast<std::size_t>(k)])
        return fail(LSDTT_GPU_ESTATE, "lsdtt_gpu_ensemble_set_surface: member has no mask yet (set_member first)");
    const PackedMember& P = E->pm[static_cast<std::size_t>(k)];
    const std::size_t n = static_cast<std::size_t>(P.nr) * P.nc;
    // Elevations only: the mask, the boundary flats and the captured step stay valid.
    const cudaError_t e = cudaMemcpyAsync(E->z + P.base, z_dev, sizeof(float) * n, cudaMemcpyDeviceToDevice,
                                          static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? LSDTT_GPU_OK : cuda_fail(e, "lsdtt_gpu_ensemble_set_surface");
}

int lsdtt_gpu_ensemble_get_member(const lsdtt_gpu_ensemble* E, int32_t k, float* z_dev, void* stream)
{
    if (!E || !z_dev || k < 0 || k >= E->M) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_ensemble_get_member: bad argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const PackedMember& P = E->pm[static_cast<std::size_t>(k)];
    cudaMemcpyAsync(z_dev, E->z + P.base, sizeof(float) * static_cast<std::size_t>(P.nr) * P.nc,
                    cudaMemcpyDeviceToDevice, st);
    const cudaError_t e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? LSDTT_GPU_OK : cuda_fail(e, "lsdtt_gpu_ensemble_get_member");
}

int lsdtt_gpu_ensemble_step(lsdtt_gpu_ensemble* E, int32_t n_steps, lsdtt_gpu_lem_stats* stats, void* stream)
{
    const char* who = "lsdtt_gpu_ensemble_step";
    if (!E || n_steps < 0) return fail(LSDTT_GPU_EINVAL, std::string(who) + ": bad argument");
    if (!E->ready) return fail(LSDTT_GPU_ESTATE, std::string(who) + ": every member needs a surface and a mask");
    // Work runs on the handle's own stream, ordered after the caller's
    // stream; the caller's stream waits for it at the end.
    cudaStream_t user = static_cast<cudaStream_t>(stream);
    cudaStream_t st = E->own;
    cudaEventRecord(E->ev_in, user);
    cudaStreamWaitEvent(st, E->ev_in, 0);
    const bool graph_ok = E->use_graph && !profiling_enabled();
    for (int s = 0; s < n_steps; ++s)
    {
        cudaError_t e = cudaSuccess;
        bool ran = false;
        if (graph_ok && E->captured)
        {
            e = cudaGraphLaunch(E->exec, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) return cuda_fail(e, who);
            ++E->info.graph_replays;
            const int* F = E->h_flags;
            if (F[1] || F[2] || F[3])
            {
                // Outgrew the captured schedule: undo and rerun eagerly.
                cudaMemcpyAsync(E->z, E->zpre, sizeof(float) * E->N, cudaMemcpyDeviceToDevice, st);
                E->captured = false;
            }
            else
                ran = true;
        }
        if (!ran)
        {
            if (E->f->n_valid < 0 || !E->captured)
            {
                // The stack checks s-vector ranges against the valid count.
                std::int64_t nv = 0;
                std::vector<std::uint8_t> hm(static_cast<std::size_t>(E->N));
                e = cudaMemcpyAsync(hm.data(), E->mask, hm.size(), cudaMemcpyDeviceToHost, st);
                if (e == cudaSuccess) e = cudaStreamSynchronize(st);
                if (e != cudaSuccess) return cuda_fail(e, who);
                for (std::uint8_t v : hm) nv += v ? 1 : 0;
                E->f->n_valid = nv;
            }
            StepRecord rec;
            e = run_step(E, st, true, &rec);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e == cudaErrorLaunchTimeout) return fail(LSDTT_GPU_ETIMEOUT, std::string(who) + ": fill did not converge");
            if (e != cudaSuccess) return cuda_fail(e, who);
            ++E->info.eager_steps;
            E->info.last_fill_passes = rec.fill_passes;
            E->info.last_max_depth = rec.max_depth;
            E->info.last_hillslope_iterations = rec.pcg_iters;
            if (graph_ok)
            {
                // Keep the eager step's flags and statistics: capturing
                // enqueues nothing that runs.
                std::vector<int> fl(E->h_flags, E->h_flags + kFlags);
                std::vector<double> sv(E->h_stats, E->h_stats + 8 * E->M);
                std::vector<int> itv(E->h_iters, E->h_iters + E->M);
                e = capture(E, rec, st);
                if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_ensemble_step (graph capture)");
                std::copy(fl.begin(), fl.end(), E->h_flags);
                std::copy(sv.begin(), sv.end(), E->h_stats);
                std::copy(itv.begin(), itv.end(), E->h_iters);
            }
        }
        if (E->h_flags[7])
            return fail(LSDTT_GPU_ETIMEOUT, std::string(who) + ": the stream-power sweep hit its wait limit");
        if (E->h_flags[8])
            return fail(LSDTT_GPU_EOVERFLOW, std::string(who) + ": a fill window replay outgrew its arrays");
        if ((E->h_err[0] & 0xffffffffull) != 0)
            return fail(LSDTT_GPU_ECYCLIC, std::string(who) + ": the receiver graph of a member has a cycle");
        if (E->h_flags[4])
            return fail(LSDTT_GPU_ENOCONV, std::string(who) + ": a member's hillslope Jacobi-PCG did not reach its "
                                                              "relative residual within hillslope_max_iter");
    }
    cudaEventRecord(E->ev_out, st);
    cudaStreamWaitEvent(user, E->ev_out, 0);
    E->info.fill_pass_cap = E->fill_cap;
    E->info.depth_cap = E->depth_cap;
    E->info.sweep_split_level = E->split;
    E->info.sweep_block = E->sweep_block;
    E->info.sweep_dataflow = E->sweep_mode;
    E->info.deep_members = E->captured ? E->n_deep : 0;
    E->info.hillslope_iteration_cap = E->it_cap;
    if (stats) fill_stats(E, stats);
    return LSDTT_GPU_OK;
}

int lsdtt_gpu_ensemble_upload(lsdtt_gpu_ensemble* E, const float* z_host, void* stream)
{
    if (!E || !z_host) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_ensemble_upload: null argument");
    const cudaError_t e = cudaMemcpyAsync(E->z, z_host, sizeof(float) * E->N, cudaMemcpyHostToDevice,
                                          static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? LSDTT_GPU_OK : cuda_fail(e, "lsdtt_gpu_ensemble_upload");
}

int lsdtt_gpu_ensemble_download(const lsdtt_gpu_ensemble* E, float* z_host, void* stream)
{
    if (!E || !z_host) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_ensemble_download: null argument");
    const cudaError_t e = cudaMemcpyAsync(z_host, E->z, sizeof(float) * E->N, cudaMemcpyDeviceToHost,
                                          static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? LSDTT_GPU_OK : cuda_fail(e, "lsdtt_gpu_ensemble_download");
}

int lsdtt_gpu_ensemble_override_schedule(lsdtt_gpu_ensemble* E, int32_t fill_pass_cap, int32_t hillslope_iteration_cap,
                                         int32_t sweep_mode)
{
    if (!E || fill_pass_cap < 0 || hillslope_iteration_cap < 0 || sweep_mode < -1 || sweep_mode > 3)
        return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_ensemble_override_schedule: bad argument");
    E->ov_fill = fill_pass_cap;
    E->ov_it = hillslope_iteration_cap;
    if (sweep_mode >= 0)
    {
        E->sweep_mode = sweep_mode;
        E->forced_mode = true;
    }
    E->captured = false;
    return LSDTT_GPU_OK;
}

int lsdtt_gpu_ensemble_set_member_groups(lsdtt_gpu_ensemble* E, int32_t enabled)
{
    if (!E || enabled < 0 || enabled > 1)
        return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_ensemble_set_member_groups: bad argument");
    E->groups_on = enabled != 0;
    E->captured = false;
    return LSDTT_GPU_OK;
}

int lsdtt_gpu_ensemble_get_info(const lsdtt_gpu_ensemble* E, lsdtt_gpu_ensemble_info* info)
{
    if (!E || !info) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_ensemble_get_info: null argument");
    *info = E->info;
    return LSDTT_GPU_OK;
}

}  // extern "C"

// lsdtt_gpu_selftest_grid_barrier (no reference counterpart): runs the
// cooperative sweep's bounded grid barrier against an arrival that never
// comes. Returns LSDTT_GPU_ETIMEOUT when the wait gave up as designed (the
// expected outcome), LSDTT_GPU_OK if it was released (a fault of the
// barrier), another status on a CUDA error. The context stays usable.
extern "C" int lsdtt_gpu_selftest_grid_barrier(int32_t spin_limit)
{
    using namespace lsdtt_gb300;
    if (spin_limit <= 0) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_selftest_grid_barrier: spin_limit must be positive");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(LSDTT_GPU_ENODEV, "lsdtt_gpu_selftest_grid_barrier: no CUDA device");
    int* buf = nullptr;  // bar[2], abort flag, released
    cudaError_t e = cudaMalloc(&buf, 4 * sizeof(int));
    if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_selftest_grid_barrier");
    int host[4] = {0, 0, 0, -1};
    e = cudaMemset(buf, 0, 4 * sizeof(int));
    if (e == cudaSuccess)
    {
        ens_barrier_selftest<<<1, 128>>>(reinterpret_cast<unsigned*>(buf), buf + 2, buf + 3, spin_limit);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(host, buf, sizeof(host), cudaMemcpyDeviceToHost);
    cudaFree(buf);
    if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_selftest_grid_barrier");
    if (host[3] == 0 && host[2] == 1)
        return fail(LSDTT_GPU_ETIMEOUT, "lsdtt_gpu_selftest_grid_barrier: the bounded grid barrier gave up after " +
                                            std::to_string(spin_limit) + " polls and raised the abort flag");
    return LSDTT_GPU_OK;
}

namespace lsdtt_gb300
{
LSDTT_DEFINE_LAUNCH_READER(ensemble)
}  // namespace lsdtt_gb300
