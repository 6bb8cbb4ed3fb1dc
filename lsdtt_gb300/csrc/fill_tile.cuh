// fill_tile.cuh -- the epsilon-fill relaxation rules, shared by the
// single-grid fill (fill.cu) and the packed ensemble (ensemble.cu).
// See fill.cu for the algorithm and its relation to the reference's
// priority flood.
#pragma once

#include <cmath>

#include "common.cuh"

namespace lsdtt_gb300
{
namespace
{

constexpr int kT = 32;                                   // tile edge (cells)
constexpr int kH = kT + 2;                               // with halo
constexpr int kMaxLocal = 4 * kT;
constexpr int kFillThreads = 256;                        // threads per tile (32 x 8 block)
constexpr int kFillBlocks = (kT / 2) * (kT / 2) / kFillThreads;  // 2 x 2 blocks per thread

// Tile colours of a fill pass. A pass relaxes its active tiles one colour
// after another, in place; no two tiles of one colour are neighbours
// (including diagonal and periodic ones), so a tile reads every neighbour
// either settled in an earlier colour of this pass or untouched since the
// last pass: the result depends only on the inputs, not on which tiles ran
// first (the discoverer rule is not monotone, so halos read from a field
// that neighbours update meanwhile made it depend on scheduling), and a
// change can still cross several tiles in one pass. Colour = cx + 3 cy with
// cx the parity of the tile column, or 2 for the last column of a periodic
// axis with an odd tile count (it neighbours column 0); cy likewise.
constexpr int kFillColours = 9;

// Bit c set: colour c can hold tiles of an ntx x nty tile grid (host side:
// the passes launch only those colours; four for a grid without wrap).
inline unsigned fill_colour_mask(int ntx, int nty, bool per_ns, bool per_ew)
{
    unsigned mx = 1u | (ntx > 1 ? 2u : 0u) | ((per_ew && (ntx & 1) && ntx > 1) ? 4u : 0u);
    unsigned my = 1u | (nty > 1 ? 2u : 0u) | ((per_ns && (nty & 1) && nty > 1) ? 4u : 0u);
    unsigned m = 0;
    for (int cy = 0; cy < 3; ++cy)
        for (int cx = 0; cx < 3; ++cx)
            if (((mx >> cx) & 1u) && ((my >> cy) & 1u)) m |= 1u << (cx + 3 * cy);
    return m;
}

__host__ __device__ __forceinline__ int fill_colour(int tx, int ty, int ntx, int nty, bool per_ns, bool per_ew)
{
    const int cx = (per_ew && (ntx & 1) && ntx > 1 && tx == ntx - 1) ? 2 : (tx & 1);
    const int cy = (per_ns && (nty & 1) && nty > 1 && ty == nty - 1) ? 2 : (ty & 1);
    return cx + 3 * cy;
}

__device__ __forceinline__ float raise_from(float zeta, float min_slope, float d)
{
    // min_slope <= 0: the neighbour takes the spill value itself (:491-494).
    if (!(min_slope > 0.0f)) return zeta;
    // max(zeta + min_slope*d, nextafter(zeta, +inf)) in float, no contraction
    const float requested = __fadd_rn(zeta, __fmul_rn(min_slope, d));
    const float strict = nextafterf(zeta, INFINITY);
    return fmaxf(requested, strict);
}

// Resolve a neighbour for the fill: periodic wrap on periodic axes only,
// otherwise off-grid = none.
__device__ __forceinline__ bool fill_nb(int nr, int nc, bool per_ns, bool per_ew, int r, int c, int d, int& rr,
                                        int& cc)
{
    rr = r + d8_dr(d);
    cc = c + d8_dc(d);
    if (per_ns) { if (rr < 0) rr += nr; else if (rr >= nr) rr -= nr; }
    if (per_ew) { if (cc < 0) cc += nc; else if (cc >= nc) cc -= nc; }
    return rr >= 0 && rr < nr && cc >= 0 && cc < nc;
}

// Initial state of one cell (row-major index i of an nr x nc grid): seeds
// (and NaN cells) hold z and are fixed, other valid cells +inf, invalid cells hold the nodata
// value (and are never read as neighbours).
__device__ __forceinline__ void fill_init_cell(int nr, int nc, bool per_ns, bool per_ew, const float* __restrict__ z,
                                               const std::uint8_t* __restrict__ mask, double nodata, int interior_nd,
                                               float* __restrict__ F, std::uint8_t* __restrict__ kind, std::int64_t i)
{
    const int r = static_cast<int>(i / nc);
    const int c = static_cast<int>(i - static_cast<std::int64_t>(r) * nc);
    auto valid_at = [&](std::int64_t k) {
        return mask[k] != 0 && !(isnan(nodata) ? isnan(z[k]) : static_cast<double>(z[k]) == nodata);
    };
    if (!valid_at(i))
    {
        F[i] = static_cast<float>(nodata);
        kind[i] = 0;  // invalid
        return;
    }
    bool seed = (!per_ns && (r == 0 || r == nr - 1)) || (!per_ew && (c == 0 || c == nc - 1));
    if (!seed && interior_nd)
        for (int d = 0; d < 8 && !seed; ++d)
        {
            const int rr = r + d8_dr(d), cc = c + d8_dc(d);
            if (rr >= 0 && rr < nr && cc >= 0 && cc < nc && !valid_at(static_cast<std::int64_t>(rr) * nc + cc))
                seed = true;
        }
    // A NaN elevation in a valid cell is kept as it is and never raised;
    // its neighbours' minimum skips it (fminf ignores NaN), so nothing
    // spills through it. (The reference's heap
    // orders a NaN key arbitrarily; its output there is not defined by
    // the algorithm.)
    const bool nan_cell = isnan(z[i]);
    F[i] = (seed || nan_cell) ? z[i] : INFINITY;
    kind[i] = (seed || nan_cell) ? 2 : 1;  // 2 seed or NaN (fixed), 1 free
}

// Does cell i of an nr x nc grid flag interior nodata (an invalid cell off
// the outer ring)?
__device__ __forceinline__ bool fill_interior_invalid(int nr, int nc, const float* __restrict__ z,
                                                      const std::uint8_t* __restrict__ mask, double nodata,
                                                      std::int64_t i)
{
    const int r = static_cast<int>(i / nc), c = static_cast<int>(i % nc);
    if (r < 1 || r >= nr - 1 || c < 1 || c >= nc - 1) return false;
    const bool valid = mask[i] != 0 && !(isnan(nodata) ? isnan(z[i]) : static_cast<double>(z[i]) == nodata);
    return !valid;
}

// One relaxation pass over tile (tx, ty) of an nr x nc grid tiled ntx x nty,
// run by one 32 x 8 thread block (kFillThreads). dirty_in / dirty_out are the grid's
// per-tile activity planes (ntx * nty entries).
__device__ __forceinline__ void fill_relax_tile(int nr, int nc, bool per_ns, bool per_ew, float L, float Ld,
                                                float min_slope, const float* __restrict__ z,
                                                const std::uint8_t* __restrict__ kind, float* __restrict__ F,
                                                int* __restrict__ changed, const std::uint8_t* __restrict__ dirty_in,
                                                std::uint8_t* __restrict__ dirty_out, const int tx, const int ty,
                                                const int ntx, const int nty, const bool gate = true)
{
    // Active-tile gate: a tile can only change if it or one of its eight
    // neighbouring tiles changed in the previous pass (periodic axes wrap).
    // Callers that list the active tiles beforehand skip it (gate = false).
    if (gate)
    {
        bool active = false;
        for (int dy = -1; dy <= 1 && !active; ++dy)
            for (int dx = -1; dx <= 1; ++dx)
            {
                int yy = ty + dy, xx = tx + dx;
                if (per_ns) yy = (yy + nty) % nty;
                if (per_ew) xx = (xx + ntx) % ntx;
                if (yy < 0 || yy >= nty || xx < 0 || xx >= ntx) continue;
                if (dirty_in[yy * ntx + xx]) { active = true; break; }
            }
        if (!active)
        {
            if (threadIdx.x == 0 && threadIdx.y == 0) dirty_out[ty * ntx + tx] = 0;
            return;
        }
    }
    // Staged tile: filled values with +inf at invalid and off-grid cells (so
    // they never win a minimum).
    __shared__ float sF[kH][kH];
    const int r0 = ty * kT - 1, c0 = tx * kT - 1;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    // Each thread owns kFillBlocks 2 x 2 blocks of the tile (block b: local
    // rows 2*(b / (kT/2))+1 .. +2, columns 2*(b % (kT/2))+1 .. +2, b = tid +
    // j * kFillThreads), so it holds kFillBlocks cells of each colour.
    unsigned free_mask = 0;  // bit 4j + k: block j's cell of colour k is free (kind 1)
    for (int k = tid; k < kH * kH; k += blockDim.x * blockDim.y)
    {
        const int lr = k / kH, lcc = k % kH;
        int r = r0 + lr, c = c0 + lcc;
        if (per_ns) { if (r < 0) r += nr; else if (r >= nr) r -= nr; }
        if (per_ew) { if (c < 0) c += nc; else if (c >= nc) c -= nc; }
        float f = INFINITY;
        if (r >= 0 && r < nr && c >= 0 && c < nc)
        {
            const std::int64_t g = static_cast<std::int64_t>(r) * nc + c;
            if (kind[g] != 0) f = F[g];
        }
        sF[lr][lcc] = f;
    }
    // The thread's own cells (its 2 x 2 blocks) live in registers as well:
    // only the owner writes them, so its copies are always the values other
    // threads read from sF. Three of a cell's eight neighbours, its own value
    // and its elevation come from the registers.
    float own[kFillBlocks][4], zown[kFillBlocks][4];
#pragma unroll
    for (int j = 0; j < kFillBlocks; ++j)
    {
        const int b = tid + j * kFillThreads, bx = b % (kT / 2), by = b / (kT / 2);
#pragma unroll
        for (int k = 0; k < 4; ++k)
        {
            const int lr = 2 * by + 1 + (k >> 1), lc = 2 * bx + 1 + (k & 1);
            const int r = r0 + lr, c = c0 + lc;
            zown[j][k] = INFINITY;
            if (r < nr && c < nc)
            {
                const std::int64_t g = static_cast<std::int64_t>(r) * nc + c;
                if (kind[g] == 1)
                {
                    free_mask |= 1u << (4 * j + k);
                    zown[j][k] = z[g];
                }
            }
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kFillBlocks; ++j)
    {
        const int b = tid + j * kFillThreads, bx = b % (kT / 2), by = b / (kT / 2);
#pragma unroll
        for (int k = 0; k < 4; ++k) own[j][k] = sF[2 * by + 1 + (k >> 1)][2 * bx + 1 + (k & 1)];
    }
    // Each local iteration updates the four colours of the 2 x 2 colouring
    // (local row parity, column parity) in turn, a barrier between them:
    // cells of one colour are never neighbours, so every update reads
    // settled values and the result depends only on the tile's inputs (the
    // discoverer rule is not monotone, so in-place updates racing with their
    // neighbours' reads could settle on different values run to run).
    bool tile_changed = false;
    for (int it = 0; it < kMaxLocal; ++it)
    {
        bool local = false;
#pragma unroll
        for (int k = 0; k < 4; ++k)
        {
#pragma unroll
            for (int j = 0; j < kFillBlocks; ++j)
            {
            const int b = tid + j * kFillThreads, bx = b % (kT / 2), by = b / (kT / 2);
            const int R = 2 * by + 1, C = 2 * bx + 1;  // the block's top-left cell
            const int lr = R + (k >> 1), lc = C + (k & 1);
            if ((free_mask >> (4 * j + k)) & 1u)
            {
                // neighbour (dy, dx): a register when it lies in this block
                // (resolved at compile time: k, dy and dx are constants)
                auto nb = [&](int dy, int dx) -> float {
                    const int yy = (k >> 1) + dy, xx = (k & 1) + dx;
                    if (yy >= 0 && yy <= 1 && xx >= 0 && xx <= 1) return own[j][2 * yy + xx];
                    return sF[R + yy][C + xx];
                };
                const float vN = nb(-1, 0), vNE = nb(-1, 1), vE = nb(0, 1);
                const float vSE = nb(1, 1), vS = nb(1, 0), vSW = nb(1, -1);
                const float vW = nb(0, -1), vNW = nb(-1, -1);
                // lowest neighbour; +inf: none reached yet (or none valid)
                const float cmin = fminf(fminf(vN, vE), fminf(vS, vW));
                const float dmin = fminf(fminf(vNE, vSE), fminf(vSW, vNW));
                const float m = fminf(cmin, dmin);
                if (m < INFINITY)
                {
                    const float zc = zown[j][k];
                    float nv = zc;
                    if (!(zc > m))
                    {
                        // the first neighbour in direction order N, NE, ...,
                        // NW at m decides the step length
                        bool diag = dmin < cmin;
                        if (cmin == dmin)
                            diag = !(vN == m) && ((vNE == m) || (!(vE == m) && ((vSE == m) ||
                                                    (!(vS == m) && ((vSW == m) || (!(vW == m)))))));
                        nv = raise_from(m, min_slope, diag ? Ld : L);
                    }
                    if (nv < own[j][k])
                    {
                        own[j][k] = nv;
                        sF[lr][lc] = nv;
                        local = true;
                    }
                }
            }
            }
            if (k < 3) __syncthreads();
        }
        if (!__syncthreads_or(local)) break;
        tile_changed = true;
    }
#pragma unroll
    for (int j = 0; j < kFillBlocks; ++j)
    {
        const int b = tid + j * kFillThreads, bx = b % (kT / 2), by = b / (kT / 2);
#pragma unroll
        for (int k = 0; k < 4; ++k)
        {
            if (!((free_mask >> (4 * j + k)) & 1u)) continue;
            const int lr = 2 * by + 1 + (k >> 1), lc = 2 * bx + 1 + (k & 1);
            const std::int64_t g = static_cast<std::int64_t>(r0 + lr) * nc + (c0 + lc);
            if (own[j][k] < F[g]) F[g] = own[j][k];
        }
    }
    if (tid == 0)
    {
        dirty_out[ty * ntx + tx] = tile_changed ? 1 : 0;
        if (tile_changed) atomicOr(changed, 1);
    }
}


}  // namespace
}  // namespace lsdtt_gb300
