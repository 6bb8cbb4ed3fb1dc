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

constexpr int kT = 32;        // tile edge (cells)
constexpr int kH = kT + 2;    // with halo
constexpr int kMaxLocal = 4 * kT;

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
// hold z and are fixed, other valid cells +inf, invalid cells hold the nodata
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
    F[i] = seed ? z[i] : INFINITY;
    kind[i] = seed ? 2 : 1;  // 2 seed (fixed), 1 free
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
// run by one 32 x 8 thread block. dirty_in / dirty_out are the grid's
// per-tile activity planes (ntx * nty entries).
__device__ __forceinline__ void fill_relax_tile(int nr, int nc, bool per_ns, bool per_ew, float L, float Ld,
                                                float min_slope, const float* __restrict__ z,
                                                const std::uint8_t* __restrict__ kind, float* __restrict__ F,
                                                int* __restrict__ changed, const std::uint8_t* __restrict__ dirty_in,
                                                std::uint8_t* __restrict__ dirty_out, const int tx, const int ty,
                                                const int ntx, const int nty)
{
    // Active-tile gate: a tile can only change if it or one of its eight
    // neighbouring tiles changed in the previous pass (periodic axes wrap).
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
    __shared__ float sF[kH][kH];
    __shared__ float sz[kH][kH];
    __shared__ std::uint8_t sk[kH][kH];
    __shared__ int any;
    const int r0 = ty * kT - 1, c0 = tx * kT - 1;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (int k = tid; k < kH * kH; k += blockDim.x * blockDim.y)
    {
        const int lr = k / kH, lc = k % kH;
        int r = r0 + lr, c = c0 + lc;
        if (per_ns) { if (r < 0) r += nr; else if (r >= nr) r -= nr; }
        if (per_ew) { if (c < 0) c += nc; else if (c >= nc) c -= nc; }
        if (r >= 0 && r < nr && c >= 0 && c < nc)
        {
            const std::int64_t g = static_cast<std::int64_t>(r) * nc + c;
            sF[lr][lc] = F[g];
            sz[lr][lc] = z[g];
            sk[lr][lc] = kind[g];
        }
        else
        {
            sF[lr][lc] = INFINITY;
            sz[lr][lc] = INFINITY;
            sk[lr][lc] = 0;
        }
    }
    if (tid == 0) any = 0;
    __syncthreads();
    // Interior cells of this tile owned by this thread: 32 columns x 4 rows.
    const int lc = threadIdx.x + 1;
    bool tile_changed = false;
    for (int it = 0; it < kMaxLocal; ++it)
    {
        bool local = false;
#pragma unroll
        for (int q = 0; q < kT / 8; ++q)
        {
            const int lr = threadIdx.y * (kT / 8) + q + 1;
            const int r = r0 + lr, c = c0 + lc;
            if (r >= nr || c >= nc || sk[lr][lc] != 1) continue;
            float m = INFINITY;
            int md = -1;
#pragma unroll
            // The halo load already resolved every neighbour: periodic axes
            // are wrapped into the tile and off-grid positions hold kind 0.
            for (int d = 0; d < 8; ++d)
            {
                const int ar = lr + d8_dr(d), ac = lc + d8_dc(d);
                if (sk[ar][ac] == 0) continue;
                const float v = sF[ar][ac];
                if (v < m) { m = v; md = d; }
            }
            if (md < 0) continue;
            const float zc = sz[lr][lc];
            const float nv = (zc > m) ? zc : raise_from(m, min_slope, (md & 1) ? Ld : L);
            if (nv < sF[lr][lc])
            {
                sF[lr][lc] = nv;
                local = true;
            }
        }
        __syncthreads();
        if (local) any = 1;
        __syncthreads();
        const int a = any;
        __syncthreads();
        if (!a) break;
        tile_changed = true;
        if (tid == 0) any = 0;
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < kT / 8; ++q)
    {
        const int lr = threadIdx.y * (kT / 8) + q + 1;
        const int r = r0 + lr, c = c0 + lc;
        if (r >= nr || c >= nc || sk[lr][lc] != 1) continue;
        const std::int64_t g = static_cast<std::int64_t>(r) * nc + c;
        if (sF[lr][lc] < F[g]) F[g] = sF[lr][lc];
    }
    if (tid == 0)
    {
        dirty_out[ty * ntx + tx] = tile_changed ? 1 : 0;
        if (tile_changed) atomicOr(changed, 1);
    }
}


}  // namespace
}  // namespace lsdtt_gb300
