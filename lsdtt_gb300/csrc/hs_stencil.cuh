// hs_stencil.cuh -- the hillslope operator's neighbour rules, shared by
// the single-grid solvers (hillslope.cu) and the packed ensemble
// (ensemble.cu). lsdtt_hillslope_domain::neighbour
// (src/cpu/lsdtt_hillslope_operator_cpu.hpp:163-175): 'p' wraps, every other
// edge and every masked neighbour resolves to the cell itself (zero flux).
#pragma once

#include "common.cuh"

namespace lsdtt_gb300
{
namespace
{

struct Hs
{
    int nr, nc;
    char bn, be, bs, bw;
    double DA;      // D / h^2
    double inv_dt;
    double U;
};

__device__ __forceinline__ bool hs_valid(const std::uint8_t* mask, int nc, int r, int c)
{
    return mask[static_cast<std::int64_t>(r) * nc + c] != 0;
}

// lsdtt_hillslope_domain::neighbour (operator_cpu.hpp:163-175)
__device__ __forceinline__ std::int64_t hs_nb(const Hs& H, const std::uint8_t* mask, int r, int c, int dr, int dc)
{
    int rr = r + dr, cc = c + dc;
    if (rr < 0) rr = (H.bn == 'p') ? H.nr - 1 : r;
    else if (rr >= H.nr) rr = (H.bs == 'p') ? 0 : r;
    if (cc < 0) cc = (H.bw == 'p') ? H.nc - 1 : c;
    else if (cc >= H.nc) cc = (H.be == 'p') ? 0 : c;
    if (!hs_valid(mask, H.nc, rr, cc)) { rr = r; cc = c; }
    return static_cast<std::int64_t>(rr) * H.nc + cc;
}

__device__ __forceinline__ bool hs_dirichlet_edge(const Hs& H, int r, int c)
{
    return (r == 0 && H.bn == 'o') || (r == H.nr - 1 && H.bs == 'o') || (c == 0 && H.bw == 'o') ||
           (c == H.nc - 1 && H.be == 'o');
}

__device__ constexpr int kDr[4] = {-1, 0, 1, 0};  // N, E, S, W
__device__ constexpr int kDc[4] = {0, 1, 0, -1};

}  // namespace
}  // namespace lsdtt_gb300
