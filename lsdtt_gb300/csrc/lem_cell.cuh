// lem_cell.cuh -- per-cell LEM rules shared by the single-grid step
// (lem.cu) and the packed ensemble (ensemble.cu).
#pragma once

#include "common.cuh"

namespace lsdtt_gb300
{
namespace
{

// build_boundary_flats (src/cpu/lsdtt_lem_cpu.cpp:735-808): valid cells with
// an off-grid neighbour across a fixed ('o'/'b') edge, or a masked in-grid
// neighbour in a direction whose edge is fixed. Cell i of an nr x nc grid.
__device__ __forceinline__ bool boundary_flat_cell(int nr, int nc, const char* bc4, const std::uint8_t* __restrict__ mask,
                                                   std::int64_t i)
{
    if (!mask[i]) return false;
    const bool fn = bc4[0] == 'o' || bc4[0] == 'b', fe = bc4[1] == 'o' || bc4[1] == 'b';
    const bool fs = bc4[2] == 'o' || bc4[2] == 'b', fw = bc4[3] == 'o' || bc4[3] == 'b';
    const int r = static_cast<int>(i / nc), c = static_cast<int>(i % nc);
    bool edge = false;
    for (int dr = -1; dr <= 1 && !edge; ++dr)
        for (int dc = -1; dc <= 1; ++dc)
        {
            if (dr == 0 && dc == 0) continue;
            const int r2 = r + dr, c2 = c + dc;
            if (r2 < 0) { if (fn) edge = true; }
            else if (r2 >= nr) { if (fs) edge = true; }
            else if (c2 < 0) { if (fw) edge = true; }
            else if (c2 >= nc) { if (fe) edge = true; }
            else if (!mask[static_cast<std::int64_t>(r2) * nc + c2])
            {
                if ((dr == -1 && fn) || (dr == 1 && fs) || (dc == -1 && fw) || (dc == 1 && fe)) edge = true;
            }
        }
    return edge;
}

}  // namespace
}  // namespace lsdtt_gb300
