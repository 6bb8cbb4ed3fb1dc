// d8_cell.cuh -- the per-cell D8 receiver rule, shared by the single-grid
// kernel (d8.cu) and the packed ensemble kernel (ensemble.cu).
//
// Restates build_receiver_graph_d8 (src/cpu/lsdtt_flowinfo_cpu.cpp:
// 1077-1329): for each valid cell the steepest downhill neighbour, slope
// (double)z - (double)z_nb over dx or dx*sqrt(2) in double, strict '>' so the
// first of equal slopes in direction order 0..7 wins. The ranking avoids FP64
// division (see the comparison below); the result is the reference's bit for
// bit.
#pragma once

#include "common.cuh"

namespace lsdtt_gb300
{
namespace
{

constexpr unsigned kErrUnresolved = 4;

struct Cand
{
    float best;
    float second;
    int dir;
    std::int64_t rec;
};

// Exact reference evaluation for one cell (used for near-ties and for the
// cells whose float ranking is ambiguous).
__device__ void exact_receiver(const Grid& g, const float* __restrict__ z, const std::uint8_t* __restrict__ mask,
                               int row, int col, int& out_dir, std::int64_t& out_rec, bool& allowed_outlet,
                               int interior_nodata_is_outlet)
{
    const std::int64_t flat = static_cast<std::int64_t>(row) * g.nc + col;
    const double card = g.cell;
    const double diag = g.cell * 1.4142135623730950488;
    const float zc = z[flat];
    double best = 0.0;
    out_dir = kNoDir;
    out_rec = kOutletReceiver;
    allowed_outlet = false;
    for (int d = 0; d < 8; ++d)
    {
        const Step s = resolve_step(g, row, col, d);
        if (s.kind == 2) { allowed_outlet = true; continue; }
        if (s.kind == 0) continue;
        const std::int64_t nf = static_cast<std::int64_t>(s.r) * g.nc + s.c;
        if (mask[nf] == 0)
        {
            if (interior_nodata_is_outlet) allowed_outlet = true;
            continue;
        }
        if (nf == flat) continue;
        const double dz = static_cast<double>(zc) - static_cast<double>(z[nf]);
        if (dz <= 0.0) continue;
        const double slope = __ddiv_rn(dz, (d & 1) ? diag : card);
        if (slope > best)
        {
            best = slope;
            out_rec = nf;
            out_dir = d;
        }
    }
}

// The receiver of cell (row, col) of grid g; z, mask, forced, receiver and
// dir are that grid's planes. An unresolved sink records its flat index
// plus err_base in err[1].
__device__ __forceinline__ void d8_receiver_cell(const Grid& g, const float* __restrict__ z,
                                                 const std::uint8_t* __restrict__ mask,
                                                 const std::uint8_t* __restrict__ forced,
                                                 int interior_nodata_is_outlet, int allow_pits, float inv_card,
                                                 float inv_diag, std::int64_t* __restrict__ receiver,
                                                 std::uint8_t* __restrict__ dir, unsigned long long* __restrict__ err,
                                                 int row, int col, std::int64_t err_base = 0)
{
    const std::int64_t flat = static_cast<std::int64_t>(row) * g.nc + col;
    if (mask[flat] == 0)
    {
        receiver[flat] = kNodataReceiver;
        dir[flat] = kNoDir;
        return;
    }
    const bool forced_edge = (row == 0 && g.bc[0] == 'b') || (col == g.nc - 1 && g.bc[1] == 'b') ||
                             (row == g.nr - 1 && g.bc[2] == 'b') || (col == 0 && g.bc[3] == 'b');
    if (forced_edge || (forced != nullptr && forced[flat] != 0))
    {
        receiver[flat] = kOutletReceiver;
        dir[flat] = kNoDir;
        return;
    }
    const float zc = z[flat];
    // Rank per direction class. Within a class (cardinal or diagonal) every
    // slope shares one divisor, so the reference's double quotients order
    // exactly like the elevation drops; a drop z - z_nb computed in float is
    // exact whenever Sterbenz's lemma applies (z_nb > 0 and z - z_nb <= z_nb,
    // or the mirrored negative case), and the first of equal drops in
    // direction order wins, as the reference's strict '>' does.
    float bdz[2] = {0.0f, 0.0f};
    int bd[2] = {kNoDir, kNoDir};
    std::int64_t br[2] = {kOutletReceiver, kOutletReceiver};
    bool allowed_outlet = false;
    bool inexact = false;
    auto consider = [&](int d, std::int64_t nf) {
        const float zn = z[nf];
        if (!(zc > zn)) return;  // (double)zc - (double)zn <= 0
        const float dz = __fsub_rn(zc, zn);
        const bool exact = (zn > 0.0f && dz <= zn) || (zc < 0.0f && dz <= -zc) || zn == 0.0f || zc == 0.0f;
        inexact |= !exact;
        const int k = d & 1;
        if (dz > bdz[k]) { bdz[k] = dz; bd[k] = d; br[k] = nf; }
    };
    if (is_interior(g, row, col))
    {
#pragma unroll
        for (int d = 0; d < 8; ++d)
        {
            const std::int64_t nf = flat + static_cast<std::int64_t>(d8_dr(d)) * g.nc + d8_dc(d);
            if (mask[nf] == 0)
            {
                if (interior_nodata_is_outlet) allowed_outlet = true;
                continue;
            }
            consider(d, nf);
        }
    }
    else
    {
        for (int d = 0; d < 8; ++d)
        {
            const Step st = resolve_step(g, row, col, d);
            if (st.kind == 2) { allowed_outlet = true; continue; }
            if (st.kind == 0) continue;
            const std::int64_t nf = static_cast<std::int64_t>(st.r) * g.nc + st.c;
            if (mask[nf] == 0)
            {
                if (interior_nodata_is_outlet) allowed_outlet = true;
                continue;
            }
            if (nf == flat) continue;
            consider(d, nf);
        }
    }
    int bdir = kNoDir;
    std::int64_t brec = kOutletReceiver;
    if (inexact)
        exact_receiver(g, z, mask, row, col, bdir, brec, allowed_outlet, interior_nodata_is_outlet);
    else if (bd[0] == kNoDir || bd[1] == kNoDir)
    {
        const int k = (bd[0] != kNoDir) ? 0 : 1;
        bdir = bd[k];
        brec = br[k];
    }
    else
    {
        // Cardinal vs diagonal: q_c = dz_c / dx against q_d = dz_d / (dx*sqrt2).
        // A float screen settles clear cases; otherwise compare dz_c*Ld with
        // dz_d*dx in double. For 24-bit drops the exact quotients cannot be
        // closer than ~2^-50 relative (sqrt2 is badly approximable:
        // |sqrt2 - p/q| > 1/(4 q^2)), so the products decide the reference's
        // rounded comparison; a residual near-tie takes the division path.
        const float sc = bdz[0] * inv_card, sd = bdz[1] * inv_diag;
        int win;
        if (sc > sd * (1.0f + 3.814697265625e-06f)) win = 0;
        else if (sd > sc * (1.0f + 3.814697265625e-06f)) win = 1;
        else
        {
            const double A = __dmul_rn(static_cast<double>(bdz[0]), g.cell * 1.4142135623730950488);
            const double B = __dmul_rn(static_cast<double>(bdz[1]), g.cell);
            const double gap = fabs(A - B);
            if (gap > 8.881784197001252e-16 * fmax(A, B)) win = (A > B) ? 0 : 1;  // 2^-50
            else win = -1;
        }
        if (win >= 0)
        {
            bdir = bd[win];
            brec = br[win];
        }
        else
            exact_receiver(g, z, mask, row, col, bdir, brec, allowed_outlet, interior_nodata_is_outlet);
    }
    if (bdir != kNoDir)
    {
        receiver[flat] = brec;
        dir[flat] = static_cast<std::uint8_t>(bdir);
        return;
    }
    receiver[flat] = kOutletReceiver;
    dir[flat] = kNoDir;
    if (!allowed_outlet && !allow_pits)
    {
        // Lexicographically first unresolved cell, as the reference reports.
        atomicMin(err + 1, static_cast<unsigned long long>(flat + err_base));
        raise_error(err, kErrUnresolved, 0);
    }
}


}  // namespace
}  // namespace lsdtt_gb300
