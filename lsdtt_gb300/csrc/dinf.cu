// dinf.cu -- the D-infinity flow graph and D-infinity stream power on the GPU.
//
// Reference: lsdtt_flowgraph_cpu with method = d_infinity
// (src/cpu/lsdtt_flowgraph_cpu.cpp:87-178 constructor, :423-662 build_dinf
// after Tarboton 1997, :874-985 donor counts and topological order,
// :988-1039 accumulate) and compute_dinf_stream_power_incision
// (src/cpu/lsdtt_stream_power_cpu.cpp:329-602).
//
// * Graph: one thread per cell evaluates the eight triangular facets with
//   the reference's float arithmetic (the in-facet angle is the double
//   atan2 rounded to float) and keeps up to two receivers with their
//   weights, the facet slope and the bearing.
// * Topological order: the reference's Kahn FIFO, exactly. Its queue is the
//   cells grouped by height (longest path from a source), sources in
//   row-major order, and within height k + 1 ordered by the queue position
//   of each cell's last donor (a height-k donor) and then by which of that
//   donor's two edges it is. Height by height, every height-k cell stamps
//   its receivers with (its position, edge) by atomic maximum and counts
//   them down; a receiver whose count reaches zero is ready, and the ready
//   cells are placed by their stamp (stamps are unique per height) and
//   compacted. One round per height.
// * Accumulate: heights in ascending order; each cell adds its donors'
//   shares in their topological order, the reference's additions in its
//   order.
// * Stream power: heights in descending order (every receiver is higher
//   than its donors), each node the reference's update; any receiver-
//   before-donor order gives its bits.
//
// Every array is allocated at create() for the grid and reused by build().

#include <cmath>
#include <string>
#include <vector>

#include "engine.cuh"
#include "sp_node.cuh"

struct lsdtt_gpu_dinf
{
    lsdtt_gb300::Grid g{};
    std::int64_t* rec = nullptr;     // [2n] receivers, -1 none
    float* w = nullptr;              // [2n] weights
    std::uint8_t* nrec = nullptr;    // [n]
    float* slope = nullptr;          // [n]
    float* bearing = nullptr;        // [n]
    std::uint8_t* valid = nullptr;   // [n]
    std::uint8_t* donors = nullptr;  // [n]
    std::uint32_t* remaining = nullptr;          // [n] Kahn counters
    unsigned long long* stamp = nullptr;         // [n] (round, position, edge) of the last donor
    std::int32_t* level = nullptr;               // [n] height
    std::int64_t* pos = nullptr;                 // [n] position in the topological order
    std::int64_t* topo = nullptr;                // [n] the topological order
    std::int64_t* slots = nullptr;               // [2n + 2] placement of one height's ready cells
    std::uint32_t* next = nullptr;               // [n] ready cells of a round (unordered)
    std::uint32_t* cnt = nullptr;                // [4] device counters
    std::uint32_t* hcnt = nullptr;               // pinned mirror
    std::int64_t* scan_tmp = nullptr;            // [2n + 2]
    double* area = nullptr;                      // [n] accumulate() of the default weights
    float* zbuf = nullptr;                       // [n] stream-power working surface
    lsdtt_gb300::Scratch ws{};
    std::vector<std::int64_t> level_start;       // host: offsets of each height in topo
    std::int64_t n_valid = 0;
    bool built = false;
};

namespace lsdtt_gb300
{
namespace
{

// Tarboton's eight facets (flowgraph_cpu.cpp:60-67): cardinal neighbour e1,
// diagonal neighbour e2, and the sector and sign of the bearing.
__constant__ int kE1r[8] = {0, -1, -1, 0, 0, 1, 1, 0};
__constant__ int kE1c[8] = {1, 0, 0, -1, -1, 0, 0, 1};
__constant__ int kE2r[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
__constant__ int kE2c[8] = {1, 1, -1, -1, -1, -1, 1, 1};
__constant__ int kAc[8] = {0, 1, 1, 2, 2, 3, 3, 4};
__constant__ int kAf[8] = {1, -1, 1, -1, 1, -1, 1, -1};

__device__ __forceinline__ bool dinf_resolve(const Grid& g, int r, int c, int dr, int dc, int& rr, int& cc)
{
    rr = r + dr;
    cc = c + dc;
    if (rr < 0) { if (g.bc[0] == 'p') rr = g.nr - 1; else return false; }
    if (rr >= g.nr) { if (g.bc[2] == 'p') rr = 0; else return false; }
    if (cc < 0) { if (g.bc[3] == 'p') cc = g.nc - 1; else return false; }
    if (cc >= g.nc) { if (g.bc[1] == 'p') cc = 0; else return false; }
    return true;
}

__global__ void dinf_valid(Grid g, const float* __restrict__ z, const std::uint8_t* __restrict__ mask,
                           std::uint8_t* __restrict__ valid)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    const float ndv = static_cast<float>(g.nodata);
    valid[i] = (mask[i] != 0 && z[i] != ndv && isfinite(z[i])) ? 1 : 0;
}

// build_dinf (flowgraph_cpu.cpp:423-662) for one cell.
__global__ void dinf_facets(Grid g, const float* __restrict__ z, const std::uint8_t* __restrict__ valid,
                            int interior_nodata_is_outlet, std::int64_t* __restrict__ rec, float* __restrict__ w,
                            std::uint8_t* __restrict__ nrec, float* __restrict__ slope, float* __restrict__ bearing)
{
    LSDTT_COUNT();
    const std::int64_t f = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (f >= g.n) return;
    const float ndv = static_cast<float>(g.nodata);
    rec[2 * f] = -1;
    rec[2 * f + 1] = -1;
    w[2 * f] = 0.0f;
    w[2 * f + 1] = 0.0f;
    nrec[f] = 0;
    slope[f] = ndv;
    bearing[f] = ndv;
    if (!valid[f]) return;
    const int r = static_cast<int>(f / g.nc), c = static_cast<int>(f % g.nc);
    const bool forced = (g.bc[0] == 'b' && r == 0) || (g.bc[2] == 'b' && r == g.nr - 1) ||
                        (g.bc[1] == 'b' && c == g.nc - 1) || (g.bc[3] == 'b' && c == 0);
    if (forced) return;
    if (interior_nodata_is_outlet)
        for (int k = 0; k < 8; ++k)
        {
            const int rr = r + d8_dr(k), cc = c + d8_dc(k);
            if (rr < 0 || rr >= g.nr || cc < 0 || cc >= g.nc) continue;
            if (!valid[static_cast<std::int64_t>(rr) * g.nc + cc]) return;  // touches interior nodata: an outlet
        }
    const float pi4 = static_cast<float>(M_PI / 4.0);
    const float L = static_cast<float>(g.cell);
    const float Ld = __fmul_rn(L, static_cast<float>(1.4142135623730950488));
    const float e0 = z[f];
    float best_s = 0.0f, best_r = 0.0f;
    int best = -1;
    std::int64_t b1 = -1, b2 = -1;
    for (int a = 0; a < 8; ++a)
    {
        int r1, c1, r2, c2;
        if (!dinf_resolve(g, r, c, kE1r[a], kE1c[a], r1, c1) || !dinf_resolve(g, r, c, kE2r[a], kE2c[a], r2, c2))
            continue;
        const std::int64_t f1 = static_cast<std::int64_t>(r1) * g.nc + c1;
        const std::int64_t f2 = static_cast<std::int64_t>(r2) * g.nc + c2;
        if (f1 == f || f2 == f) continue;
        if (!valid[f1] || !valid[f2]) continue;
        const float e1 = z[f1], e2 = z[f2];
        if (e0 <= e1 && e0 <= e2) continue;
        float rr, ss;
        const float s1 = __fdiv_rn(__fsub_rn(e0, e1), L);
        const float s2 = __fdiv_rn(__fsub_rn(e1, e2), L);
        if (e0 > e1 && e0 > e2)
        {
            rr = static_cast<float>(atan2(static_cast<double>(s2), static_cast<double>(s1)));
            if (rr < 0.0f) { rr = 0.0f; ss = s1; }
            else if (rr > pi4) { rr = pi4; ss = __fdiv_rn(__fsub_rn(e0, e2), Ld); }
            else ss = __fsqrt_rn(__fadd_rn(__fmul_rn(s1, s1), __fmul_rn(s2, s2)));
        }
        else if (e0 > e1) { rr = 0.0f; ss = s1; }
        else { rr = pi4; ss = __fdiv_rn(__fsub_rn(e0, e2), Ld); }
        if (ss > best_s) { best_s = ss; best_r = rr; best = a; b1 = f1; b2 = f2; }
    }
    if (best < 0) return;
    const float ang = __fadd_rn(__fmul_rn(static_cast<float>(kAf[best]), best_r),
                                __fmul_rn(static_cast<float>(kAc[best]), __fmul_rn(static_cast<float>(M_PI), 0.5f)));
    float b = __fadd_rn(__fsub_rn(360.0f, __fmul_rn(ang, static_cast<float>(180.0 / M_PI))), 90.0f);
    while (b >= 360.0f) b = __fsub_rn(b, 360.0f);
    while (b < 0.0f) b = __fadd_rn(b, 360.0f);
    slope[f] = best_s;
    bearing[f] = b;
    if (best_r == 0.0f || (best_r < pi4 && b1 == b2))
    {
        nrec[f] = 1;
        rec[2 * f] = b1;
        w[2 * f] = 1.0f;
    }
    else if (best_r >= pi4)
    {
        nrec[f] = 1;
        rec[2 * f] = b2;
        w[2 * f] = 1.0f;
    }
    else
    {
        const float p2 = __fdiv_rn(best_r, pi4);
        nrec[f] = 2;
        rec[2 * f] = b1;
        w[2 * f] = __fsub_rn(1.0f, p2);
        rec[2 * f + 1] = b2;
        w[2 * f + 1] = p2;
    }
}

// Unique donors (counted as the reference counts them, capped at 255) and
// the Kahn counters (one per incoming edge).
__global__ void dinf_count(std::int64_t n, const std::int64_t* __restrict__ rec, const std::uint8_t* __restrict__ nrec,
                           std::uint32_t* __restrict__ remaining)
{
    LSDTT_COUNT();
    const std::int64_t f = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (f >= n) return;
    for (int k = 0; k < nrec[f]; ++k) atomicAdd(remaining + rec[2 * f + k], 1u);
}

__global__ void dinf_donors(std::int64_t n, const std::uint32_t* __restrict__ remaining,
                            std::uint8_t* __restrict__ donors)
{
    LSDTT_COUNT();
    const std::int64_t f = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (f >= n) return;
    donors[f] = static_cast<std::uint8_t>(remaining[f] < 255u ? remaining[f] : 255u);
}

// Sources (valid cells without donors) flagged into slots[f] for the
// row-major compaction of height 0.
__global__ void dinf_sources(std::int64_t n, const std::uint8_t* __restrict__ valid,
                             const std::uint32_t* __restrict__ remaining, std::int64_t* __restrict__ slots)
{
    LSDTT_COUNT();
    const std::int64_t f = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (f >= n) return;
    slots[f] = (valid[f] && remaining[f] == 0) ? f : -1;
}

__global__ void slot_flags(std::int64_t m, const std::int64_t* __restrict__ slots, std::uint8_t* __restrict__ flag)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < m) flag[i] = slots[i] >= 0 ? 1 : 0;
}

// Compaction of the placed cells of a height into the topological order at
// `base`, with their positions and heights.
__global__ void slot_compact(std::int64_t m, const std::int64_t* __restrict__ slots,
                             const std::int64_t* __restrict__ at, std::int64_t base, int lvl,
                             std::int64_t* __restrict__ topo, std::int64_t* __restrict__ pos,
                             std::int32_t* __restrict__ level)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= m || slots[i] < 0) return;
    const std::int64_t f = slots[i];
    const std::int64_t p = base + at[i];
    topo[p] = f;
    pos[f] = p;
    level[f] = lvl;
}

// One round of Kahn's order: every cell of the height [lo, hi) stamps and
// counts down its receivers; a receiver reaching zero is ready (appended,
// unordered).
__global__ void dinf_round(const std::int64_t* __restrict__ topo, std::int64_t lo, std::int64_t hi, int round,
                           const std::int64_t* __restrict__ rec, const std::uint8_t* __restrict__ nrec,
                           unsigned long long* __restrict__ stamp, std::uint32_t* __restrict__ remaining,
                           std::uint32_t* __restrict__ next, std::uint32_t* __restrict__ cnt)
{
    LSDTT_COUNT();
    const std::int64_t i = lo + static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= hi) return;
    const std::int64_t f = topo[i];
    const unsigned long long p = static_cast<unsigned long long>(i - lo);
    for (int k = 0; k < nrec[f]; ++k)
    {
        const std::int64_t r = rec[2 * f + k];
        atomicMax(stamp + r, (static_cast<unsigned long long>(round) << 40) | (p << 1) | static_cast<unsigned>(k));
        if (atomicSub(remaining + r, 1u) == 1u) next[atomicAdd(cnt, 1u)] = static_cast<std::uint32_t>(r);
    }
}

// The ready cells placed by their last donor's (position, edge).
__global__ void dinf_place(std::uint32_t m, const std::uint32_t* __restrict__ next,
                           const unsigned long long* __restrict__ stamp, std::int64_t* __restrict__ slots)
{
    LSDTT_COUNT();
    const std::uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const std::uint32_t r = next[i];
    slots[stamp[r] & ((1ull << 40) - 1ull)] = r;
}

__global__ void fill_i64(std::int64_t m, std::int64_t* __restrict__ a, std::int64_t v)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < m) a[i] = v;
}

// ---- accumulate --------------------------------------------------------------
// Seed of every valid cell (the default dx^2 or its weight).
__global__ void dinf_acc_seed(std::int64_t n, const std::uint8_t* __restrict__ valid, const double* __restrict__ wts,
                              double dw, double* __restrict__ acc)
{
    LSDTT_COUNT();
    const std::int64_t f = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (f >= n) return;
    acc[f] = valid[f] ? (wts ? wts[f] : dw) : 0.0;
}

// Cells of one height gather their donors' shares in the donors' order.
__global__ void dinf_acc_level(Grid g, const std::int64_t* __restrict__ topo, std::int64_t lo, std::int64_t hi,
                               const std::int64_t* __restrict__ rec, const float* __restrict__ w,
                               const std::uint8_t* __restrict__ nrec, const std::int64_t* __restrict__ pos,
                               double* __restrict__ acc)
{
    LSDTT_COUNT();
    const std::int64_t i = lo + static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= hi) return;
    const std::int64_t c = topo[i];
    const int row = static_cast<int>(c / g.nc), col = static_cast<int>(c % g.nc);
    std::int64_t dn[8];
    float dw[8];
    int k = 0;
    for (int dr = -1; dr <= 1; ++dr)
        for (int dc = -1; dc <= 1; ++dc)
        {
            if (!dr && !dc) continue;
            int rr, cc;
            if (!dinf_resolve(g, row, col, dr, dc, rr, cc)) continue;
            const std::int64_t d = static_cast<std::int64_t>(rr) * g.nc + cc;
            if (d == c) continue;
            bool dup = false;
            for (int j = 0; j < k; ++j) dup |= dn[j] == d;
            if (dup) continue;
            for (int e = 0; e < nrec[d]; ++e)
                if (rec[2 * d + e] == c)
                {
                    dn[k] = d;
                    dw[k] = w[2 * d + e];
                    ++k;
                    break;
                }
        }
    // donors by topological position
    for (int a = 1; a < k; ++a)
    {
        const std::int64_t d = dn[a];
        const float ww = dw[a];
        int b = a - 1;
        while (b >= 0 && pos[dn[b]] > pos[d])
        {
            dn[b + 1] = dn[b];
            dw[b + 1] = dw[b];
            --b;
        }
        dn[b + 1] = d;
        dw[b + 1] = ww;
    }
    double a = acc[c];
    for (int j = 0; j < k; ++j) a = __dadd_rn(a, __dmul_rn(acc[dn[j]], static_cast<double>(dw[j])));
    acc[c] = a;
}

// ---- stream power ------------------------------------------------------------
struct DinfSp
{
    SpParams sp;
    const std::int64_t* rec;
    const float* w;
    const std::uint8_t* nrec;
    const std::uint8_t* valid;
    const double* area;
    const float* z_old;
    float* z;
    std::int64_t n;
};

// compute_dinf_stream_power_incision (stream_power_cpu.cpp:329-602) for one
// node whose receivers are final.
__device__ void dinf_sp_node(const DinfSp& A, std::int64_t f)
{
    if (!A.valid[f] || A.nrec[f] == 0) return;
    const SpParams& P = A.sp;
    double area = A.area[f];
    if (P.divide_by_dx) area = __ddiv_rn(area, static_cast<double>(P.dx));
    if (P.threshold > 0.0f && area < static_cast<double>(P.threshold)) return;
    const float zo = A.z_old[f];
    float zn = zo;
    const int nr = A.nrec[f];
    const float w0 = nr > 0 ? A.w[2 * f] : 0.0f;
    const float w1 = nr > 1 ? A.w[2 * f + 1] : 0.0f;
    const bool only_card = nr == 1 || w0 >= 1.0f - 1e-6f;
    const bool only_diag = nr > 1 && w1 >= 1.0f - 1e-6f;
    const bool two = nr > 1 && !only_card && !only_diag;
    auto recv = [&](int k) -> float {
        if (k >= nr) return zo;
        const std::int64_t i = A.rec[2 * f + k];
        if (i < 0 || i >= A.n) return zo;
        return __ldcg(A.z + i);
    };
    const float ze1 = recv(0), ze2 = recv(1);
    const double kam = __dmul_rn(__dmul_rn(static_cast<double>(P.K), 1.0), pow(area, static_cast<double>(P.m)));
    const float dxc = P.dx;
    const double tol = __dmul_rn(static_cast<double>(P.slope_clamp), static_cast<double>(dxc));
    const double nd = static_cast<double>(P.n);
    if (two)
    {
        double eps = tol + 1.0;
        int it = 0;
        do
        {
            const double a1 = static_cast<double>(__fdiv_rn(__fsub_rn(ze1, zn), dxc));
            const double a2 = static_cast<double>(__fdiv_rn(__fsub_rn(ze2, ze1), dxc));
            const double sbt = __dadd_rn(__dmul_rn(a1, a1), __dmul_rn(a2, a2));
            if (sbt <= 0.0) eps = 0.0;
            else
            {
                const double fz = __dadd_rn(static_cast<double>(__fsub_rn(zn, zo)),
                                            __dmul_rn(__dmul_rn(kam, pow(sbt, __dmul_rn(0.5, nd))),
                                                      static_cast<double>(P.dt)));
                const double t = __ddiv_rn(__dmul_rn(__dmul_rn(kam, nd), static_cast<double>(__fsub_rn(ze1, zn))),
                                           static_cast<double>(__fmul_rn(dxc, dxc)));
                const double fdz = __dsub_rn(
                    1.0, __dmul_rn(__dmul_rn(t, pow(sbt, __dsub_rn(__dmul_rn(0.5, nd), 1.0))), static_cast<double>(P.dt)));
                eps = __ddiv_rn(fz, fdz);
            }
            zn = __fsub_rn(zn, static_cast<float>(eps));
            ++it;
            if (it > 100) eps = tol / 2.0;
        } while (fabs(eps) > tol);
        if (__fsub_rn(zn, zo) > static_cast<float>(tol) || isnan(zn)) zn = zo;
        const float zmin = fminf(ze1, ze2);
        if (zn < zmin) zn = __fadd_rn(zmin, __fmul_rn(P.slope_clamp, dxc));
    }
    else
    {
        const float zr = only_diag ? ze2 : ze1;
        zn = sp_solve_tol(P, only_diag, kam, zo, zr, dxc);
    }
    A.z[f] = zn;
}

__global__ void dinf_sp_level(DinfSp A, const std::int64_t* __restrict__ topo, std::int64_t lo, std::int64_t hi)
{
    LSDTT_COUNT();
    for (std::int64_t i = lo + static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < hi;
         i += static_cast<std::int64_t>(gridDim.x) * blockDim.x)
        dinf_sp_node(A, topo[i]);
}

__global__ void copy_f32(std::int64_t n, const float* __restrict__ a, float* __restrict__ b)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) b[i] = a[i];
}

void free_dinf(lsdtt_gpu_dinf* D)
{
    if (!D) return;
    cudaFree(D->rec);
    cudaFree(D->w);
    cudaFree(D->nrec);
    cudaFree(D->slope);
    cudaFree(D->bearing);
    cudaFree(D->valid);
    cudaFree(D->donors);
    cudaFree(D->remaining);
    cudaFree(D->stamp);
    cudaFree(D->level);
    cudaFree(D->pos);
    cudaFree(D->topo);
    cudaFree(D->slots);
    cudaFree(D->next);
    cudaFree(D->cnt);
    cudaFreeHost(D->hcnt);
    cudaFree(D->scan_tmp);
    cudaFree(D->area);
    cudaFree(D->zbuf);
    cudaFree(D->ws.base);
    delete D;
}

// Default-weight accumulate into out.
cudaError_t dinf_accumulate(lsdtt_gpu_dinf* D, const double* wts, double* out, cudaStream_t st)
{
    const std::int64_t n = D->g.n;
    dinf_acc_seed<<<grid_blocks(n, 256), 256, 0, st>>>(n, D->valid, wts, D->g.cell * D->g.cell, out);
    const std::size_t L = D->level_start.size() - 1;
    for (std::size_t k = 1; k < L; ++k)
    {
        const std::int64_t lo = D->level_start[k], hi = D->level_start[k + 1];
        dinf_acc_level<<<grid_blocks(hi - lo, 256), 256, 0, st>>>(D->g, D->topo, lo, hi, D->rec, D->w, D->nrec,
                                                                  D->pos, out);
    }
    return cudaGetLastError();
}

}  // namespace
}  // namespace lsdtt_gb300

using namespace lsdtt_gb300;

extern "C" {

int lsdtt_gpu_dinf_create(const lsdtt_gpu_grid* grid, lsdtt_gpu_dinf** out)
{
    if (!out) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_dinf_create: out is null");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(LSDTT_GPU_ENODEV, "lsdtt_gpu_dinf_create: no CUDA device");
    if (!grid || !(grid->n_rows > 0 && grid->n_cols > 0 && grid->cell_size > 0.0))
        return fail(LSDTT_GPU_EINVAL, "lsdtt_flowgraph_cpu: raster metadata is invalid");
    char b[4];
    for (int i = 0; i < 4; ++i)
    {
        const char c = grid->boundary_conditions[i];
        b[i] = (c >= 'A' && c <= 'Z') ? static_cast<char>(c - 'A' + 'a') : c;
        if (b[i] != 'o' && b[i] != 'n' && b[i] != 'p' && b[i] != 'b')
            return fail(LSDTT_GPU_EINVAL, "lsdtt_flowgraph_cpu: boundary_conditions contains an invalid character. "
                                          "Allowed values are o, n, p, b.");
    }
    if ((b[0] == 'p') != (b[2] == 'p'))
        return fail(LSDTT_GPU_EINVAL, "lsdtt_flowgraph_cpu: north and south periodic boundary flags must match");
    if ((b[1] == 'p') != (b[3] == 'p'))
        return fail(LSDTT_GPU_EINVAL, "lsdtt_flowgraph_cpu: east and west periodic boundary flags must match");
    const std::int64_t n = static_cast<std::int64_t>(grid->n_rows) * grid->n_cols;
    if (n >= (std::int64_t(1) << 31)) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_dinf_create: grid too large");
    auto* D = new lsdtt_gpu_dinf();
    D->g.nr = grid->n_rows;
    D->g.nc = grid->n_cols;
    D->g.cell = grid->cell_size;
    D->g.nodata = grid->no_data_value;
    for (int i = 0; i < 4; ++i) D->g.bc[i] = b[i];
    D->g.n = n;
    const std::size_t un = static_cast<std::size_t>(n);
    cudaError_t e = cudaSuccess;
    auto al = [&](auto** p, std::size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(p), bytes);
    };
    al(&D->rec, sizeof(std::int64_t) * 2 * un);
    al(&D->w, sizeof(float) * 2 * un);
    al(&D->nrec, un);
    al(&D->slope, sizeof(float) * un);
    al(&D->bearing, sizeof(float) * un);
    al(&D->valid, un);
    al(&D->donors, un);
    al(&D->remaining, sizeof(std::uint32_t) * un);
    al(&D->stamp, sizeof(unsigned long long) * un);
    al(&D->level, sizeof(std::int32_t) * un);
    al(&D->pos, sizeof(std::int64_t) * un);
    al(&D->topo, sizeof(std::int64_t) * un);
    al(&D->slots, sizeof(std::int64_t) * (2 * un + 2));
    al(&D->next, sizeof(std::uint32_t) * un);
    al(&D->cnt, sizeof(std::uint32_t) * 4);
    al(&D->scan_tmp, sizeof(std::int64_t) * (2 * un + 2));
    al(&D->area, sizeof(double) * un);
    al(&D->zbuf, sizeof(float) * un);
    D->ws.cap = (2 * un + 2) * 2 + (std::size_t(16) << 20);
    al(&D->ws.base, D->ws.cap);
    if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&D->hcnt), sizeof(std::uint32_t) * 4);
    if (e != cudaSuccess)
    {
        free_dinf(D);
        return cuda_fail(e, "lsdtt_gpu_dinf_create");
    }
    *out = D;
    return LSDTT_GPU_OK;
}

int lsdtt_gpu_dinf_destroy(lsdtt_gpu_dinf* D)
{
    free_dinf(D);
    return LSDTT_GPU_OK;
}

int lsdtt_gpu_dinf_build(lsdtt_gpu_dinf* D, const float* z_dev, const std::uint8_t* mask_dev,
                         int32_t interior_nodata_is_outlet, void* stream)
{
    const char* who = "lsdtt_gpu_dinf_build";
    if (!D || !z_dev || !mask_dev) return fail(LSDTT_GPU_EINVAL, std::string(who) + ": null argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const std::int64_t n = D->g.n;
    const unsigned nb = grid_blocks(n, 256);
    D->built = false;
    dinf_valid<<<nb, 256, 0, st>>>(D->g, z_dev, mask_dev, D->valid);
    dinf_facets<<<nb, 256, 0, st>>>(D->g, z_dev, D->valid, interior_nodata_is_outlet ? 1 : 0, D->rec, D->w, D->nrec,
                                    D->slope, D->bearing);
    cudaMemsetAsync(D->remaining, 0, sizeof(std::uint32_t) * static_cast<std::size_t>(n), st);
    cudaMemsetAsync(D->stamp, 0, sizeof(unsigned long long) * static_cast<std::size_t>(n), st);
    dinf_count<<<nb, 256, 0, st>>>(n, D->rec, D->nrec, D->remaining);
    dinf_donors<<<nb, 256, 0, st>>>(n, D->remaining, D->donors);
    // Height 0: the sources in row-major order.
    std::uint8_t* flag = reinterpret_cast<std::uint8_t*>(D->ws.base);
    auto place = [&](std::int64_t m, std::int64_t base, int lvl, std::int64_t* placed) -> cudaError_t {
        slot_flags<<<grid_blocks(m, 256), 256, 0, st>>>(m, D->slots, flag);
        D->ws.used = (static_cast<std::size_t>(m) + 255) & ~std::size_t(255);
        cudaError_t pe = exclusive_scan<std::uint8_t, std::int64_t>(flag, m, D->scan_tmp, D->scan_tmp + m, D->ws, st);
        if (pe != cudaSuccess) return pe;
        slot_compact<<<grid_blocks(m, 256), 256, 0, st>>>(m, D->slots, D->scan_tmp, base, lvl, D->topo, D->pos,
                                                          D->level);
        pe = cudaMemcpyAsync(placed, D->scan_tmp + m, sizeof(std::int64_t), cudaMemcpyDeviceToHost, st);
        if (pe == cudaSuccess) pe = cudaStreamSynchronize(st);
        return pe;
    };
    dinf_sources<<<nb, 256, 0, st>>>(n, D->valid, D->remaining, D->slots);
    std::int64_t placed = 0;
    cudaError_t e = place(n, 0, 0, &placed);
    if (e != cudaSuccess) return cuda_fail(e, who);
    D->level_start.assign(1, 0);
    D->level_start.push_back(placed);
    std::int64_t total = placed;
    int round = 0;
    while (placed > 0)
    {
        const std::int64_t lo = D->level_start[static_cast<std::size_t>(round)], hi = lo + placed;
        cudaMemsetAsync(D->cnt, 0, sizeof(std::uint32_t), st);
        dinf_round<<<grid_blocks(placed, 256), 256, 0, st>>>(D->topo, lo, hi, round + 1, D->rec, D->nrec, D->stamp,
                                                             D->remaining, D->next, D->cnt);
        e = cudaMemcpyAsync(D->hcnt, D->cnt, sizeof(std::uint32_t), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return cuda_fail(e, who);
        const std::uint32_t ready = D->hcnt[0];
        if (ready == 0) break;
        const std::int64_t m = 2 * placed;
        fill_i64<<<grid_blocks(m, 256), 256, 0, st>>>(m, D->slots, -1);
        dinf_place<<<grid_blocks(ready, 256), 256, 0, st>>>(ready, D->next, D->stamp, D->slots);
        std::int64_t got = 0;
        e = place(m, hi, round + 1, &got);
        if (e != cudaSuccess) return cuda_fail(e, who);
        ++round;
        D->level_start.push_back(hi + got);
        total += got;
        placed = got;
    }
    if (D->level_start.back() == D->level_start[D->level_start.size() - 2] && D->level_start.size() > 2)
        D->level_start.pop_back();
    // The valid count the order must cover (the reference's cycle guard).
    std::vector<std::uint8_t> hv(static_cast<std::size_t>(n));
    e = cudaMemcpyAsync(hv.data(), D->valid, hv.size(), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, who);
    std::int64_t nv = 0;
    for (std::uint8_t v : hv) nv += v ? 1 : 0;
    D->n_valid = nv;
    if (total != nv)
        return fail(LSDTT_GPU_ECYCLIC, "lsdtt_flowgraph_cpu: cycle detected in receiver graph or inconsistent cell "
                                       "validity. Ensure the DEM is pit-filled and that valid cells have finite, "
                                       "non-nodata elevations.");
    e = dinf_accumulate(D, nullptr, D->area, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, who);
    D->built = true;
    return LSDTT_GPU_OK;
}

int lsdtt_gpu_dinf_get_view(const lsdtt_gpu_dinf* D, lsdtt_gpu_dinf_view* v)
{
    if (!D || !v) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_dinf_get_view: null argument");
    if (!D->built) return fail(LSDTT_GPU_ESTATE, "lsdtt_gpu_dinf_get_view: the graph is not built");
    v->receivers = D->rec;
    v->weights = D->w;
    v->n_receivers = D->nrec;
    v->slope = D->slope;
    v->bearing = D->bearing;
    v->donor_count = D->donors;
    v->topological_order = D->topo;
    v->n_cells = D->g.n;
    v->n_valid_cells = D->n_valid;
    v->n_levels = static_cast<int64_t>(D->level_start.size()) - 1;
    return LSDTT_GPU_OK;
}

int lsdtt_gpu_dinf_accumulate(lsdtt_gpu_dinf* D, const double* weights_dev, double* out_dev, void* stream)
{
    if (!D || !out_dev) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_dinf_accumulate: null argument");
    if (!D->built) return fail(LSDTT_GPU_ESTATE, "lsdtt_gpu_dinf_accumulate: the graph is not built");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = dinf_accumulate(D, weights_dev, out_dev, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? LSDTT_GPU_OK : cuda_fail(e, "lsdtt_gpu_dinf_accumulate");
}

int lsdtt_gpu_dinf_stream_power(lsdtt_gpu_dinf* D, const float* z_dev, float K, float m, float n, float dt,
                                float incision_threshold_area, int32_t divide_area_by_dx, float slope_clamp,
                                float* z_out_dev, void* stream)
{
    const char* who = "lsdtt_gpu_dinf_stream_power";
    if (!D || !z_dev || !z_out_dev) return fail(LSDTT_GPU_EINVAL, std::string(who) + ": null argument");
    if (!D->built) return fail(LSDTT_GPU_ESTATE, std::string(who) + ": the graph is not built");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const std::int64_t N = D->g.n;
    DinfSp A{};
    A.sp.K = K;
    A.sp.m = m;
    A.sp.n = n;
    A.sp.dt = dt;
    A.sp.threshold = incision_threshold_area;
    A.sp.slope_clamp = slope_clamp;
    A.sp.dx = static_cast<float>(D->g.cell);
    A.sp.dx_diag = static_cast<float>(D->g.cell) * static_cast<float>(1.4142135623730950488);
    A.sp.divide_by_dx = divide_area_by_dx ? 1 : 0;
    A.sp.n_is_one = std::fabs(n - 1.0f) < 1e-6f ? 1 : 0;
    A.rec = D->rec;
    A.w = D->w;
    A.nrec = D->nrec;
    A.valid = D->valid;
    A.area = D->area;
    A.z_old = z_dev;
    A.z = z_out_dev;
    A.n = N;
    copy_f32<<<grid_blocks(N, 256), 256, 0, st>>>(N, z_dev, z_out_dev);
    // heights from the top down: every receiver before its donors
    for (std::int64_t k = static_cast<std::int64_t>(D->level_start.size()) - 2; k >= 0; --k)
    {
        const std::int64_t lo = D->level_start[static_cast<std::size_t>(k)];
        const std::int64_t hi = D->level_start[static_cast<std::size_t>(k) + 1];
        if (hi > lo) dinf_sp_level<<<grid_blocks(hi - lo, 128), 128, 0, st>>>(A, D->topo, lo, hi);
    }
    const cudaError_t e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? LSDTT_GPU_OK : cuda_fail(e, who);
}

}  // extern "C"

namespace lsdtt_gb300
{
LSDTT_DEFINE_LAUNCH_READER(dinf)
}  // namespace lsdtt_gb300
