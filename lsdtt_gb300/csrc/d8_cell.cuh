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

struct D8Exact
{
    int dir;
    std::int64_t rec;
    bool allowed_outlet;
};

// Exact reference evaluation for one cell (used for near-ties and for the
// cells whose float ranking is ambiguous).
__device__ __noinline__ D8Exact exact_receiver(const Grid& g, const float* __restrict__ z,
                                               const std::uint8_t* __restrict__ mask, int row, int col,
                                               int interior_nodata_is_outlet)
{
    const std::int64_t flat = static_cast<std::int64_t>(row) * g.nc + col;
    const double card = g.cell;
    const double diag = g.cell * 1.4142135623730950488;
    const float zc = z[flat];
    double best = 0.0;
    D8Exact o{kNoDir, kOutletReceiver, false};
    for (int d = 0; d < 8; ++d)
    {
        const Step s = resolve_step(g, row, col, d);
        if (s.kind == 2) { o.allowed_outlet = true; continue; }
        if (s.kind == 0) continue;
        const std::int64_t nf = static_cast<std::int64_t>(s.r) * g.nc + s.c;
        if (mask[nf] == 0)
        {
            if (interior_nodata_is_outlet) o.allowed_outlet = true;
            continue;
        }
        if (nf == flat) continue;
        const double dz = static_cast<double>(zc) - static_cast<double>(z[nf]);
        if (dz <= 0.0) continue;
        const double slope = __ddiv_rn(dz, (d & 1) ? diag : card);
        if (slope > best)
        {
            best = slope;
            o.rec = nf;
            o.dir = d;
        }
    }
    return o;
}

// Class-wise ranking of one cell's downhill neighbours. Within a class
// (cardinal d even, diagonal d odd) the reference's slopes share one divisor
// L, so its choice is the first neighbour in direction order with the largest
// fl64(fl64(zc - zn) / L). For float elevations that is the first neighbour
// with the lowest zn (strict '<'): two distinct neighbours zn1 < zn2 are
// at least 2^-24 |zn1| apart, so once |zn1| >= 2^-20 of the drop neither the
// double subtraction nor the division can merge them. d8_decide sends the
// cells outside that bound (and infinities) to the reference's arithmetic.
struct D8Rank
{
    float bz[2];
    int bd[2];
    bool allowed_outlet;
};

__device__ __forceinline__ D8Rank d8_rank(float zc)
{
    D8Rank R;
    R.bz[0] = zc;
    R.bz[1] = zc;
    R.bd[0] = kNoDir;
    R.bd[1] = kNoDir;
    R.allowed_outlet = false;
    return R;
}

// Neighbour d of elevation zn (NaN for a masked neighbour: never taken).
__device__ __forceinline__ void d8_consider(D8Rank& R, float zn, int d)
{
    const int k = d & 1;
    const bool take = zn < R.bz[k];  // downhill of zc and below the class's best so far
    R.bz[k] = take ? zn : R.bz[k];
    R.bd[k] = take ? d : R.bd[k];
}

// zc - zn is exact in float (Sterbenz's lemma, or a zero operand).
__device__ __forceinline__ bool d8_exact_drop(float zc, float zn, float dz)
{
    return (zn > 0.0f && dz <= zn) || (zc < 0.0f && dz <= -zc) || zn == 0.0f || zc == 0.0f;
}

// The winning direction (kNoDir: no downhill neighbour), or -1 when only the
// reference's own double division can decide.
__device__ __forceinline__ int d8_decide(const D8Rank& R, float zc, float inv_card, float inv_diag, double cell)
{
    float dz[2] = {0.0f, 0.0f};
#pragma unroll
    for (int k = 0; k < 2; ++k)
    {
        if (R.bd[k] == kNoDir) continue;
        dz[k] = __fsub_rn(zc, R.bz[k]);  // within 2^-24 of the exact drop
        if (!(fabsf(R.bz[k]) >= dz[k] * 9.5367431640625e-07f) || isinf(dz[k])) return -1;  // 2^-20
    }
    if (R.bd[0] == kNoDir || R.bd[1] == kNoDir) return (R.bd[0] != kNoDir) ? R.bd[0] : R.bd[1];
    // Cardinal vs diagonal: q_c = dz_c / dx against q_d = dz_d / (dx*sqrt2).
    // The float quotients are within 4 * 2^-24 of the exact ones, so a
    // 2^-18 screen settles every clear case. A near-tie between exact 24-bit
    // drops compares dz_c*Ld with dz_d*dx in double: the exact quotients
    // cannot be closer than ~2^-50 relative (sqrt2 is badly approximable:
    // |sqrt2 - p/q| > 1/(4 q^2)), so the products decide the reference's
    // rounded comparison; anything else takes the division path.
    const float sc = __fmul_rn(dz[0], inv_card), sd = __fmul_rn(dz[1], inv_diag);
    if (!(fminf(sc, sd) >= 1.17549435e-38f)) return -1;  // subnormal quotients carry no bound
    if (sc > __fmul_rn(sd, 1.0f + 3.814697265625e-06f)) return R.bd[0];
    if (sd > __fmul_rn(sc, 1.0f + 3.814697265625e-06f)) return R.bd[1];
    if (!d8_exact_drop(zc, R.bz[0], dz[0]) || !d8_exact_drop(zc, R.bz[1], dz[1])) return -1;
    const double A = __dmul_rn(static_cast<double>(dz[0]), cell * 1.4142135623730950488);
    const double B = __dmul_rn(static_cast<double>(dz[1]), cell);
    const double gap = fabs(A - B);
    if (gap > 8.881784197001252e-16 * fmax(A, B)) return (A > B) ? R.bd[0] : R.bd[1];  // 2^-50
    return -1;
}

// Reports a valid cell left without a receiver when neither an outlet
// neighbour nor allow_pits excuses it: the lexicographically first such cell
// (flat + err_base) goes to err[1], as the reference reports it.
__device__ __forceinline__ void d8_unresolved(std::int64_t flat, bool allowed_outlet, int allow_pits,
                                              unsigned long long* __restrict__ err, std::int64_t err_base)
{
    if (!allowed_outlet && !allow_pits)
    {
        atomicMin(err + 1, static_cast<unsigned long long>(flat + err_base));
        raise_error(err, kErrUnresolved, 0);
    }
}

struct D8Out
{
    std::int64_t rec;  // flat index in grid g, or a receiver sentinel
    int dir;
};

// The receiver of cell (row, col) of grid g from global memory, under the
// full boundary rules (grid edges, periodic wrap, 'b' edges, forced outlets,
// nodata); z, mask and forced are that grid's planes.
__device__ __noinline__ D8Out d8_receiver_cell(const Grid& g, const float* __restrict__ z,
                                               const std::uint8_t* __restrict__ mask,
                                               const std::uint8_t* __restrict__ forced, int interior_nodata_is_outlet,
                                               int allow_pits, float inv_card, float inv_diag,
                                               unsigned long long* __restrict__ err, int row, int col,
                                               std::int64_t err_base)
{
    const std::int64_t flat = static_cast<std::int64_t>(row) * g.nc + col;
    if (mask[flat] == 0) return D8Out{kNodataReceiver, kNoDir};
    const bool forced_edge = (row == 0 && g.bc[0] == 'b') || (col == g.nc - 1 && g.bc[1] == 'b') ||
                             (row == g.nr - 1 && g.bc[2] == 'b') || (col == 0 && g.bc[3] == 'b');
    if (forced_edge || (forced != nullptr && forced[flat] != 0)) return D8Out{kOutletReceiver, kNoDir};
    const float zc = z[flat];
    D8Rank R = d8_rank(zc);
    for (int d = 0; d < 8; ++d)
    {
        const Step st = resolve_step(g, row, col, d);
        if (st.kind == 2) { R.allowed_outlet = true; continue; }
        if (st.kind == 0) continue;
        const std::int64_t nf = static_cast<std::int64_t>(st.r) * g.nc + st.c;
        if (mask[nf] == 0)
        {
            if (interior_nodata_is_outlet) R.allowed_outlet = true;
            continue;
        }
        if (nf == flat) continue;
        d8_consider(R, z[nf], d);
    }
    int bdir = d8_decide(R, zc, inv_card, inv_diag, g.cell);
    bool allowed = R.allowed_outlet;
    D8Out o{kOutletReceiver, kNoDir};
    if (bdir == -1)
    {
        const D8Exact e = exact_receiver(g, z, mask, row, col, interior_nodata_is_outlet);
        bdir = e.dir;
        allowed = e.allowed_outlet;
        if (bdir != kNoDir) o = D8Out{e.rec, bdir};
    }
    else if (bdir != kNoDir)
    {
        const Step st = resolve_step(g, row, col, bdir);
        o = D8Out{static_cast<std::int64_t>(st.r) * g.nc + st.c, bdir};
    }
    if (bdir == kNoDir) d8_unresolved(flat, allowed, allow_pits, err, err_base);
    return o;
}

// Direction code the tile pass leaves on an interior cell it cannot settle
// in float (a cross-class near-tie, a drop its bounds do not cover, an
// unexcused pit); the fixup pass replaces it.
constexpr std::uint8_t kD8Undecided = 254;

// Tile pass: the receivers of the interior cells of a 128 x 32 tile, one
// block of 256 threads per tile. The tile and a one-cell halo are staged in
// shared memory (elevations, NaN where masked, and validity bytes) with
// 16-byte loads where the rows are 16-byte aligned; each thread then ranks 4
// consecutive cells of 4 rows from 16-byte shared reads and writes 4 int64
// receivers and 4 direction codes with vector stores. The ranking is
// branch-free and the pass makes no calls: an interior cell it cannot settle
// gets kD8Undecided and raises *undecided; cells on a grid's perimeter get
// provisional values. d8_fixup_cell settles both.
constexpr int kD8TileCols = 128;
constexpr int kD8TileRows = 32;

struct D8TileBuf
{
    float sz[kD8TileRows + 2][136];  // column c0 + k at index 4 + k
    std::uint8_t sm[kD8TileRows + 2][136];
};

// One tile of work: the grid it belongs to, its planes and its position.
struct D8Job
{
    Grid g;
    const float* z;
    const std::uint8_t* mask;
    std::int64_t* receiver;
    std::uint8_t* dir;
    float inv_card, inv_diag;
    int tx, ty;
    std::int64_t rec_base;
};

__device__ __forceinline__ bool d8_job_vec(const D8Job& J)
{
    return (J.g.nc & 3) == 0 && (reinterpret_cast<std::uintptr_t>(J.z) & 15u) == 0 &&
           (reinterpret_cast<std::uintptr_t>(J.receiver) & 15u) == 0 &&
           (reinterpret_cast<std::uintptr_t>(J.mask) & 3u) == 0 && (reinterpret_cast<std::uintptr_t>(J.dir) & 3u) == 0;
}

// Stages a tile (16-byte loads when vec); returns whether this thread saw an
// invalid cell inside the grid.
__device__ __forceinline__ int d8_stage(const D8Job& J, D8TileBuf& B, bool vec)
{
    const float kNan = __int_as_float(0x7fc00000);
    const Grid& g = J.g;
    const int c0 = J.tx * kD8TileCols, r0 = J.ty * kD8TileRows;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int masked = 0;
    for (int lr = w; lr < kD8TileRows + 2; lr += 8)
    {
        const int r = r0 - 1 + lr;
        const bool row_in = r >= 0 && r < g.nr;
        const std::int64_t rf = static_cast<std::int64_t>(r) * g.nc + c0;
        if (vec)
        {
            const int c = c0 + 4 * lane;
            float a[4] = {kNan, kNan, kNan, kNan};
            unsigned ok = 0;
            if (row_in && c + 4 <= g.nc)
            {
                const float4 q = *reinterpret_cast<const float4*>(J.z + rf + 4 * lane);
                ok = *reinterpret_cast<const unsigned*>(J.mask + rf + 4 * lane);
                a[0] = q.x;
                a[1] = q.y;
                a[2] = q.z;
                a[3] = q.w;
                const unsigned zero = __vcmpeq4(ok, 0u);  // 0xff in each invalid byte
                if (zero != 0u)
                {
                    masked = 1;
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        if ((zero >> (8 * j)) & 1u) a[j] = kNan;
                }
            }
            *reinterpret_cast<float4*>(&B.sz[lr][4 + 4 * lane]) = make_float4(a[0], a[1], a[2], a[3]);
            *reinterpret_cast<unsigned*>(&B.sm[lr][4 + 4 * lane]) = ok;
        }
        else
        {
            // rows not 16-byte aligned: four coalesced passes of 32 columns
#pragma unroll
            for (int j = 0; j < 4; ++j)
            {
                const int col = 32 * j + lane;
                float v = kNan;
                std::uint8_t m = 0;
                if (row_in && c0 + col < g.nc)
                {
                    m = J.mask[rf + col];
                    const float zf = J.z[rf + col];
                    v = m ? zf : kNan;
                    masked |= (m == 0);
                }
                B.sz[lr][4 + col] = v;
                B.sm[lr][4 + col] = m;
            }
        }
    }
    if (threadIdx.x < 2 * (kD8TileRows + 2))  // halo columns c0 - 1 and c0 + 128
    {
        const int lr = threadIdx.x >> 1, side = threadIdx.x & 1;
        const int r = r0 - 1 + lr, c = side ? c0 + kD8TileCols : c0 - 1;
        float v = kNan;
        std::uint8_t m = 0;
        if (r >= 0 && r < g.nr && c >= 0 && c < g.nc)
        {
            const std::int64_t f = static_cast<std::int64_t>(r) * g.nc + c;
            m = J.mask[f];
            const float zf = J.z[f];
            v = m ? zf : kNan;
            masked |= (m == 0);
        }
        B.sz[lr][side ? 132 : 3] = v;
        B.sm[lr][side ? 132 : 3] = m;
    }
    return masked;
}

// Ranks the tile staged in B. kMasked: the tile holds invalid cells or a
// forced-outlet plane is given (otherwise every cell is valid and none is
// forced); kInner: the tile lies inside the grid's perimeter (every cell is
// interior, no row or column is ragged). Returns whether an interior cell was
// left undecided.
template <bool kMasked, bool kInner>
__device__ __forceinline__ bool d8_rank_tile(const D8Job& J, const D8TileBuf& B, const int* soff, bool vec,
                                             const std::uint8_t* __restrict__ forced, int interior_nodata_is_outlet,
                                             int allow_pits)
{
    constexpr int TH = kD8TileRows;
    const Grid& g = J.g;
    const float inv_card = J.inv_card, inv_diag = J.inv_diag;
    const int c0 = J.tx * kD8TileCols, r0 = J.ty * TH;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int lc = 4 + 4 * lane, cb = c0 + 4 * lane;
    bool raise = false;
#pragma unroll
    for (int q = 0; q < TH / 8; ++q)
    {
        const int lr = 1 + w + 8 * q, r = r0 + lr - 1;
        if (!kInner && (r >= g.nr || cb >= g.nc)) continue;
        float u[6], m_[6], d_[6];
        {
            const float4 a = *reinterpret_cast<const float4*>(&B.sz[lr - 1][lc]);
            const float4 b = *reinterpret_cast<const float4*>(&B.sz[lr][lc]);
            const float4 e = *reinterpret_cast<const float4*>(&B.sz[lr + 1][lc]);
            u[0] = B.sz[lr - 1][lc - 1];
            u[1] = a.x;
            u[2] = a.y;
            u[3] = a.z;
            u[4] = a.w;
            u[5] = B.sz[lr - 1][lc + 4];
            m_[0] = B.sz[lr][lc - 1];
            m_[1] = b.x;
            m_[2] = b.y;
            m_[3] = b.z;
            m_[4] = b.w;
            m_[5] = B.sz[lr][lc + 4];
            d_[0] = B.sz[lr + 1][lc - 1];
            d_[1] = e.x;
            d_[2] = e.y;
            d_[3] = e.z;
            d_[4] = e.w;
            d_[5] = B.sz[lr + 1][lc + 4];
        }
        const unsigned okc = *reinterpret_cast<const unsigned*>(&B.sm[lr][lc]);
        // Pair minima shared by neighbouring cells: the vertical pair of
        // column k serves the cardinal minimum of cell k - 1 and the diagonal
        // minima of cells k - 2 and k; the horizontal pair k, k + 2 serves
        // the cardinal minimum of cell k.
        float vmin[6], hmin[4];
#pragma unroll
        for (int k = 0; k < 6; ++k) vmin[k] = fminf(u[k], d_[k]);
#pragma unroll
        for (int k = 0; k < 4; ++k) hmin[k] = fminf(m_[k], m_[k + 2]);
        const std::int64_t row_flat = static_cast<std::int64_t>(r) * g.nc;
        const std::int64_t rec_row = row_flat + cb + J.rec_base;  // receiver of cell j: rec_row + j + offset
        const bool row_inner = kInner || (r >= 1 && r <= g.nr - 2);
        std::int64_t rec[4];
        unsigned dirs = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j)
        {
            const int c = cb + j;
            const std::int64_t flat = row_flat + c;
            const float zc = m_[j + 1];
            const float zN = u[j + 1], zNE = u[j + 2], zE = m_[j + 2], zSE = d_[j + 2];
            const float zS = d_[j + 1], zSW = d_[j];  // W = m_[j], NW = u[j]: the class fallbacks below
            // Lowest neighbour per class (fminf skips the NaNs of masked
            // cells); downhill when strictly below zc.
            const float cmin = fminf(vmin[j + 1], hmin[j]);
            const float dmin = fminf(vmin[j], vmin[j + 2]);
            const bool hc = cmin < zc, hd = dmin < zc;
            // The rule of d8_decide, branch-free: float screen of the two
            // class winners (quotients within 4 * 2^-24 of the exact ones,
            // margin 2^-18); the winning class's merge bound (its lowest
            // neighbour at least 2^-20 of the drop away from zero); normal
            // quotients when both classes compete. Everything else is left
            // to the fixup pass.
            const float dzc = __fsub_rn(zc, cmin), dzd = __fsub_rn(zc, dmin);
            const float sc = __fmul_rn(dzc, inv_card), sd = __fmul_rn(dzd, inv_diag);
            const bool cw = sc > __fmul_rn(sd, 1.0f + 3.814697265625e-06f);
            const bool dw = sd > __fmul_rn(sc, 1.0f + 3.814697265625e-06f);
            const bool card = hc && (!hd || cw);
            const float bw = card ? cmin : dmin, dzw = card ? dzc : dzd;
            // first neighbour of the winning class (direction order) at its minimum
            const float q0 = card ? zN : zNE, q1 = card ? zE : zSE, q2 = card ? zS : zSW;
            int k = (q2 == bw) ? 2 : 3;
            k = (q1 == bw) ? 1 : k;
            k = (q0 == bw) ? 0 : k;
            const int bd = 2 * k + (card ? 0 : 1);
            const bool none = !hc && !hd;
            const bool merge_ok = fabsf(bw) >= __fmul_rn(dzw, 9.5367431640625e-07f) && dzw < INFINITY;
            bool allowed = false;
            if (kMasked)
            {
#pragma unroll
                for (int d = 0; d < 8; ++d) allowed |= B.sm[lr + d8_dr(d)][lc + j + d8_dc(d)] == 0;
                allowed = allowed && interior_nodata_is_outlet != 0;
            }
            bool undec = none ? (!allowed && !allow_pits)
                              : (!merge_ok || (hc && hd && (!(cw || dw) || !(fminf(sc, sd) >= 1.17549435e-38f))));
            std::int64_t rj = rec_row + (j + soff[bd]);
            int dj = bd;
            if (none)
            {
                rj = kOutletReceiver;
                dj = kNoDir;
            }
            if (kMasked)
            {
                if (((okc >> (8 * j)) & 0xffu) == 0u)
                {
                    rj = kNodataReceiver;
                    dj = kNoDir;
                    undec = false;
                }
                else if (forced != nullptr && c < g.nc && forced[flat] != 0)
                {
                    rj = kOutletReceiver;
                    dj = kNoDir;
                    undec = false;
                }
            }
            if (undec) dj = kD8Undecided;
            raise |= undec && (kInner || (row_inner && c >= 1 && c <= g.nc - 2));
            rec[j] = rj;
            dirs |= static_cast<unsigned>(dj & 0xff) << (8 * j);
        }
        const std::int64_t f0 = row_flat + cb;
        if (vec && cb + 4 <= g.nc)
        {
            reinterpret_cast<longlong2*>(J.receiver + f0)[0] = make_longlong2(rec[0], rec[1]);
            reinterpret_cast<longlong2*>(J.receiver + f0)[1] = make_longlong2(rec[2], rec[3]);
            *reinterpret_cast<unsigned*>(J.dir + f0) = dirs;
        }
        else
        {
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (cb + j < g.nc)
                {
                    J.receiver[f0 + j] = rec[j];
                    J.dir[f0 + j] = static_cast<std::uint8_t>(dirs >> (8 * j));
                }
        }
    }
    return raise;
}

// The tile pass for tile job J, one block.
__device__ __forceinline__ void d8_receivers_tile(const D8Job& J, const std::uint8_t* __restrict__ forced,
                                                  int interior_nodata_is_outlet, int allow_pits,
                                                  unsigned* __restrict__ undecided)
{
    __shared__ __align__(16) D8TileBuf B;
    __shared__ int soff[8];  // flat offset of each direction
    const bool vec = d8_job_vec(J);
    const int masked = d8_stage(J, B, vec);
    if (threadIdx.x < 8) soff[threadIdx.x] = d8_dr(threadIdx.x) * J.g.nc + d8_dc(threadIdx.x);
    const bool tile_masked = __syncthreads_or(masked) != 0 || forced != nullptr;
    const int c0 = J.tx * kD8TileCols, r0 = J.ty * kD8TileRows;
    const bool inner = r0 >= 1 && r0 + kD8TileRows <= J.g.nr - 1 && c0 >= 1 && c0 + kD8TileCols <= J.g.nc - 1;
    bool raise;
    if (tile_masked)
        raise = inner ? d8_rank_tile<true, true>(J, B, soff, vec, forced, interior_nodata_is_outlet, allow_pits)
                      : d8_rank_tile<true, false>(J, B, soff, vec, forced, interior_nodata_is_outlet, allow_pits);
    else
        raise = inner ? d8_rank_tile<false, true>(J, B, soff, vec, forced, interior_nodata_is_outlet, allow_pits)
                      : d8_rank_tile<false, false>(J, B, soff, vec, forced, interior_nodata_is_outlet, allow_pits);
    if (__any_sync(0xffffffffu, raise) && (threadIdx.x & 31) == 0) atomicOr(undecided, 1u);
}

// Fixup pass, one cell: the full rule from global memory (d8_receiver_cell)
// for a perimeter cell or a cell the tile pass left undecided.
__device__ __forceinline__ void d8_fixup_cell(const Grid& g, const float* __restrict__ z,
                                              const std::uint8_t* __restrict__ mask,
                                              const std::uint8_t* __restrict__ forced, int interior_nodata_is_outlet,
                                              int allow_pits, float inv_card, float inv_diag,
                                              std::int64_t* __restrict__ receiver, std::uint8_t* __restrict__ dir,
                                              unsigned long long* __restrict__ err, int row, int col,
                                              std::int64_t err_base, std::int64_t rec_base)
{
    const D8Out o = d8_receiver_cell(g, z, mask, forced, interior_nodata_is_outlet, allow_pits, inv_card, inv_diag,
                                     err, row, col, err_base);
    const std::int64_t flat = static_cast<std::int64_t>(row) * g.nc + col;
    receiver[flat] = o.rec >= 0 ? o.rec + rec_base : o.rec;
    dir[flat] = static_cast<std::uint8_t>(o.dir);
}

// Number of perimeter cells of grid g and the (row, col) of the i-th.
__host__ __device__ inline std::int64_t d8_perimeter(int nr, int nc)
{
    if (nr <= 2 || nc <= 2) return static_cast<std::int64_t>(nr) * nc;
    return 2 * static_cast<std::int64_t>(nc) + 2 * static_cast<std::int64_t>(nr - 2);
}

__host__ __device__ inline void d8_perimeter_cell(int nr, int nc, std::int64_t i, int& row, int& col)
{
    if (nr <= 2 || nc <= 2)
    {
        row = static_cast<int>(i / nc);
        col = static_cast<int>(i % nc);
        return;
    }
    if (i < nc)
    {
        row = 0;
        col = static_cast<int>(i);
    }
    else if (i < 2 * static_cast<std::int64_t>(nc))
    {
        row = nr - 1;
        col = static_cast<int>(i - nc);
    }
    else
    {
        const std::int64_t j = i - 2 * static_cast<std::int64_t>(nc);
        row = 1 + static_cast<int>(j >> 1);
        col = (j & 1) ? nc - 1 : 0;
    }
}

}  // namespace
}  // namespace lsdtt_gb300
