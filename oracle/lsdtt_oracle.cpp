// lsdtt_oracle.cpp -- TEST INFRASTRUCTURE ONLY (the CPU oracle).
//
// A restatement, in plain C++17, of the reference lsdtt3 algorithms on the
// landscape-evolution hot path. It is the checker for the GPU kernels (GPU
// parity tests), the CPU baseline that bench.py times, and it is itself
// pinned against (a) the reference's golden FNV-1a vectors in
// tests/cpp/test_flow_d8_identity.cpp and (b) the reference's own sources
// compiled into oracle/_ref/liblsdtt_ref.so. The product never links it.
//
// Reference file paths below are relative to the lsdtt3 checkout.
//
// Floating point: build with -ffp-contract=off (oracle/Makefile). Every
// expression keeps the reference's operand types (float vs double), because the
// results must be bitwise those of the reference's x86-64 build.

#include <algorithm>
#include <array>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <deque>
#include <functional>
#include <limits>
#include <queue>
#include <stdexcept>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace
{

// D8 clockwise N, NE, E, SE, S, SW, W, NW -- direction codes 0..7
// (src/utils/lsdtt_grid_neighbours.hpp:50-51).
constexpr int kDr[8] = {-1, -1, 0, 1, 1, 1, 0, -1};
constexpr int kDc[8] = {0, 1, 1, 1, 0, -1, -1, -1};
constexpr double kSqrt2d = 1.4142135623730950488;
constexpr float kSqrt2f = static_cast<float>(kSqrt2d);

constexpr std::int64_t kNodataReceiver = -1;  // src/core/lsdtt_types.hpp:142
constexpr std::int64_t kOutletReceiver = -2;  // src/core/lsdtt_types.hpp:143
constexpr std::uint8_t kNoDirection = 255;    // src/core/lsdtt_types.hpp:144

void put_err(char* err, int errlen, const std::string& what)
{
    if (!err || errlen <= 0) return;
    std::strncpy(err, what.c_str(), static_cast<std::size_t>(errlen - 1));
    err[errlen - 1] = '\0';
}

bool is_nodata(double v, double ndv)
{
    if (std::isnan(ndv)) return std::isnan(v);
    return v == ndv;
}

// ============================================================================
// Fill: improved priority-flood with epsilon (Barnes et al. 2014)
// src/cpu/lsdtt_raster_flow_preprocessing_cpu.cpp:416-511 (core),
// :518-589 (seeding), :350-392 (inputs), :727-782 (dispatch).
// ============================================================================

struct Node
{
    float zeta;
    int row;
    int col;
};
// Min-heap keyed on zeta only, exactly std::priority_queue<.., greater<>>
// with a comparator that looks at zeta alone (:55-62): ties fall wherever
// libstdc++'s push_heap/pop_heap leave them, and the restatement performs the
// same push/pop sequence, so it leaves them in the same places.
//
// With index_ties, equal keys are ordered by (row, col) instead: the rule the
// GPU fill uses (a parallel fill cannot reproduce a binary heap's layout).
// That variant is a test instrument, not a restatement of the reference.
struct NodeGreater
{
    bool index_ties = false;
    bool operator()(const Node& a, const Node& b) const
    {
        if (a.zeta != b.zeta || !index_ties) return a.zeta > b.zeta;
        return a.row != b.row ? a.row > b.row : a.col > b.col;
    }
};
using Heap = std::priority_queue<Node, std::vector<Node>, NodeGreater>;

enum : int { kOpen = 0, kQueued = 1, kClosed = 2, kNoCell = -1 };

struct FillTrace
{
    std::int64_t* discoverer = nullptr;  // flat index of the cell that queued it; -1 seed
    std::int64_t* order = nullptr;       // position in the processing sequence
    std::uint8_t* via_fifo = nullptr;    // 1 = raised (went through the FIFO)
};

void priority_flood(std::vector<float>& dem, std::vector<int>& idx, int nr, int nc,
                    float L, float min_slope, bool per_ns, bool per_ew, FillTrace tr, bool index_ties = false)
{
    NodeGreater cmp;
    cmp.index_ties = index_ties;
    Heap pq(cmp);

    // Seeding (:518-589): every non-nodata cell on a non-periodic raster edge,
    // plus cells with an in-bounds nodata neighbour when the interior has any
    // nodata at all. Row-major push order.
    bool interior_nodata = false;
    for (int r = 1; r < nr - 1 && !interior_nodata; ++r)
        for (int c = 1; c < nc - 1; ++c)
            if (idx[static_cast<std::size_t>(r) * nc + c] == kNoCell) { interior_nodata = true; break; }

    for (int r = 0; r < nr; ++r)
        for (int c = 0; c < nc; ++c)
        {
            const std::size_t k = static_cast<std::size_t>(r) * nc + c;
            if (idx[k] == kNoCell) continue;
            bool seed = (!per_ns && (r == 0 || r == nr - 1)) || (!per_ew && (c == 0 || c == nc - 1));
            if (!seed && interior_nodata)
                for (int n = 0; n < 8 && !seed; ++n)
                {
                    const int rr = r + kDr[n], cc = c + kDc[n];
                    if (rr >= 0 && rr < nr && cc >= 0 && cc < nc &&
                        idx[static_cast<std::size_t>(rr) * nc + cc] == kNoCell)
                        seed = true;
                }
            if (seed && idx[k] == kOpen)
            {
                pq.push(Node{dem[k], r, c});
                idx[k] = kQueued;
                if (tr.discoverer) tr.discoverer[k] = -1;
            }
        }

    std::deque<Node> fifo;
    std::int64_t seq = 0;
    while (!pq.empty() || !fifo.empty())
    {
        Node cur;
        bool from_fifo = false;
        if (!fifo.empty() && (pq.empty() || fifo.front().zeta <= pq.top().zeta))
        {
            cur = fifo.front();
            fifo.pop_front();
            from_fifo = true;
        }
        else
        {
            cur = pq.top();
            pq.pop();
        }
        const std::size_t ck = static_cast<std::size_t>(cur.row) * nc + cur.col;
        if (idx[ck] == kClosed) continue;
        idx[ck] = kClosed;
        if (tr.order) tr.order[ck] = seq;
        if (tr.via_fifo) tr.via_fifo[ck] = from_fifo ? 1 : 0;
        ++seq;

        for (int n = 0; n < 8; ++n)
        {
            int rr = cur.row + kDr[n];
            int cc = cur.col + kDc[n];
            if (per_ns) { if (rr < 0) rr += nr; else if (rr >= nr) rr -= nr; }
            if (per_ew) { if (cc < 0) cc += nc; else if (cc >= nc) cc -= nc; }
            if (rr < 0 || rr >= nr || cc < 0 || cc >= nc) continue;
            const std::size_t k = static_cast<std::size_t>(rr) * nc + cc;
            if (idx[k] != kOpen) continue;
            float nz = dem[k];
            if (nz <= cur.zeta)
            {
                if (min_slope > 0.0f)
                {
                    const float d = (n % 2 == 0) ? L : L * kSqrt2f;
                    const float requested = cur.zeta + min_slope * d;
                    const float strict = std::nextafter(cur.zeta, std::numeric_limits<float>::infinity());
                    nz = std::max(requested, strict);
                }
                else
                {
                    nz = cur.zeta;
                }
                dem[k] = nz;
                fifo.push_back(Node{nz, rr, cc});
            }
            else
            {
                pq.push(Node{nz, rr, cc});
            }
            idx[k] = kQueued;
            if (tr.discoverer) tr.discoverer[k] = static_cast<std::int64_t>(ck);
        }
    }
}

// ============================================================================
// D8 engine: lsdtt_flowinfo (src/cpu/lsdtt_flowinfo_cpu.cpp)
// ============================================================================

struct Bc
{
    char c[4];  // N E S W
};

Bc parse_bc(const char* s)
{
    // parse_boundary_conditions (:845-884): length 4, codes o/n/p/b folded to
    // lower case, periodic flags must match per axis.
    const std::string b = s ? s : "";
    if (b.size() != 4)
        throw std::runtime_error("lsdtt_flowinfo: boundary_conditions must have length 4 (north, east, south, west)");
    Bc out{};
    for (int i = 0; i < 4; ++i)
    {
        const char ch = static_cast<char>(std::tolower(static_cast<unsigned char>(b[i])));
        if (ch != 'o' && ch != 'n' && ch != 'p' && ch != 'b')
            throw std::runtime_error(std::string("lsdtt_flowinfo: invalid boundary code '") + b[i] + "'");
        out.c[i] = ch;
    }
    if ((out.c[0] == 'p') != (out.c[2] == 'p'))
        throw std::runtime_error("lsdtt_flowinfo: north and south periodic boundary flags must match");
    if ((out.c[1] == 'p') != (out.c[3] == 'p'))
        throw std::runtime_error("lsdtt_flowinfo: east and west periodic boundary flags must match");
    return out;
}

struct Resolved
{
    bool inside = false;
    bool outlet = false;
    int r = 0, c = 0;
};

// resolve_neighbour (:101-158)
Resolved resolve(int row, int col, int dir, int nr, int nc, const Bc& bc)
{
    Resolved res;
    int r = row + kDr[dir], c = col + kDc[dir];
    bool out = false;
    if (r < 0)
    {
        if (bc.c[0] == 'p') r = nr - 1;
        else if (bc.c[0] == 'o' || bc.c[0] == 'b') out = true;
        else return res;
    }
    else if (r >= nr)
    {
        if (bc.c[2] == 'p') r = 0;
        else if (bc.c[2] == 'o' || bc.c[2] == 'b') out = true;
        else return res;
    }
    if (c < 0)
    {
        if (bc.c[3] == 'p') c = nc - 1;
        else if (bc.c[3] == 'o' || bc.c[3] == 'b') out = true;
        else return res;
    }
    else if (c >= nc)
    {
        if (bc.c[1] == 'p') c = 0;
        else if (bc.c[1] == 'o' || bc.c[1] == 'b') out = true;
        else return res;
    }
    if (out) { res.outlet = true; return res; }
    res.inside = true;
    res.r = r;
    res.c = c;
    return res;
}

struct FlowOpts
{
    Bc bc;
    bool interior_nodata_is_outlet = true;
    bool allow_pits_as_outlets = false;
    bool build_topo = true;
    bool build_sv = true;
    bool require_acyclic = true;
    int n_threads = 0;
};

struct Flow
{
    int nr = 0, nc = 0;
    double cell = 0.0;
    std::vector<std::uint8_t> mask;
    std::vector<std::int64_t> receiver;
    std::vector<std::uint8_t> dir;
    std::vector<std::uint8_t> donors;
    std::vector<std::int64_t> outlets;
    std::vector<std::int64_t> topo;
    bool has_topo = false;
    bool acyclic = false;
    std::vector<std::int64_t> svec, sv_start;
    std::vector<std::uint64_t> sv_size;
    bool has_sv = false;
    std::int64_t n_valid = 0;
};

// build_receiver_graph_d8 (:1077-1329). Every cell's receiver is independent of
// every other's; the strict '>' in direction order 0..7 keeps the first of
// equal slopes. Slopes are double: (double)z - (double)z_nb over dx or dx*sqrt2.
void build_receivers(Flow& F, const float* z, const FlowOpts& o,
                     const std::vector<std::uint8_t>& forced_plane)
{
    const int nr = F.nr, nc = F.nc;
    const double card = F.cell, diag = F.cell * kSqrt2d;
    bool failed = false;
    int fail_r = 0, fail_c = 0;
    int nthreads = o.n_threads;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for collapse(2) schedule(static) num_threads(nthreads)
#endif
    for (int row = 0; row < nr; ++row)
        for (int col = 0; col < nc; ++col)
        {
            const std::int64_t flat = static_cast<std::int64_t>(row) * nc + col;
            if (F.mask[flat] == 0) { F.receiver[flat] = kNodataReceiver; F.dir[flat] = kNoDirection; continue; }
            const bool forced_edge = (row == 0 && o.bc.c[0] == 'b') || (col == nc - 1 && o.bc.c[1] == 'b') ||
                                     (row == nr - 1 && o.bc.c[2] == 'b') || (col == 0 && o.bc.c[3] == 'b');
            if (forced_edge || (!forced_plane.empty() && forced_plane[flat]))
            {
                F.receiver[flat] = kOutletReceiver;
                F.dir[flat] = kNoDirection;
                continue;
            }
            const float zc = z[flat];
            double best = 0.0;
            std::int64_t best_rec = kOutletReceiver;
            std::uint8_t best_dir = kNoDirection;
            bool allowed_outlet = false;
            for (int d = 0; d < 8; ++d)
            {
                const Resolved nb = resolve(row, col, d, nr, nc, o.bc);
                if (nb.outlet) { allowed_outlet = true; continue; }
                if (!nb.inside) continue;
                const std::int64_t nf = static_cast<std::int64_t>(nb.r) * nc + nb.c;
                if (F.mask[nf] == 0)
                {
                    if (o.interior_nodata_is_outlet) allowed_outlet = true;
                    continue;
                }
                if (nf == flat) continue;
                const double dz = static_cast<double>(zc) - static_cast<double>(z[nf]);
                if (dz <= 0.0) continue;
                const double slope = dz / ((d % 2 == 0) ? card : diag);
                if (slope > best) { best = slope; best_rec = nf; best_dir = static_cast<std::uint8_t>(d); }
            }
            if (best_dir != kNoDirection) { F.receiver[flat] = best_rec; F.dir[flat] = best_dir; }
            else
            {
                F.receiver[flat] = kOutletReceiver;
                F.dir[flat] = kNoDirection;
                if (!allowed_outlet && !o.allow_pits_as_outlets)
                {
#ifdef _OPENMP
#pragma omp critical(oracle_receiver_failure)
#endif
                    {
                        if (!failed || row < fail_r || (row == fail_r && col < fail_c))
                        {
                            failed = true;
                            fail_r = row;
                            fail_c = col;
                        }
                    }
                }
            }
        }
    if (failed)
        throw std::runtime_error("lsdtt_flowinfo: could not assign a receiver at row " + std::to_string(fail_r) +
                                 ", col " + std::to_string(fail_c) +
                                 ". The DEM likely contains an unresolved sink or flat.");
}

// build_donor_counts_and_outlets_d8 (:1359-1408)
void build_donors(Flow& F)
{
    const std::int64_t n = static_cast<std::int64_t>(F.nr) * F.nc;
    F.outlets.clear();
    for (std::int64_t f = 0; f < n; ++f)
    {
        if (!F.mask[f]) continue;
        const std::int64_t r = F.receiver[f];
        if (r >= 0)
        {
            if (F.donors[r] == 255) throw std::runtime_error("lsdtt_flowinfo: donor count overflow while building donor counts");
            ++F.donors[r];
        }
        else if (r == kOutletReceiver)
            F.outlets.push_back(f);
    }
}

// build_topological_order (:1428-1522): Kahn's FIFO, headwaters seeded in
// row-major order; a short result means the graph is cyclic.
void build_topo(Flow& F)
{
    const std::int64_t n = static_cast<std::int64_t>(F.nr) * F.nc;
    F.topo.clear();
    F.topo.reserve(static_cast<std::size_t>(F.n_valid));
    if (F.n_valid == 0) { F.has_topo = true; F.acyclic = true; return; }
    std::vector<std::uint8_t> rem(F.donors);
    for (std::int64_t f = 0; f < n; ++f)
        if (F.mask[f] && rem[f] == 0) F.topo.push_back(f);
    for (std::size_t head = 0; head < F.topo.size(); ++head)
    {
        const std::int64_t r = F.receiver[F.topo[head]];
        if (r >= 0 && --rem[r] == 0) F.topo.push_back(r);
    }
    if (static_cast<std::int64_t>(F.topo.size()) != F.n_valid)
    {
        F.topo.clear();
        F.has_topo = false;
        F.acyclic = false;
        return;
    }
    F.has_topo = true;
    F.acyclic = true;
}

// build_s_vector (:1544-1731): iterative DFS preorder from each outlet in
// row-major order, donors visited in ascending flat index.
void build_svector(Flow& F, const Bc& bc)
{
    if (!F.acyclic) throw std::runtime_error("lsdtt_flowinfo: cannot build s_vector from a cyclic or invalid routing graph");
    const std::int64_t n = static_cast<std::int64_t>(F.nr) * F.nc;
    F.sv_start.assign(static_cast<std::size_t>(n), kNodataReceiver);
    F.sv_size.assign(static_cast<std::size_t>(n), 0);
    F.svec.clear();
    F.svec.reserve(static_cast<std::size_t>(F.n_valid));
    if (F.n_valid == 0) { F.has_sv = true; return; }
    if (F.outlets.empty()) throw std::runtime_error("lsdtt_flowinfo: cannot build s_vector because no outlets were found");

    struct Frame
    {
        std::int64_t flat;
        std::int64_t donors[8];
        int nd;
        int next;
    };
    auto make = [&](std::int64_t flat) {
        Frame fr{};
        fr.flat = flat;
        F.sv_start[flat] = static_cast<std::int64_t>(F.svec.size());
        F.sv_size[flat] = 1;
        F.svec.push_back(flat);
        const int row = static_cast<int>(flat / F.nc), col = static_cast<int>(flat % F.nc);
        for (int d = 0; d < 8; ++d)
        {
            const Resolved nb = resolve(row, col, d, F.nr, F.nc, bc);
            if (!nb.inside) continue;
            const std::int64_t df = static_cast<std::int64_t>(nb.r) * F.nc + nb.c;
            if (!F.mask[df] || F.receiver[df] != flat) continue;
            bool dup = false;
            for (int i = 0; i < fr.nd; ++i) dup = dup || fr.donors[i] == df;
            if (!dup) fr.donors[fr.nd++] = df;
        }
        std::sort(fr.donors, fr.donors + fr.nd);
        return fr;
    };
    std::vector<Frame> st;
    for (const std::int64_t o : F.outlets)
    {
        if (F.sv_start[o] >= 0) continue;
        st.clear();
        st.push_back(make(o));
        while (!st.empty())
        {
            Frame& fr = st.back();
            if (fr.next < fr.nd)
            {
                const std::int64_t child = fr.donors[fr.next++];
                if (F.sv_start[child] >= 0) throw std::runtime_error("lsdtt_flowinfo: duplicate visit while building s_vector");
                st.push_back(make(child));
                continue;
            }
            const std::int64_t done = fr.flat;
            const std::uint64_t sz = F.sv_size[done];
            st.pop_back();
            if (!st.empty()) F.sv_size[st.back().flat] += sz;
        }
    }
    if (static_cast<std::int64_t>(F.svec.size()) != F.n_valid)
        throw std::runtime_error("lsdtt_flowinfo: s_vector does not cover all valid cells");
    F.has_sv = true;
}

Flow build_flow(const float* z, const std::uint8_t* mask, int nr, int nc, double cell, double nodata,
                const FlowOpts& o, const std::int64_t* forced, std::int64_t n_forced)
{
    if (!(nr > 0 && nc > 0 && cell > 0.0)) throw std::runtime_error("lsdtt_flowinfo: raster metadata is invalid");
    Flow F;
    F.nr = nr;
    F.nc = nc;
    F.cell = cell;
    const std::int64_t n = static_cast<std::int64_t>(nr) * nc;
    F.mask.assign(mask, mask + n);
    // validate_inputs (:887-966): valid cells need finite, non-nodata z.
    const float ndv = static_cast<float>(nodata);
    for (int r = 0; r < nr; ++r)
        for (int c = 0; c < nc; ++c)
        {
            const std::int64_t f = static_cast<std::int64_t>(r) * nc + c;
            if (!F.mask[f]) continue;
            if (!std::isfinite(z[f]) || z[f] == ndv)
                throw std::runtime_error("lsdtt_flowinfo: valid mask cell has nodata or non-finite DEM value at row " +
                                         std::to_string(r) + ", col " + std::to_string(c));
        }
    // validate_forced_outlet_flats (:969-1009)
    std::vector<std::uint8_t> plane;
    if (n_forced > 0)
    {
        plane.assign(static_cast<std::size_t>(n), 0);
        for (std::int64_t i = 0; i < n_forced; ++i)
        {
            const std::int64_t f = forced[i];
            if (f < 0 || f >= n)
                throw std::invalid_argument("lsdtt_flowinfo: forced outlet flat index " + std::to_string(f) + " (entry " +
                                            std::to_string(i) + ") is outside the raster, which has " +
                                            std::to_string(n) + " cells");
            if (!F.mask[f])
                throw std::invalid_argument("lsdtt_flowinfo: forced outlet flat index " + std::to_string(f) + " (entry " +
                                            std::to_string(i) + ", row " + std::to_string(f / nc) + ", col " +
                                            std::to_string(f % nc) +
                                            ") lands on a nodata or masked cell, so it cannot act as a flow termination");
            plane[f] = 1;
        }
    }
    for (std::int64_t f = 0; f < n; ++f) F.n_valid += F.mask[f] ? 1 : 0;
    F.receiver.assign(static_cast<std::size_t>(n), kNodataReceiver);
    F.dir.assign(static_cast<std::size_t>(n), kNoDirection);
    F.donors.assign(static_cast<std::size_t>(n), 0);
    build_receivers(F, z, o, plane);
    build_donors(F);
    if (o.build_topo || o.build_sv || o.require_acyclic)
    {
        build_topo(F);
        if (!F.acyclic && o.require_acyclic)
            throw std::runtime_error(
                "lsdtt_flowinfo: routing graph is cyclic or incomplete. This usually means the DEM still contains "
                "unresolved flats, pits, or incompatible periodic routing.");
    }
    if (o.build_sv) build_svector(F, o.bc);
    return F;
}

// accumulate (:1979-2046): seed every valid cell with its weight (dx^2 by
// default), then push acc[rec] += acc[flat] in topological order.
std::vector<double> accumulate(const Flow& F, const double* w)
{
    const std::int64_t n = static_cast<std::int64_t>(F.nr) * F.nc;
    const double dw = F.cell * F.cell;
    if (w)
        for (std::int64_t f = 0; f < n; ++f)
            if (F.mask[f] && !std::isfinite(w[f]))
                throw std::invalid_argument("lsdtt_flowinfo::accumulate: cell_weights must be finite for all valid cells");
    std::vector<double> acc(static_cast<std::size_t>(n), 0.0);
    for (std::int64_t f = 0; f < n; ++f)
        if (F.mask[f]) acc[f] = w ? w[f] : dw;
    for (const std::int64_t f : F.topo)
    {
        const std::int64_t r = F.receiver[f];
        if (r >= 0) acc[r] += acc[f];
    }
    return acc;
}

std::uint64_t splitmix64(std::uint64_t x)
{
    // Steele, Lea & Flood (2014) splitmix64 with Vigna's published constants.
    x += 0x9E3779B97F4A7C15ULL;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
    return x ^ (x >> 31);
}

std::uint64_t mix_in(std::uint64_t h, std::uint64_t v)
{
    return splitmix64(h ^ (v + 0x9E3779B97F4A7C15ULL + (h << 6) + (h >> 2)));
}

// ============================================================================
// D-infinity flow graph and stream power: lsdtt_flowgraph_cpu with
// method = d_infinity (src/cpu/lsdtt_flowgraph_cpu.cpp:87-178 constructor,
// :423-662 build_dinf after Tarboton 1997, :874-985 topological order,
// :988-1039 accumulate, :1179-1226 build_reverse_levels) and
// compute_dinf_stream_power_incision (src/cpu/lsdtt_stream_power_cpu.cpp:
// 329-602).
// ============================================================================

struct Dinf
{
    int nr = 0, nc = 0;
    double cell = 1.0;
    std::vector<std::uint8_t> valid;
    std::vector<std::int64_t> rec;  // [2n], -1 none
    std::vector<float> w;           // [2n]
    std::vector<std::uint8_t> nrec, donors;
    std::vector<float> slope, bearing;
    std::vector<std::int64_t> topo;
};

Dinf build_dinf_graph(const float* z, const std::uint8_t* mask, int nr, int nc, double cell, double nodata,
                      const char* bcs, bool interior_nodata_is_outlet)
{
    // Tarboton's eight facets: cardinal e1 and diagonal e2 offsets, the
    // sector and sign that turn the in-facet angle into a bearing (:60-67).
    static const int e1r[8] = {0, -1, -1, 0, 0, 1, 1, 0}, e1c[8] = {1, 0, 0, -1, -1, 0, 0, 1};
    static const int e2r[8] = {-1, -1, -1, -1, 1, 1, 1, 1}, e2c[8] = {1, 1, -1, -1, -1, -1, 1, 1};
    static const int ac[8] = {0, 1, 1, 2, 2, 3, 3, 4}, af[8] = {1, -1, 1, -1, 1, -1, 1, -1};
    static const int nbr[8] = {-1, 0, 0, 1, -1, -1, 1, 1}, nbc[8] = {0, -1, 1, 0, -1, 1, -1, 1};
    const float pi4 = static_cast<float>(M_PI / 4.0);
    const float rad2deg = static_cast<float>(180.0 / M_PI);
    const std::string b = bcs ? bcs : "";
    if (b.size() != 4)
        throw std::invalid_argument("lsdtt_flowgraph_cpu: boundary_conditions must have exactly 4 characters "
                                    "(north, east, south, west)");
    char c4[4];
    for (int i = 0; i < 4; ++i) c4[i] = static_cast<char>(std::tolower(static_cast<unsigned char>(b[i])));
    for (int i = 0; i < 4; ++i)
        if (c4[i] != 'o' && c4[i] != 'n' && c4[i] != 'p' && c4[i] != 'b')
            throw std::invalid_argument("lsdtt_flowgraph_cpu: boundary_conditions contains an invalid character. "
                                        "Allowed values are o, n, p, b.");
    if ((c4[0] == 'p') != (c4[2] == 'p'))
        throw std::invalid_argument("lsdtt_flowgraph_cpu: north and south periodic boundary flags must match");
    if ((c4[1] == 'p') != (c4[3] == 'p'))
        throw std::invalid_argument("lsdtt_flowgraph_cpu: east and west periodic boundary flags must match");
    Dinf G;
    G.nr = nr;
    G.nc = nc;
    G.cell = cell;
    const std::size_t n = static_cast<std::size_t>(nr) * nc;
    const float ndv = static_cast<float>(nodata);
    G.valid.assign(n, 0);
    std::int64_t nvalid = 0;
    for (std::size_t i = 0; i < n; ++i)
        if (mask[i] && z[i] != ndv && std::isfinite(z[i])) { G.valid[i] = 1; ++nvalid; }
    G.rec.assign(2 * n, -1);
    G.w.assign(2 * n, 0.0f);
    G.nrec.assign(n, 0);
    G.slope.assign(n, ndv);
    G.bearing.assign(n, ndv);
    auto resolve = [&](int r, int c, int dr, int dc, int& rr, int& cc) {
        rr = r + dr;
        cc = c + dc;
        if (rr < 0) { if (c4[0] == 'p') rr = nr - 1; else return false; }
        if (rr >= nr) { if (c4[2] == 'p') rr = 0; else return false; }
        if (cc < 0) { if (c4[3] == 'p') cc = nc - 1; else return false; }
        if (cc >= nc) { if (c4[1] == 'p') cc = 0; else return false; }
        return true;
    };
    const float L = static_cast<float>(cell);
    for (int r = 0; r < nr; ++r)
        for (int c = 0; c < nc; ++c)
        {
            const std::size_t f = static_cast<std::size_t>(r) * nc + c;
            if (!G.valid[f]) continue;
            const bool forced = (c4[0] == 'b' && r == 0) || (c4[2] == 'b' && r == nr - 1) ||
                                (c4[1] == 'b' && c == nc - 1) || (c4[3] == 'b' && c == 0);
            if (forced) continue;
            if (interior_nodata_is_outlet)
            {
                bool touches = false;
                for (int k = 0; k < 8 && !touches; ++k)
                {
                    const int rr = r + nbr[k], cc = c + nbc[k];
                    if (rr < 0 || rr >= nr || cc < 0 || cc >= nc) continue;
                    touches = !G.valid[static_cast<std::size_t>(rr) * nc + cc];
                }
                if (touches) continue;
            }
            const float e0 = z[f];
            float best_s = 0.0f, best_r = 0.0f;
            int best = -1;
            std::int64_t b1 = -1, b2 = -1;
            for (int a = 0; a < 8; ++a)
            {
                int r1, c1, r2, c2;
                if (!resolve(r, c, e1r[a], e1c[a], r1, c1) || !resolve(r, c, e2r[a], e2c[a], r2, c2)) continue;
                const std::int64_t f1 = static_cast<std::int64_t>(r1) * nc + c1;
                const std::int64_t f2 = static_cast<std::int64_t>(r2) * nc + c2;
                if (f1 == static_cast<std::int64_t>(f) || f2 == static_cast<std::int64_t>(f)) continue;
                if (!G.valid[f1] || !G.valid[f2]) continue;
                const float e1 = z[f1], e2 = z[f2];
                if (e0 <= e1 && e0 <= e2) continue;
                float rr, ss;
                const float s1 = (e0 - e1) / L;
                const float s2 = (e1 - e2) / L;
                if (e0 > e1 && e0 > e2)
                {
                    rr = std::atan2(s2, s1);
                    if (rr < 0.0f) { rr = 0.0f; ss = s1; }
                    else if (rr > pi4) { rr = pi4; ss = (e0 - e2) / (L * kSqrt2f); }
                    else ss = std::sqrt(s1 * s1 + s2 * s2);
                }
                else if (e0 > e1) { rr = 0.0f; ss = s1; }
                else { rr = pi4; ss = (e0 - e2) / (L * kSqrt2f); }
                if (ss > best_s) { best_s = ss; best_r = rr; best = a; b1 = f1; b2 = f2; }
            }
            if (best < 0) continue;
            const float ang = static_cast<float>(af[best]) * best_r +
                              static_cast<float>(ac[best]) * (static_cast<float>(M_PI) * 0.5f);
            float bearing = 360.0f - (ang * rad2deg) + 90.0f;
            while (bearing >= 360.0f) bearing -= 360.0f;
            while (bearing < 0.0f) bearing += 360.0f;
            G.slope[f] = best_s;
            G.bearing[f] = bearing;
            if (best_r == 0.0f) { G.nrec[f] = 1; G.rec[2 * f] = b1; G.w[2 * f] = 1.0f; }
            else if (best_r >= pi4) { G.nrec[f] = 1; G.rec[2 * f] = b2; G.w[2 * f] = 1.0f; }
            else
            {
                const float p2 = best_r / pi4;
                const float p1 = 1.0f - p2;
                if (b1 == b2) { G.nrec[f] = 1; G.rec[2 * f] = b1; G.w[2 * f] = 1.0f; }
                else
                {
                    G.nrec[f] = 2;
                    G.rec[2 * f] = b1;
                    G.w[2 * f] = p1;
                    G.rec[2 * f + 1] = b2;
                    G.w[2 * f + 1] = p2;
                }
            }
        }
    // Donor counts (unique donors) and Kahn's order (FIFO, row-major seeds).
    G.donors.assign(n, 0);
    for (std::size_t f = 0; f < n; ++f)
        for (int k = 0; k < G.nrec[f]; ++k)
        {
            const std::int64_t r = G.rec[2 * f + k];
            if (k == 1 && r == G.rec[2 * f]) continue;
            if (G.donors[r] < 255) ++G.donors[r];
        }
    std::vector<std::uint8_t> remaining = G.donors;
    std::deque<std::int64_t> q;
    for (std::size_t f = 0; f < n; ++f)
        if (G.valid[f] && remaining[f] == 0) q.push_back(static_cast<std::int64_t>(f));
    G.topo.reserve(static_cast<std::size_t>(nvalid));
    while (!q.empty())
    {
        const std::int64_t f = q.front();
        q.pop_front();
        G.topo.push_back(f);
        for (int k = 0; k < G.nrec[f]; ++k)
        {
            const std::int64_t r = G.rec[2 * f + k];
            if (--remaining[r] == 0) q.push_back(r);
        }
    }
    if (static_cast<std::int64_t>(G.topo.size()) != nvalid)
        throw std::runtime_error("lsdtt_flowgraph_cpu: cycle detected in receiver graph or inconsistent cell validity. "
                                 "Ensure the DEM is pit-filled and that valid cells have finite, non-nodata "
                                 "elevations.");
    return G;
}

std::vector<double> dinf_accumulate(const Dinf& G, const double* w)
{
    const std::size_t n = G.valid.size();
    std::vector<double> acc(n, 0.0);
    const double dw = G.cell * G.cell;
    for (const std::int64_t f : G.topo) acc[f] = w ? w[f] : dw;
    for (const std::int64_t f : G.topo)
    {
        const double a = acc[f];
        for (int k = 0; k < G.nrec[f]; ++k) acc[G.rec[2 * f + k]] += a * static_cast<double>(G.w[2 * f + k]);
    }
    return acc;
}

// build_reverse_levels: depth 0 for cells without receivers, else one more
// than the deepest receiver; each level in reverse topological order.
std::vector<std::vector<std::int64_t>> dinf_reverse_levels(const Dinf& G)
{
    std::vector<int> depth(G.valid.size(), -1);
    int maxd = 0;
    for (std::int64_t i = static_cast<std::int64_t>(G.topo.size()) - 1; i >= 0; --i)
    {
        const std::int64_t f = G.topo[static_cast<std::size_t>(i)];
        int d = 0;
        for (int k = 0; k < G.nrec[f]; ++k)
        {
            const std::int64_t r = G.rec[2 * f + k];
            if (r >= 0 && depth[r] >= 0) d = std::max(d, depth[r] + 1);
        }
        depth[f] = d;
        maxd = std::max(maxd, d);
    }
    std::vector<std::vector<std::int64_t>> levels(static_cast<std::size_t>(maxd) + 1);
    for (std::int64_t i = static_cast<std::int64_t>(G.topo.size()) - 1; i >= 0; --i)
    {
        const std::int64_t f = G.topo[static_cast<std::size_t>(i)];
        levels[static_cast<std::size_t>(depth[f])].push_back(f);
    }
    return levels;
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------------------
// oracle_fill_pits: fill_pits(raster, min_slope, bc, n_threads, binary_heap)
// (src/cpu/lsdtt_raster_flow_preprocessing_cpu.cpp:727-782). min_slope <= 0
// runs the flood with a zero rise, which the reference documents as bitwise
// equal to its reconstruction backend (docs/design_and_algorithms/
// flow_routing.md:603-620).
// ---------------------------------------------------------------------------
int oracle_fill_pits_traced_ties(const float* z, const std::uint8_t* mask, int nr, int nc, double cell, double nodata,
                                 const char* bc, float min_slope, float* out, std::int64_t* discoverer,
                                 std::int64_t* order, std::uint8_t* via_fifo, int index_ties, char* err, int errlen)
{
    try
    {
        if (!(nr > 0 && nc > 0 && cell > 0.0)) throw std::runtime_error("lsdtt::fill_pits: invalid raster metadata");
        const std::string b = bc ? bc : "";
        auto is_p = [&](std::size_t i) { return b.size() > i && (b[i] == 'p' || b[i] == 'P'); };
        const bool per_ns = is_p(0), per_ew = is_p(1);
        if (per_ns != is_p(2))
            throw std::runtime_error("lsdtt::fill_pits: north and south periodic flags must match (boundary_conditions '" + b + "')");
        if (per_ew != is_p(3))
            throw std::runtime_error("lsdtt::fill_pits: east and west periodic flags must match (boundary_conditions '" + b + "')");
        if (per_ns && per_ew)
            throw std::runtime_error("lsdtt::fill_pits: boundary_conditions '" + b +
                                     "' is periodic in BOTH directions, so the grid has no drainage exit at all and every "
                                     "cell would fill to the global maximum. Leave one pair open.");
        const std::size_t n = static_cast<std::size_t>(nr) * nc;
        std::vector<float> dem(n);
        std::vector<int> idx(n);
        const float ndv = static_cast<float>(nodata);
        for (std::size_t k = 0; k < n; ++k)
        {
            if (mask[k] != 0 && !is_nodata(z[k], nodata)) { dem[k] = z[k]; idx[k] = kOpen; }
            else { dem[k] = ndv; idx[k] = kNoCell; }
        }
        FillTrace tr{discoverer, order, via_fifo};
        if (discoverer) std::fill(discoverer, discoverer + n, static_cast<std::int64_t>(-2));
        if (order) std::fill(order, order + n, static_cast<std::int64_t>(-1));
        priority_flood(dem, idx, nr, nc, static_cast<float>(cell), min_slope > 0.0f ? min_slope : 0.0f, per_ns, per_ew, tr,
                       index_ties != 0);
        std::memcpy(out, dem.data(), sizeof(float) * n);
        return 0;
    }
    catch (const std::exception& e) { put_err(err, errlen, e.what()); return 1; }
}

int oracle_fill_pits_traced(const float* z, const std::uint8_t* mask, int nr, int nc, double cell, double nodata,
                            const char* bc, float min_slope, float* out, std::int64_t* discoverer,
                            std::int64_t* order, std::uint8_t* via_fifo, char* err, int errlen)
{
    return oracle_fill_pits_traced_ties(z, mask, nr, nc, cell, nodata, bc, min_slope, out, discoverer, order, via_fifo,
                                        0, err, errlen);
}

int oracle_fill_pits(const float* z, const std::uint8_t* mask, int nr, int nc, double cell, double nodata,
                     const char* bc, float min_slope, int /*radix_queue*/, float* out, char* err, int errlen)
{
    return oracle_fill_pits_traced(z, mask, nr, nc, cell, nodata, bc, min_slope, out, nullptr, nullptr, nullptr, err,
                                   errlen);
}

// The fill with heap ties taken in (row, col) order (NodeGreater).
int oracle_fill_pits_index_ties(const float* z, const std::uint8_t* mask, int nr, int nc, double cell, double nodata,
                                const char* bc, float min_slope, float* out, char* err, int errlen)
{
    return oracle_fill_pits_traced_ties(z, mask, nr, nc, cell, nodata, bc, min_slope, out, nullptr, nullptr, nullptr,
                                        1, err, errlen);
}

// ---------------------------------------------------------------------------
// oracle_flowinfo: lsdtt_flowinfo::create (src/cpu/lsdtt_flowinfo_cpu.cpp:
// 197-253) and every component tests/cpp/test_flow_d8_identity.cpp pins.
// Same argument layout as ref_flowinfo in oracle/ref_shim.cpp.
// ---------------------------------------------------------------------------
int oracle_flowinfo(const float* z, const std::uint8_t* mask, int nr, int nc, double cell, double nodata,
                    const char* bc, int interior_nodata_is_outlet, int allow_pits_as_outlets, int build_topo,
                    int build_sv, int require_acyclic, const std::int64_t* forced, std::int64_t n_forced,
                    int n_threads, std::int64_t* receiver, std::uint8_t* dir, std::uint8_t* donors,
                    std::int64_t* outlets, std::int64_t* n_outlets, std::int64_t* topo, std::int64_t* n_topo,
                    std::int64_t* svec, std::int64_t* sv_start, std::uint64_t* sv_size, std::int32_t* flags,
                    const double* weights, double* accum, char* err, int errlen)
{
    try
    {
        FlowOpts o;
        o.bc = parse_bc(bc);
        o.interior_nodata_is_outlet = interior_nodata_is_outlet != 0;
        o.allow_pits_as_outlets = allow_pits_as_outlets != 0;
        o.build_topo = build_topo != 0;
        o.build_sv = build_sv != 0;
        o.require_acyclic = require_acyclic != 0;
        o.n_threads = n_threads;
        Flow F = build_flow(z, mask, nr, nc, cell, nodata, o, forced, n_forced);
        const std::size_t n = static_cast<std::size_t>(nr) * nc;
        std::memcpy(receiver, F.receiver.data(), sizeof(std::int64_t) * n);
        std::memcpy(dir, F.dir.data(), n);
        std::memcpy(donors, F.donors.data(), n);
        *n_outlets = static_cast<std::int64_t>(F.outlets.size());
        std::memcpy(outlets, F.outlets.data(), sizeof(std::int64_t) * F.outlets.size());
        // The topological order is kept only when asked for (:240-247).
        const bool keep_topo = F.has_topo && o.build_topo;
        flags[0] = keep_topo ? 1 : 0;
        flags[1] = F.has_sv ? 1 : 0;
        *n_topo = 0;
        if (keep_topo)
        {
            *n_topo = static_cast<std::int64_t>(F.topo.size());
            std::memcpy(topo, F.topo.data(), sizeof(std::int64_t) * F.topo.size());
        }
        if (F.has_sv)
        {
            // The outlets' slices, concatenated in outlet order, ARE the
            // s-vector: each outlet's DFS appends a contiguous block.
            std::memcpy(svec, F.svec.data(), sizeof(std::int64_t) * F.svec.size());
            std::memcpy(sv_start, F.sv_start.data(), sizeof(std::int64_t) * n);
            std::memcpy(sv_size, F.sv_size.data(), sizeof(std::uint64_t) * n);
        }
        if (accum && keep_topo)
        {
            const std::vector<double> a = accumulate(F, weights);
            std::memcpy(accum, a.data(), sizeof(double) * n);
        }
        return 0;
    }
    catch (const std::exception& e) { put_err(err, errlen, e.what()); return 1; }
}

// ---------------------------------------------------------------------------
// oracle_flow_query: the lsdtt_flow_base query rasters built on the stack
// (src/cpu/lsdtt_flowinfo_cpu.cpp:2255-2965), on a flow object built with
// pits as outlets. kind:
//   0 get_distance_from_outlet_raster                    (:2255-2302)
//   1 get_height_above_channel_raster(elev, emask, thr)  (:2309-2382)
//   2 get_height_above_channel_mask_donor_raster(elev, emask, channel_mask)
//                                                        (:2407-2474; donor out)
//   3 get_distance_to_channel_raster(thr)                (:2482-2553)
//   4 get_height_to_farthest_ridge_raster(elev, emask)   (:2571-2649)
//   5 get_distance_to_farthest_ridge_raster()            (:2651-2713)
//   6 get_downstream_path_sum_raster(values, vmask, sink_mask) (:2721-2791)
//   7 get_upslope_sum_raster(values, vmask, include_self)      (:2800-2868)
//   8 get_upslope_mean_raster(values, vmask, include_self)     (:2876-2960)
// The passes run over the s-vector in the reference's order (forward =
// receiver before donor, reverse = donors before receiver) with its double
// accumulators and float outputs.
// ---------------------------------------------------------------------------
int oracle_flow_query(const float* z, const std::uint8_t* mask, int nr, int nc, double cell, double nodata,
                      const char* bc, int kind, const float* values, const std::uint8_t* vmask,
                      const std::uint8_t* cmask, int threshold, int include_self, float* out,
                      std::uint8_t* out_mask, std::int64_t* donor_out, char* err, int errlen)
{
    try
    {
        FlowOpts o;
        o.bc = parse_bc(bc);
        o.allow_pits_as_outlets = true;
        Flow F = build_flow(z, mask, nr, nc, cell, nodata, o, nullptr, 0);
        const std::size_t n = static_cast<std::size_t>(nr) * nc;
        const float ndv = static_cast<float>(nodata);
        const double dx = cell, dxy = cell * kSqrt2d;
        const std::vector<std::int64_t>& sv = F.svec;
        auto step_of = [&](std::int64_t f) {
            const std::uint8_t d = F.dir[f];
            return (d == 255u || d % 2u == 0u) ? dx : dxy;
        };
        auto dist_outlet = [&]() {
            std::vector<double> d(n, 0.0);
            for (const std::int64_t f : sv)
            {
                const std::int64_t r = F.receiver[f];
                if (r == -2) continue;
                d[f] = d[r] + step_of(f);
            }
            return d;
        };
        for (std::size_t i = 0; i < n; ++i) { out[i] = ndv; out_mask[i] = 0; }
        if (kind == 0)
        {
            const std::vector<double> d = dist_outlet();
            for (std::size_t i = 0; i < n; ++i)
                if (mask[i]) { out[i] = static_cast<float>(d[i]); out_mask[i] = 1; }
        }
        else if (kind == 1 || kind == 2)
        {
            std::vector<float> ch(n, 0.0f);
            std::vector<std::int64_t> donor(n, -1);
            for (const std::int64_t f : sv)
            {
                if (!mask[f] || !vmask[f]) continue;
                const bool is_ch = kind == 1 ? static_cast<std::int64_t>(F.sv_size[f]) >= threshold : cmask[f] != 0;
                if (is_ch) { ch[f] = values[f]; donor[f] = f; }
                else
                {
                    const std::int64_t r = F.receiver[f];
                    if (r != -2 && donor[r] >= 0) { ch[f] = ch[r]; donor[f] = donor[r]; }
                }
            }
            for (std::size_t i = 0; i < n; ++i)
                if (mask[i] && vmask[i] && donor[i] >= 0) { out[i] = values[i] - ch[i]; out_mask[i] = 1; }
            if (donor_out) std::memcpy(donor_out, donor.data(), sizeof(std::int64_t) * n);
        }
        else if (kind == 3)
        {
            std::vector<double> d(n, 0.0);
            std::vector<std::uint8_t> ok(n, 0);
            auto is_ch = [&](std::int64_t f) { return static_cast<std::int64_t>(F.sv_size[f]) >= threshold; };
            for (const std::int64_t f : sv)
            {
                if (!mask[f]) continue;
                if (is_ch(f)) { d[f] = 0.0; ok[f] = 1; continue; }
                const std::int64_t r = F.receiver[f];
                if (r == -2) continue;
                if (is_ch(r)) { d[f] = step_of(f); ok[f] = 1; }
                else if (ok[r]) { d[f] = step_of(f) + d[r]; ok[f] = 1; }
            }
            for (std::size_t i = 0; i < n; ++i)
                if (mask[i] && ok[i]) { out[i] = static_cast<float>(d[i]); out_mask[i] = 1; }
        }
        else if (kind == 4 || kind == 5)
        {
            const std::vector<double> d = dist_outlet();
            std::vector<double> up(d);
            std::vector<float> fe(n, 0.0f);
            if (kind == 4)
                for (std::size_t i = 0; i < n; ++i) fe[i] = (mask[i] && vmask[i]) ? values[i] : 0.0f;
            for (std::int64_t i = static_cast<std::int64_t>(sv.size()) - 1; i >= 0; --i)
            {
                const std::int64_t f = sv[static_cast<std::size_t>(i)];
                const std::int64_t r = F.receiver[f];
                if (r == -2) continue;
                if (up[f] > up[r]) { up[r] = up[f]; fe[r] = fe[f]; }
            }
            for (std::size_t i = 0; i < n; ++i)
            {
                if (!mask[i]) continue;
                if (kind == 4)
                {
                    if (!vmask[i]) continue;
                    out[i] = fe[i] - values[i];
                }
                else
                    out[i] = static_cast<float>(up[i] - d[i]);
                out_mask[i] = 1;
            }
        }
        else if (kind == 6)
        {
            std::vector<double> acc(n, 0.0);
            for (const std::int64_t f : sv)
            {
                if (!mask[f]) continue;
                if (cmask[f]) { acc[f] = 0.0; continue; }
                const double own = vmask[f] ? static_cast<double>(values[f]) : 0.0;
                const std::int64_t r = F.receiver[f];
                const bool terminal = r == -2 || cmask[r] != 0;
                acc[f] = terminal ? own : own + acc[r];
            }
            for (std::size_t i = 0; i < n; ++i)
                if (mask[i] && !cmask[i]) { out[i] = static_cast<float>(acc[i]); out_mask[i] = 1; }
        }
        else if (kind == 7 || kind == 8)
        {
            std::vector<double> sum(n, 0.0);
            std::vector<std::int64_t> cnt(n, 0);
            for (std::size_t i = 0; i < n; ++i)
                if (mask[i] && include_self && vmask[i]) { sum[i] = values[i]; cnt[i] = 1; }
            for (std::int64_t i = static_cast<std::int64_t>(sv.size()) - 1; i >= 0; --i)
            {
                const std::int64_t f = sv[static_cast<std::size_t>(i)];
                const std::int64_t r = F.receiver[f];
                if (r == -2) continue;
                sum[r] += sum[f];
                cnt[r] += cnt[f];
            }
            for (std::size_t i = 0; i < n; ++i)
            {
                if (!mask[i]) continue;
                if (kind == 7) { out[i] = static_cast<float>(sum[i]); out_mask[i] = 1; }
                else if (cnt[i] > 0)
                {
                    out[i] = static_cast<float>(sum[i] / static_cast<double>(cnt[i]));
                    out_mask[i] = 1;
                }
            }
        }
        else
            throw std::invalid_argument("oracle_flow_query: unknown kind");
        return 0;
    }
    catch (const std::exception& e) { put_err(err, errlen, e.what()); return 1; }
}

// ---------------------------------------------------------------------------
// oracle_stream_power: compute_d8_stream_power_incision
// (src/cpu/lsdtt_stream_power_cpu.cpp:159-326) on a flow object built as
// run_lem_step builds it (src/cpu/lsdtt_lem_cpu.cpp:329-339), moving-average
// kernel 1 (identity), no width correction.
// ---------------------------------------------------------------------------
int oracle_stream_power(const float* z, const std::uint8_t* mask, int nr, int nc, double cell, double nodata,
                        const char* bc, float K, float m, float n_exp, float dt, float threshold_area,
                        int divide_area_by_dx, float slope_clamp, const float* k_field, float* out, char* err,
                        int errlen)
{
    try
    {
        FlowOpts o;
        o.bc = parse_bc(bc);
        o.interior_nodata_is_outlet = true;
        o.allow_pits_as_outlets = true;
        const Flow F = build_flow(z, mask, nr, nc, cell, nodata, o, nullptr, 0);
        const std::int64_t ncell = static_cast<std::int64_t>(nr) * nc;
        const float dx = static_cast<float>(cell);
        const float dx_diag = dx * kSqrt2f;
        std::vector<float> zz(z, z + ncell);
        const std::vector<double> area_d = accumulate(F, nullptr);
        const bool n_is_one = std::abs(n_exp - 1.0f) < 1e-6f;
        const double width_factor = 1.0;
        for (std::int64_t ti = static_cast<std::int64_t>(F.topo.size()) - 1; ti >= 0; --ti)
        {
            const std::int64_t flat = F.topo[static_cast<std::size_t>(ti)];
            const std::int64_t recv = F.receiver[flat];
            if (recv == kOutletReceiver || !F.mask[flat]) continue;
            if (recv < 0 || recv >= ncell) continue;
            const std::uint8_t d = F.dir[flat];
            const float dx_eff = (d & 1u) ? dx_diag : dx;
            double area = area_d[flat];
            if (divide_area_by_dx) area /= dx;
            if (threshold_area > 0.0f && area < static_cast<double>(threshold_area)) continue;
            const float z_old = z[flat];
            const float z_r = zz[recv];
            float z_new = z_old;
            if (z_r >= z_old) continue;
            const double tol = static_cast<double>(slope_clamp) * dx_eff;
            const float Ki = k_field ? k_field[flat] : K;
            const double kam = static_cast<double>(Ki) * width_factor * std::pow(area, static_cast<double>(m));
            if (n_is_one)
            {
                const double spf = kam * (dt / dx_eff);
                z_new = static_cast<float>((z_old + z_r * spf) / (1.0 + spf));
                if ((z_new - z_old) > static_cast<float>(tol) || std::isnan(z_new)) z_new = z_old;
            }
            else
            {
                double eps = tol + 1.0;
                int it = 0;
                do
                {
                    const double slope = (z_new - z_r) / dx_eff;
                    if (slope <= 0.0) eps = 0.0;
                    else
                    {
                        const double fz = z_new - z_old + kam * dt * std::pow(slope, n_exp);
                        const double fdz = 1.0 + kam * dt * (n_exp / dx_eff) * std::pow(slope, n_exp - 1.0);
                        eps = fz / fdz;
                    }
                    z_new -= static_cast<float>(eps);
                    ++it;
                    if (it > 100) eps = tol / 2.0;
                } while (std::abs(eps) > tol);
                if ((z_new - z_old) > static_cast<float>(tol) || std::isnan(z_new)) z_new = z_old;
                if (z_new < z_r) z_new = static_cast<float>(z_r + slope_clamp * dx_eff);
            }
            zz[flat] = z_new;
        }
        std::memcpy(out, zz.data(), sizeof(float) * ncell);
        return 0;
    }
    catch (const std::exception& e) { put_err(err, errlen, e.what()); return 1; }
}

// ---------------------------------------------------------------------------
// oracle_boundary_flats: build_boundary_flats (src/cpu/lsdtt_lem_cpu.cpp:735-808)
// ---------------------------------------------------------------------------
std::int64_t oracle_boundary_flats(const std::uint8_t* mask, int nr, int nc, const char* bc, std::int64_t* out)
{
    const std::string b = bc ? bc : "";
    auto fixed = [&](std::size_t i) { return b.size() > i && (b[i] == 'o' || b[i] == 'b'); };
    const bool fn = fixed(0), fe = fixed(1), fs = fixed(2), fw = fixed(3);
    std::int64_t k = 0;
    for (int r = 0; r < nr; ++r)
        for (int c = 0; c < nc; ++c)
        {
            const std::int64_t f = static_cast<std::int64_t>(r) * nc + c;
            if (!mask[f]) continue;
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
            if (edge) out[k++] = f;
        }
    return k;
}

// ---------------------------------------------------------------------------
// oracle_lem_finish: the end of run_lem_step (src/cpu/lsdtt_lem_cpu.cpp:
// 611-731) -- uplift on valid cells, restore the boundary flats to their
// pre-step value minus base-level fall, then the step statistics.
// z is updated in place; z_before is the step's input surface.
// stats: delta_max, delta_mean, max_local, p999_local, mean_erosion, max_erosion.
// ---------------------------------------------------------------------------
void oracle_lem_finish(float* z, const float* z_before, const std::uint8_t* mask, std::int64_t n, float U, float dt,
                       float baselevel_fall, const std::int64_t* bflats, std::int64_t n_bf, float* stats)
{
    const float uplift_dz = U * dt;
    for (std::int64_t i = 0; i < n; ++i)
        if (mask[i]) z[i] += uplift_dz;
    const float bl = baselevel_fall * dt;
    for (std::int64_t i = 0; i < n_bf; ++i)
        if (bflats[i] >= 0 && bflats[i] < n) z[bflats[i]] = z_before[bflats[i]] - bl;
    double sb = 0.0, sa = 0.0, mb = -1e30, ma = -1e30, ml = 0.0, se = 0.0, me = 0.0;
    std::vector<float> lc;
    lc.reserve(static_cast<std::size_t>(n));
    std::int64_t nv = 0;
    const double udz = static_cast<double>(U * dt);
    for (std::int64_t i = 0; i < n; ++i)
    {
        if (!mask[i]) continue;
        ++nv;
        const double zb = z_before[i], za = z[i];
        sb += zb;
        sa += za;
        mb = std::max(mb, zb);
        ma = std::max(ma, za);
        const double d = std::abs(za - zb);
        ml = std::max(ml, d);
        lc.push_back(static_cast<float>(d));
        const double ero = zb - (za - udz);
        if (ero > 0.0) { se += ero; me = std::max(me, ero); }
    }
    const double inv_dt = 1.0 / static_cast<double>(dt);
    const double inv_n = nv > 0 ? 1.0 / static_cast<double>(nv) : 0.0;
    stats[0] = static_cast<float>(std::abs(ma - mb));
    stats[1] = static_cast<float>(std::abs((sa - sb) * inv_n));
    stats[2] = static_cast<float>(ml);
    if (!lc.empty())
    {
        // compute_quantile_floor_in_place (src/utils/lsdtt_statistics.cpp:420-429):
        // the order statistic at floor(q*(n-1)).
        std::size_t k = static_cast<std::size_t>(0.999 * static_cast<double>(lc.size() - 1));
        k = std::min(k, lc.size() - 1);
        std::nth_element(lc.begin(), lc.begin() + static_cast<std::ptrdiff_t>(k), lc.end());
        stats[3] = lc[k];
    }
    else
        stats[3] = 0.0f;
    stats[4] = static_cast<float>(se * inv_n * inv_dt);
    stats[5] = static_cast<float>(me * inv_dt);
}

// ---------------------------------------------------------------------------
// oracle_noise_tilt_surface: generate_uniform_random_noise_surface followed by
// superimpose_open_boundary_gradient (src/cpu/lsdtt_raster_synthetic_surfaces_
// cpu.cpp:118-147, 359-459). The noise is a splitmix64 hash of
// (seed, tag, row, col, 0, 0) mapped to [0,1) by its top 53 bits.
// ---------------------------------------------------------------------------
int oracle_noise_tilt_surface(int nr, int nc, double cell, int seed, double lo, double hi, const char* bc,
                              float slope, float* out, char* /*err*/, int /*errlen*/)
{
    const double span = hi - lo;
    const std::uint64_t tag = 0x554E49464F524DULL;
    for (int r = 0; r < nr; ++r)
        for (int c = 0; c < nc; ++c)
        {
            std::uint64_t h = splitmix64(static_cast<std::uint64_t>(static_cast<std::uint32_t>(seed)));
            h = mix_in(h, tag);
            h = mix_in(h, static_cast<std::uint64_t>(r));
            h = mix_in(h, static_cast<std::uint64_t>(c));
            h = mix_in(h, 0);
            h = mix_in(h, 0);
            const std::uint64_t key = splitmix64(h);
            const double u = static_cast<double>(key >> 11) * (1.0 / 9007199254740992.0);
            out[static_cast<std::size_t>(r) * nc + c] = static_cast<float>(lo + span * u);
        }
    const std::string b = bc ? bc : "";
    auto open = [&](std::size_t i) { return b.size() > i && (b[i] == 'o' || b[i] == 'b'); };
    const bool on = open(0), oe = open(1), os = open(2), ow = open(3);
    if (slope == 0.0f || !(on || oe || os || ow)) return 0;
    const float dx = static_cast<float>(cell);
    for (int r = 0; r < nr; ++r)
        for (int c = 0; c < nc; ++c)
        {
            int d = nr + nc;
            if (on) d = std::min(d, r);
            if (oe) d = std::min(d, nc - 1 - c);
            if (os) d = std::min(d, nr - 1 - r);
            if (ow) d = std::min(d, c);
            out[static_cast<std::size_t>(r) * nc + c] += slope * dx * static_cast<float>(d);
        }
    return 0;
}

// ---------------------------------------------------------------------------
// oracle_dinf_graph: the D-infinity graph of lsdtt_flowgraph_cpu
// (flowgraph_cpu.cpp:423-662, 874-985): per cell up to two receivers
// (-1 none) and their weights, the receiver count, the facet slope and
// bearing rasters (nodata where a cell has no receiver), unique-donor counts
// and the topological order (n_topo entries).
// ---------------------------------------------------------------------------
int oracle_dinf_graph(const float* z, const std::uint8_t* mask, int nr, int nc, double cell, double nodata,
                      const char* bc, int interior_nodata_is_outlet, std::int64_t* rec, float* w,
                      std::uint8_t* nrec, float* slope, float* bearing, std::uint8_t* donors, std::int64_t* topo,
                      std::int64_t* n_topo, char* err, int errlen)
{
    try
    {
        const Dinf G = build_dinf_graph(z, mask, nr, nc, cell, nodata, bc, interior_nodata_is_outlet != 0);
        const std::size_t n = static_cast<std::size_t>(nr) * nc;
        std::memcpy(rec, G.rec.data(), sizeof(std::int64_t) * 2 * n);
        std::memcpy(w, G.w.data(), sizeof(float) * 2 * n);
        std::memcpy(nrec, G.nrec.data(), n);
        std::memcpy(slope, G.slope.data(), sizeof(float) * n);
        std::memcpy(bearing, G.bearing.data(), sizeof(float) * n);
        std::memcpy(donors, G.donors.data(), n);
        *n_topo = static_cast<std::int64_t>(G.topo.size());
        std::memcpy(topo, G.topo.data(), sizeof(std::int64_t) * G.topo.size());
        return 0;
    }
    catch (const std::exception& e) { put_err(err, errlen, e.what()); return 1; }
}

int oracle_dinf_accumulate(const float* z, const std::uint8_t* mask, int nr, int nc, double cell, double nodata,
                           const char* bc, const double* weights, double* out, char* err, int errlen)
{
    try
    {
        const Dinf G = build_dinf_graph(z, mask, nr, nc, cell, nodata, bc, true);
        const std::vector<double> a = dinf_accumulate(G, weights);
        std::memcpy(out, a.data(), sizeof(double) * a.size());
        return 0;
    }
    catch (const std::exception& e) { put_err(err, errlen, e.what()); return 1; }
}

// compute_dinf_stream_power_incision (stream_power_cpu.cpp:329-602) with the
// identity area smoothing and no width correction.
int oracle_dinf_stream_power(const float* z, const std::uint8_t* mask, int nr, int nc, double cell, double nodata,
                             const char* bc, float K, float m, float n, float dt, float threshold_area,
                             int divide_area_by_dx, float slope_clamp, float* out, char* err, int errlen)
{
    try
    {
        const Dinf G = build_dinf_graph(z, mask, nr, nc, cell, nodata, bc, true);
        const std::size_t cells = static_cast<std::size_t>(nr) * nc;
        std::vector<float> zz(z, z + cells);
        const float dxc = static_cast<float>(cell);
        const float dxd = static_cast<float>(cell) * kSqrt2f;
        const std::vector<double> area_d = dinf_accumulate(G, nullptr);
        const auto levels = dinf_reverse_levels(G);
        const bool n_is_one = std::abs(n - 1.0f) < 1e-6f;
        for (const auto& level : levels)
            for (const std::int64_t f : level)
            {
                if (!G.valid[f] || G.nrec[f] == 0) continue;
                double area = area_d[f];
                if (divide_area_by_dx) area /= dxc;
                if (threshold_area > 0.0f && area < static_cast<double>(threshold_area)) continue;
                const float zo = z[f];
                float zn = zo;
                const int nrc = G.nrec[f];
                const float w0 = nrc > 0 ? G.w[2 * f] : 0.0f;
                const float w1 = nrc > 1 ? G.w[2 * f + 1] : 0.0f;
                const bool only_card = nrc == 1 || w0 >= 1.0f - 1e-6f;
                const bool only_diag = nrc > 1 && w1 >= 1.0f - 1e-6f;
                const bool two = nrc > 1 && !only_card && !only_diag;
                auto recv = [&](int k) -> float {
                    if (k >= nrc) return zo;
                    const std::int64_t i = G.rec[2 * f + k];
                    if (i < 0 || i >= static_cast<std::int64_t>(cells)) return zo;
                    return zz[i];
                };
                const float ze1 = recv(0), ze2 = recv(1);
                const double kam = static_cast<double>(K) * 1.0 * std::pow(area, static_cast<double>(m));
                const double tol = static_cast<double>(slope_clamp) * dxc;
                if (two)
                {
                    double eps = tol + 1.0;
                    int it = 0;
                    do
                    {
                        const double sbt = std::pow((ze1 - zn) / dxc, 2.0) + std::pow((ze2 - ze1) / dxc, 2.0);
                        if (sbt <= 0.0) eps = 0.0;
                        else
                        {
                            const double fz = zn - zo + kam * std::pow(sbt, 0.5 * n) * dt;
                            const double fdz =
                                1.0 - kam * n * (ze1 - zn) / (dxc * dxc) * std::pow(sbt, 0.5 * n - 1.0) * dt;
                            eps = fz / fdz;
                        }
                        zn -= static_cast<float>(eps);
                        ++it;
                        if (it > 100) eps = tol / 2.0;
                    } while (std::abs(eps) > tol);
                    if ((zn - zo) > static_cast<float>(tol) || std::isnan(zn)) zn = zo;
                    const float zmin = std::min(ze1, ze2);
                    if (zn < zmin) zn = zmin + slope_clamp * dxc;
                }
                else
                {
                    const float zr = only_diag ? ze2 : ze1;
                    const float dxe = only_diag ? dxd : dxc;
                    if (zr >= zo) zn = zo;
                    else if (n_is_one)
                    {
                        const double spf = kam * (dt / dxe);
                        zn = static_cast<float>((zo + zr * spf) / (1.0 + spf));
                        if ((zn - zo) > static_cast<float>(tol) || std::isnan(zn)) zn = zo;
                    }
                    else
                    {
                        double eps = tol + 1.0;
                        int it = 0;
                        do
                        {
                            const double slope = (zn - zr) / dxe;
                            if (slope <= 0.0) eps = 0.0;
                            else
                            {
                                const double fz = zn - zo + kam * dt * std::pow(slope, n);
                                const double fdz = 1.0 + kam * dt * (n / dxe) * std::pow(slope, n - 1.0);
                                eps = fz / fdz;
                            }
                            zn -= static_cast<float>(eps);
                            ++it;
                            if (it > 100) eps = tol / 2.0;
                        } while (std::abs(eps) > tol);
                        if ((zn - zo) > static_cast<float>(tol) || std::isnan(zn)) zn = zo;
                        if (zn < zr) zn = static_cast<float>(zr + slope_clamp * dxe);
                    }
                }
                zz[f] = zn;
            }
        std::memcpy(out, zz.data(), sizeof(float) * cells);
        return 0;
    }
    catch (const std::exception& e) { put_err(err, errlen, e.what()); return 1; }
}

}  // extern "C"
