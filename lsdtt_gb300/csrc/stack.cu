// stack.cu -- s-vector, contributing-cell counts, depths, heights and the
// Kahn topological order of the D8 receiver forest, all without a
// level-by-level sweep.
//
// 1. Euler tour. The reference's s-vector (src/cpu/lsdtt_flowinfo_cpu.cpp:
//    1544-1731) is a DFS preorder from each outlet in row-major order with
//    donors visited in ascending flat index. That preorder is the order of
//    "enter" events on the Euler tour of the forest whose children lists are
//    sorted ascending and whose trees are chained in outlet order. Each valid
//    cell c owns two tour nodes, enter(c) = 2c and exit(c) = 2c+1, and the
//    successor of every node follows from first child / next sibling /
//    parent / next outlet.
// 2. List ranking by a sparse ruling set: every 64th node (plus the head)
//    starts a walk to the next ruler, the rulers' list is ranked
//    recursively, then every node adds its ruler's rank. With weights
//    (enter: +1, exit: 0) the prefix is the preorder index; with (+1, -1)
//    it is the depth. s_vector_start = prefix at enter, s_vector_size =
//    prefix at exit - prefix at enter, depth = signed prefix at enter.
// 3. Kahn order (build_topological_order, :1428-1522). The FIFO processes
//    level L_k (cells whose longest path from a headwater is k) before
//    L_{k+1}, and L_{k+1} is the list of receivers pushed by L_k in L_k
//    order, each pushed by its last-processed donor. By induction the order
//    inside every level is the order of the flat index of a single
//    headwater per cell: the deepest headwater of its subtree, the largest
//    flat index among equally deep ones. Both the height and that headwater
//    are one range-max over the cell's s-vector interval of the key
//    (depth << 32 | flat). The order is then a stable radix sort by
//    (height, headwater).

#include <cmath>
#include <cstdlib>

#include "engine.cuh"

namespace lsdtt_gb300
{
namespace
{

constexpr std::uint32_t kEnd = 0xffffffffu;
constexpr std::uint32_t kNone = 0xffffffffu;
constexpr unsigned kErrCycle = 5;
// Mean sublist length of the ruling set (a power of two). The first level's
// walk is bound by its longest sublist, ~kRuler ln(#rulers) dependent steps;
// a smaller kRuler shortens it but adds rulers and levels. Of 16, 32 and 64,
// 32 gave the fastest s-vector on an 89.5 M-cell ensemble. The ruler
// buffers take 24 B per ruler, sized for four times the mean count.
constexpr int kRuler = 32;
constexpr int kSerialLimit = 96;  // rank lists this short with one thread

__device__ __forceinline__ bool is_ruler(std::uint32_t v)
{
    // Spread rulers pseudo-randomly so sublists stay short on any layout.
    std::uint32_t h = v * 0x9E3779B1u;
    h ^= h >> 15;
    return (h & (kRuler - 1)) == 0;
}

// Sorted donor list of a valid cell: ascending flat index, de-duplicated
// (a donor matches exactly one direction, see donors_kernel).
__device__ int donor_list(const Grid& g, const std::uint8_t* __restrict__ mask, const std::uint8_t* __restrict__ dir,
                          std::int64_t flat, std::int64_t out[8])
{
    const int row = static_cast<int>(flat / g.nc), col = static_cast<int>(flat % g.nc);
    int k = 0;
    if (is_interior(g, row, col))
    {
        // NW, N, NE, W, E, SW, S, SE: ascending flat order; code of each and
        // the code that points back (opposite).
        const int order[8] = {7, 0, 1, 6, 2, 5, 4, 3};
#pragma unroll
        for (int i = 0; i < 8; ++i)
        {
            const int d = order[i];
            const std::int64_t nf = flat + static_cast<std::int64_t>(d8_dr(d)) * g.nc + d8_dc(d);
            if (mask[nf] && dir[nf] == ((d + 4) & 7)) out[k++] = nf;
        }
        return k;
    }
    for (int d = 0; d < 8; ++d)
    {
        const Step s = resolve_step(g, row, col, d);
        if (s.kind != 1) continue;
        const std::int64_t nf = static_cast<std::int64_t>(s.r) * g.nc + s.c;
        if (nf == flat || !mask[nf] || dir[nf] != ((d + 4) & 7)) continue;
        bool dup = false;
        for (int i = 0; i < k; ++i) dup |= (out[i] == nf);
        if (!dup) out[k++] = nf;
    }
    for (int i = 1; i < k; ++i)
    {
        const std::int64_t key = out[i];
        int j = i;
        while (j > 0 && out[j - 1] > key) { out[j] = out[j - 1]; --j; }
        out[j] = key;
    }
    return k;
}

// first child / next sibling links of the cell at `flat` (an index into the
// grid g's planes; written links get `base` added). next_sibling of each
// donor is written by its (unique) receiver. Interior cells scan their eight
// neighbours in ascending flat order (NW, N, NE, W, E, SW, S, SE) and chain
// the donors as they are found; edge cells take donor_list.
__device__ __forceinline__ void link_cell(const Grid& g, const std::uint8_t* __restrict__ mask,
                                          const std::uint8_t* __restrict__ dir, std::int64_t flat, std::int64_t base,
                                          std::uint32_t* __restrict__ first_child,
                                          std::uint32_t* __restrict__ next_sib)
{
    const int row = static_cast<int>(flat / g.nc), col = static_cast<int>(flat % g.nc);
    std::uint32_t first = kNone, prev = kNone;
    auto chain = [&](std::int64_t nf) {
        const std::uint32_t v = static_cast<std::uint32_t>(base + nf);
        if (prev == kNone) first = v;
        else next_sib[prev] = v;
        prev = v;
    };
    if (is_interior(g, row, col))
    {
        const int order[8] = {7, 0, 1, 6, 2, 5, 4, 3};  // the codes of NW, N, NE, W, E, SW, S, SE
#pragma unroll
        for (int i = 0; i < 8; ++i)
        {
            const int d = order[i];
            const std::int64_t nf = flat + static_cast<std::int64_t>(d8_dr(d)) * g.nc + d8_dc(d);
            if (mask[nf] && dir[nf] == ((d + 4) & 7)) chain(nf);
        }
    }
    else
    {
        std::int64_t d[8];
        const int k = donor_list(g, mask, dir, flat, d);
        for (int i = 0; i < k; ++i) chain(d[i]);
    }
    first_child[base + flat] = first;
    if (prev != kNone) next_sib[prev] = kNone;
}

__global__ void links_kernel(Grid g, const std::uint8_t* __restrict__ mask, const std::uint8_t* __restrict__ dir,
                             std::uint32_t* __restrict__ first_child, std::uint32_t* __restrict__ next_sib)
{
    LSDTT_COUNT();
    const std::int64_t flat = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (flat >= g.n || !mask[flat]) return;
    link_cell(g, mask, dir, flat, 0, first_child, next_sib);
}

// links_kernel for a packed ensemble: each member's donors in its own
// geometry, written as packed indices. Blocks are kPackAlign cells, so each
// lies in one member.
__global__ void links_packed(Packed P, const std::uint8_t* __restrict__ mask, const std::uint8_t* __restrict__ dir,
                             std::uint32_t* __restrict__ first_child, std::uint32_t* __restrict__ next_sib)
{
    LSDTT_COUNT();
    const std::int64_t flat = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (flat >= P.n || !mask[flat]) return;
    const PackedMember& M = P.m[P.blk_member[blockIdx.x]];
    const std::int64_t local = flat - M.base;
    if (local >= static_cast<std::int64_t>(M.nr) * M.nc) return;
    link_cell(member_grid(M), mask + M.base, dir + M.base, local, M.base, first_child, next_sib);
}

__global__ void root_links_kernel(const std::int64_t* __restrict__ outlets, const std::int64_t* __restrict__ n_out,
                                  std::uint32_t* __restrict__ next_sib, std::uint32_t* __restrict__ head)
{
    LSDTT_COUNT();
    const std::int64_t n = *n_out;
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i == 0) *head = n > 0 ? static_cast<std::uint32_t>(2 * outlets[0]) : kEnd;
    if (i < n) next_sib[outlets[i]] = (i + 1 < n) ? static_cast<std::uint32_t>(outlets[i + 1]) : kNone;
}

// Successor of every tour node. For a root the "next sibling" link holds the
// next outlet, and a root's exit with no next outlet ends the list.
__global__ void succ_kernel(Grid g, const std::uint8_t* __restrict__ mask, const std::int64_t* __restrict__ receiver,
                            const std::uint32_t* __restrict__ first_child, const std::uint32_t* __restrict__ next_sib,
                            std::uint32_t* __restrict__ succ)
{
    LSDTT_COUNT();
    const std::int64_t flat = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (flat >= g.n) return;
    if (!mask[flat])
    {
        succ[2 * flat] = kEnd;
        succ[2 * flat + 1] = kEnd;
        return;
    }
    const std::uint32_t fc = first_child[flat];
    const std::uint32_t ns = next_sib[flat];
    const std::int64_t p = receiver[flat];
    succ[2 * flat] = (fc != kNone) ? 2u * fc : static_cast<std::uint32_t>(2 * flat + 1);
    if (ns != kNone) succ[2 * flat + 1] = 2u * ns;
    else if (p >= 0) succ[2 * flat + 1] = static_cast<std::uint32_t>(2 * p + 1);
    else succ[2 * flat + 1] = kEnd;
}

struct RankLevel
{
    std::uint32_t n;                 // node capacity of this level
    const std::uint32_t* succ;       // [n]
    const std::int32_t* w0;          // [n] or null: parity weights
    const std::int32_t* w1;          // [n] or null
    const std::uint8_t* cell_mask;   // level 0: node v valid iff cell_mask[v>>1]
    const std::uint32_t* head;       // device scalar
    const std::uint32_t* count;      // device scalar: valid nodes at this level (null: n)
};

__device__ __forceinline__ void weights(const RankLevel& L, std::uint32_t v, int& a, int& b)
{
    if (L.w0) { a = L.w0[v]; b = L.w1[v]; }
    else { a = (v & 1u) ? 0 : 1; b = (v & 1u) ? -1 : 1; }
}

__device__ __forceinline__ bool node_valid(const RankLevel& L, std::uint32_t v)
{
    if (L.cell_mask) return L.cell_mask[v >> 1] != 0;
    return v < *L.count;
}

// Per tour node of a ranking level: the ruler whose walk reached it and the
// two prefixes from that ruler, one 16-byte record (a walk step writes one
// sector, not three).
struct alignas(16) RankRec
{
    std::uint32_t owner;
    std::int32_t loc0, loc1, pad;
};

// Ruler compaction in one pass: each thread takes 16 consecutive nodes, a
// block scans its rulers and claims a range of the ruler list with one
// atomic (ruler numbers then depend on block order; the ranks do not). Also
// counts the level's valid nodes (cnt[2]) for the coverage check.
constexpr int kCompactPer = 16;

__global__ void __launch_bounds__(256) ruler_compact(RankLevel L, std::uint32_t cap, std::uint32_t* __restrict__ rulers,
                                                     RankRec* __restrict__ rec, std::uint32_t* __restrict__ cnt)
{
    LSDTT_COUNT();
    __shared__ unsigned wsum[8], wval[8], s_base;
    const std::uint32_t head = *L.head;
    const std::uint32_t v0 = (blockIdx.x * blockDim.x + threadIdx.x) * kCompactPer;
    unsigned rmask = 0, nvalid = 0;
#pragma unroll
    for (int j = 0; j < kCompactPer; ++j)
    {
        const std::uint32_t v = v0 + j;
        if (v < L.n && node_valid(L, v))
        {
            ++nvalid;
            if (is_ruler(v) || v == head) rmask |= 1u << j;
        }
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned nr = __popc(rmask);
    unsigned incl = nr;
    for (int o = 1; o < 32; o <<= 1)
    {
        const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    unsigned val = nvalid;
    for (int o = 16; o > 0; o >>= 1) val += __shfl_down_sync(0xffffffffu, val, o);
    if (lane == 31) wsum[w] = incl;
    if (lane == 0) wval[w] = val;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        unsigned tot = 0, tv = 0;
        for (int k = 0; k < static_cast<int>(blockDim.x >> 5); ++k)
        {
            const unsigned t = wsum[k];
            wsum[k] = tot;
            tot += t;
            tv += wval[k];
        }
        s_base = tot ? atomicAdd(&cnt[0], tot) : 0u;
        if (tv) atomicAdd(&cnt[2], tv);
    }
    __syncthreads();
    std::uint32_t pos = s_base + wsum[w] + incl - nr;
#pragma unroll
    for (int j = 0; j < kCompactPer; ++j)
        if ((rmask >> j) & 1u)
        {
            if (pos < cap)
            {
                rulers[pos] = v0 + j;
                rec[v0 + j].owner = pos;
            }
            ++pos;  // a count above cap is reported by ruler_checks
        }
}

// After the walks: too many rulers, or walks that did not cover every valid
// node of the level (a successor structure that is not one list).
__global__ void ruler_checks(const std::uint32_t* cnt, std::uint32_t cap, unsigned long long* err)
{
    LSDTT_COUNT();
    if (cnt[0] > cap) raise_error(err, 9, cnt[0]);
    else if (cnt[3] != cnt[2]) raise_error(err, kErrCycle, 2);
}

// A walk from ruler i to the next ruler. A node of the list is a ruler iff
// is_ruler(v) or it is the head (ruler_compact), so the stop test needs no
// load.
__global__ void ruler_walk(RankLevel L, const std::uint32_t* __restrict__ rulers,
                           const std::uint32_t* __restrict__ n_rulers, RankRec* __restrict__ rec,
                           std::int32_t* __restrict__ sub0, std::int32_t* __restrict__ sub1,
                           std::uint32_t* __restrict__ nxt, std::uint32_t* __restrict__ next_head,
                           std::uint32_t* __restrict__ walked, std::uint32_t cap,
                           unsigned long long* __restrict__ err)
{
    LSDTT_COUNT();
    const std::uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const std::uint32_t nr = *n_rulers;
    if (i >= nr || i >= cap) return;
    const std::uint32_t head = *L.head;
    std::uint32_t v = rulers[i];
    if (v == head) *next_head = i;
    int a0 = 0, a1 = 0;
    std::uint32_t steps = 0;
    do
    {
        rec[v] = RankRec{i, a0, a1, 0};
        int w0, w1;
        weights(L, v, w0, w1);
        a0 += w0;
        a1 += w1;
        v = L.succ[v];
        ++steps;
    } while (v != kEnd && !is_ruler(v) && v != head && steps <= L.n);
    if (steps > L.n) raise_error(err, kErrCycle, 0);
    sub0[i] = a0;
    sub1[i] = a1;
    nxt[i] = (v == kEnd) ? kEnd : rec[v].owner;
    // coverage: the walks visit every valid node exactly once (one atomic per
    // converged group of lanes)
    const unsigned grp = __activemask();
    const unsigned tot = __reduce_add_sync(grp, steps);
    if ((threadIdx.x & 31) == static_cast<unsigned>(__ffs(grp) - 1)) atomicAdd(walked, tot);
}

__global__ void serial_rank(RankLevel L, std::int32_t* __restrict__ p0, std::int32_t* __restrict__ p1,
                            unsigned long long* __restrict__ err)
{
    LSDTT_COUNT();
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    std::uint32_t v = *L.head;
    int a0 = 0, a1 = 0;
    std::uint32_t steps = 0;
    while (v != kEnd && steps <= L.n)
    {
        p0[v] = a0;
        p1[v] = a1;
        int w0, w1;
        weights(L, v, w0, w1);
        a0 += w0;
        a1 += w1;
        v = L.succ[v];
        ++steps;
    }
    if (steps > L.n) raise_error(err, kErrCycle, 1);
}

__global__ void rank_finish(RankLevel L, const RankRec* __restrict__ rec, const std::int32_t* __restrict__ P0,
                            const std::int32_t* __restrict__ P1, std::uint32_t cap, std::int32_t* __restrict__ p0,
                            std::int32_t* __restrict__ p1, unsigned long long* __restrict__ err)
{
    LSDTT_COUNT();
    const std::uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= L.n || !node_valid(L, v)) return;
    const RankRec r = rec[v];
    const std::uint32_t o = r.owner;
    if (o >= cap)
    {
        // Not reached by any walk: the tour does not cover every valid node.
        raise_error(err, kErrCycle, 2);
        p0[v] = -1;
        p1[v] = 0;
        return;
    }
    p0[v] = P0[o] + r.loc0;
    p1[v] = P1[o] + r.loc1;
}

// Per-cell s-vector outputs, written straight from the level-0 ranking
// (sv_finish) or from its prefix arrays (sv_outputs). start and svec may be
// null (a caller that needs the counts and depths only).
struct SvOut
{
    Grid g;
    const std::uint8_t* mask;
    std::int64_t n_valid;
    std::int64_t* start;
    std::uint64_t* size;
    std::int32_t* depth;
    std::int64_t* svec;
};

__device__ __forceinline__ void sv_store(const SvOut& o, std::int64_t c, std::int32_t s, std::int32_t e,
                                         std::int32_t dep, unsigned long long* __restrict__ err)
{
    if (s < 0 || e <= s || static_cast<std::int64_t>(e) > o.n_valid)
    {
        raise_error(err, kErrCycle, 3);
        if (o.start) o.start[c] = kNodataReceiver;
        o.size[c] = 0;
        o.depth[c] = 0;
        return;
    }
    if (o.start) o.start[c] = s;
    o.size[c] = static_cast<std::uint64_t>(e - s);
    o.depth[c] = dep;
    if (o.svec) o.svec[s] = c;
}

__device__ __forceinline__ bool sv_masked(const SvOut& o, std::int64_t c)
{
    if (o.mask[c]) return false;
    if (o.start) o.start[c] = kNodataReceiver;
    o.size[c] = 0;
    o.depth[c] = -1;
    return true;
}

// rank_finish and sv_outputs in one pass over the cells of the level-0
// (Euler tour) list: cell c's enter and exit records are adjacent.
__global__ void sv_finish(RankLevel L, const RankRec* __restrict__ rec, const std::int32_t* __restrict__ P0,
                          const std::int32_t* __restrict__ P1, std::uint32_t cap, SvOut o,
                          unsigned long long* __restrict__ err)
{
    LSDTT_COUNT();
    const std::int64_t c = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= o.g.n || sv_masked(o, c)) return;
    const RankRec a = rec[2 * c], b = rec[2 * c + 1];
    if (a.owner >= cap || b.owner >= cap)
    {
        // Not reached by any walk: the tour does not cover every valid node.
        raise_error(err, kErrCycle, 2);
        sv_store(o, c, -1, -1, 0, err);
        return;
    }
    sv_store(o, c, P0[a.owner] + a.loc0, P0[b.owner] + b.loc0, P1[a.owner] + a.loc1, err);
}

// Recursive list ranking. p0/p1 receive the exclusive prefix sums of the two
// weights along the list starting at *L.head; with sv (the level-0 Euler
// tour of a grid, longer than kSerialLimit) the per-cell s-vector outputs are
// written instead and p0/p1 are not used.
cudaError_t rank_list(const RankLevel& L, std::int32_t* p0, std::int32_t* p1, Scratch& ws,
                      unsigned long long* err, cudaStream_t st, const SvOut* sv = nullptr)
{
    if (L.n <= static_cast<std::uint32_t>(kSerialLimit))
    {
        serial_rank<<<1, 32, 0, st>>>(L, p0, p1, err);
        return cudaGetLastError();
    }
    const std::size_t mark = ws.used;
    const std::uint32_t cap = L.n / (kRuler / 4) + 64;  // generous bound on the ruler count
    // cnt: [0] rulers, [1] the head's ruler, [2] valid nodes, [3] nodes walked
    std::uint32_t* cnt = ws.take<std::uint32_t>(4);
    RankRec* rec = ws.take<RankRec>(L.n);
    // The ruler count is data dependent; size everything by `cap` and let the
    // kernels read the true count. A count above `cap` is reported.
    std::uint32_t* rulers = ws.take<std::uint32_t>(cap);
    std::uint32_t* nxt = ws.take<std::uint32_t>(cap);
    std::int32_t* sub0 = ws.take<std::int32_t>(cap);
    std::int32_t* sub1 = ws.take<std::int32_t>(cap);
    std::int32_t* P0 = ws.take<std::int32_t>(cap);
    std::int32_t* P1 = ws.take<std::int32_t>(cap);
    std::uint32_t* nhead = cnt + 1;
    if (!cnt || !rec || !rulers || !nxt || !sub0 || !sub1 || !P0 || !P1) return cudaErrorMemoryAllocation;
    const unsigned nb = grid_blocks(L.n, 256);
    cudaMemsetAsync(cnt, 0, sizeof(std::uint32_t) * 4, st);
    ruler_compact<<<grid_blocks((L.n + kCompactPer - 1) / kCompactPer, 256), 256, 0, st>>>(L, cap, rulers, rec, cnt);
    // Bytes touched per tour node: successor 4 in, the 16-byte record out.
    LSDTT_TIMED("stack_ruler_walk", 20.0 * static_cast<double>(L.n), st,
                (ruler_walk<<<grid_blocks(cap, 128), 128, 0, st>>>(L, rulers, cnt, rec, sub0, sub1, nxt, nhead,
                                                                   cnt + 3, cap, err)));
    ruler_checks<<<1, 1, 0, st>>>(cnt, cap, err);
    cudaError_t e = cudaSuccess;
    RankLevel up{cap, nxt, sub0, sub1, nullptr, nhead, cnt};
    e = rank_list(up, P0, P1, ws, err, st);
    if (e != cudaSuccess) return e;
    if (sv)
        sv_finish<<<grid_blocks(sv->g.n, 256), 256, 0, st>>>(L, rec, P0, P1, cap, *sv, err);
    else
        rank_finish<<<nb, 256, 0, st>>>(L, rec, P0, P1, cap, p0, p1, err);
    ws.used = mark;
    return cudaGetLastError();
}



// Per-cell s-vector outputs from the two prefix sums (lists short enough for
// the serial ranking).
__global__ void sv_outputs(SvOut o, const std::int32_t* __restrict__ p0, const std::int32_t* __restrict__ p1,
                           unsigned long long* __restrict__ err)
{
    LSDTT_COUNT();
    const std::int64_t c = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= o.g.n || sv_masked(o, c)) return;
    sv_store(o, c, p0[2 * c], p0[2 * c + 1], p1[2 * c], err);
}

// ---- range max over the s-vector: blocks of 32, sparse table over blocks ----
__global__ void rmq_base(const std::int64_t* __restrict__ svec, const std::int32_t* __restrict__ depth,
                         std::int64_t n, std::uint64_t* __restrict__ A, std::uint64_t* __restrict__ pre,
                         std::uint64_t* __restrict__ suf, std::uint64_t* __restrict__ blk)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    std::uint64_t a = 0;
    if (i < n)
    {
        const std::int64_t c = svec[i];
        a = (static_cast<std::uint64_t>(static_cast<std::uint32_t>(depth[c])) << 32) | static_cast<std::uint32_t>(c);
        A[i] = a;
    }
    std::uint64_t p = a;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const std::uint64_t y = __shfl_up_sync(0xffffffffu, p, o);
        if (lane >= o && y > p) p = y;
    }
    std::uint64_t s = a;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const std::uint64_t y = __shfl_down_sync(0xffffffffu, s, o);
        if (lane + o < 32 && y > s) s = y;
    }
    if (i < n)
    {
        pre[i] = p;
        suf[i] = s;
    }
    if (lane == 31 && (i - 31) < n) blk[i >> 5] = p;
}

__global__ void rmq_level(const std::uint64_t* __restrict__ prev, std::int64_t nb, std::int64_t half,
                          std::uint64_t* __restrict__ next)
{
    LSDTT_COUNT();
    const std::int64_t b = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    std::uint64_t v = prev[b];
    if (b + half < nb && prev[b + half] > v) v = prev[b + half];
    next[b] = v;
}

struct Rmq
{
    const std::uint64_t* A;
    const std::uint64_t* pre;
    const std::uint64_t* suf;
    const std::uint64_t* const* table;  // device array of level pointers
    int levels;
};

__device__ std::uint64_t rmq_query(const Rmq& R, std::int64_t a, std::int64_t b)  // inclusive
{
    const std::int64_t ba = a >> 5, bb = b >> 5;
    if (ba == bb)
    {
        std::uint64_t m = 0;
        for (std::int64_t i = a; i <= b; ++i)
            if (R.A[i] > m) m = R.A[i];
        return m;
    }
    std::uint64_t m = R.suf[a];
    if (R.pre[b] > m) m = R.pre[b];
    const std::int64_t lo = ba + 1, hi = bb - 1;
    if (lo <= hi)
    {
        const std::int64_t len = hi - lo + 1;
        const int k = 63 - __clzll(static_cast<unsigned long long>(len));
        const std::uint64_t* T = R.table[k];
        std::uint64_t x = T[lo];
        const std::uint64_t y = T[hi - (std::int64_t(1) << k) + 1];
        if (y > x) x = y;
        if (x > m) m = x;
    }
    return m;
}

__global__ void topo_heights(Grid g, const std::uint8_t* __restrict__ mask, const std::int64_t* __restrict__ start,
                             const std::uint64_t* __restrict__ size, const std::int32_t* __restrict__ depth, Rmq R,
                             std::int32_t* __restrict__ height, std::uint32_t* __restrict__ leaf,
                             unsigned long long* __restrict__ maxh)
{
    LSDTT_COUNT();
    const std::int64_t c = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= g.n) return;
    if (!mask[c])
    {
        height[c] = -1;
        return;
    }
    const std::int64_t a = start[c];
    const std::int64_t b = a + static_cast<std::int64_t>(size[c]) - 1;
    std::int32_t h = 0;
    if (a < 0 || b < a)
    {
        height[c] = 0;  // already reported by sv_outputs
        leaf[c] = static_cast<std::uint32_t>(c);
    }
    else
    {
        const std::uint64_t m = rmq_query(R, a, b);
        h = static_cast<std::int32_t>(m >> 32) - depth[c];
        height[c] = h;
        leaf[c] = static_cast<std::uint32_t>(m & 0xffffffffull);
    }
    // Warp-aggregated max keeps the atomic traffic low.
    unsigned long long v = static_cast<unsigned long long>(h);
    for (int o = 16; o > 0; o >>= 1)
    {
        const unsigned long long y = __shfl_down_sync(__activemask(), v, o);
        if (y > v) v = y;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(maxh, v);
}

// Sort keys (height, headwater); invalid cells get height maxh+1 so they
// sort after every valid cell and are dropped.
__global__ void topo_keys(Grid g, const std::uint8_t* __restrict__ mask, const std::int32_t* __restrict__ height,
                          const std::uint32_t* __restrict__ leaf, int leaf_bits, std::uint64_t maxh,
                          std::uint64_t* __restrict__ keys, std::uint32_t* __restrict__ vals)
{
    LSDTT_COUNT();
    const std::int64_t c = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= g.n) return;
    const std::uint64_t h = mask[c] ? static_cast<std::uint64_t>(height[c]) : maxh + 1;
    const std::uint64_t l = mask[c] ? leaf[c] : 0u;
    keys[c] = (h << leaf_bits) | l;
    vals[c] = static_cast<std::uint32_t>(c);
}

__global__ void topo_store(const std::uint32_t* __restrict__ vals, std::int64_t n_valid, std::int64_t* __restrict__ topo,
                           std::uint32_t* __restrict__ topo_pos)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n_valid) return;
    const std::uint32_t c = vals[i];
    topo[i] = c;
    topo_pos[c] = static_cast<std::uint32_t>(i);
}

int bits_for(std::uint64_t v)
{
    int b = 0;
    while (v) { ++b; v >>= 1; }
    return b;
}

}  // namespace

cudaError_t build_stack(lsdtt_gpu_flow* f, bool want_topo, cudaStream_t st, const Packed* packed)
{
    const Grid& g = f->g;
    const std::int64_t n = g.n;
    Scratch& ws = f->ws;
    const std::size_t mark = ws.used;
    const unsigned nb = grid_blocks(n, 256);

    std::uint32_t* first_child = ws.take<std::uint32_t>(n);
    std::uint32_t* next_sib = ws.take<std::uint32_t>(n);
    std::uint32_t* succ = ws.take<std::uint32_t>(2 * n);
    std::uint32_t* head = ws.take<std::uint32_t>(1);
    // A tour longer than kSerialLimit writes the s-vector outputs straight
    // from the ruler records; only the serial ranking needs prefix arrays.
    const bool fused = 2 * n > kSerialLimit;
    std::int32_t* p0 = fused ? nullptr : ws.take<std::int32_t>(2 * n);
    std::int32_t* p1 = fused ? nullptr : ws.take<std::int32_t>(2 * n);
    if (!first_child || !next_sib || !succ || !head || (!fused && (!p0 || !p1))) return cudaErrorMemoryAllocation;

    if (packed)
    {
        if (want_topo) return cudaErrorInvalidValue;  // the ensemble needs the s-vector only
        links_packed<<<nb, 256, 0, st>>>(*packed, f->mask, f->dir, first_child, next_sib);
    }
    else
        links_kernel<<<nb, 256, 0, st>>>(g, f->mask, f->dir, first_child, next_sib);
    root_links_kernel<<<grid_blocks(n, 256), 256, 0, st>>>(f->outlets, f->dscal + 1, next_sib, head);
    succ_kernel<<<nb, 256, 0, st>>>(g, f->mask, f->receiver, first_child, next_sib, succ);

    RankLevel L0{static_cast<std::uint32_t>(2 * n), succ, nullptr, nullptr, f->mask, head, nullptr};
    // The ensemble reads the counts and depths only.
    const SvOut sv{g,          f->mask, f->n_valid, packed ? nullptr : f->sv_start, f->sv_size, f->depth,
                   packed ? nullptr : f->svec};
    cudaError_t e = rank_list(L0, p0, p1, ws, f->derr, st, fused ? &sv : nullptr);
    if (e != cudaSuccess) return e;
    if (!fused) sv_outputs<<<nb, 256, 0, st>>>(sv, p0, p1, f->derr);
    ws.used = mark;  // tour buffers are no longer needed
    if (!want_topo) return cudaGetLastError();

    // Range-max structure over the s-vector.
    const std::int64_t nv = f->n_valid;
    if (nv == 0) return cudaGetLastError();
    const std::int64_t nblk = (nv + 31) / 32;
    std::uint64_t* A = ws.take<std::uint64_t>(nv);
    std::uint64_t* pre = ws.take<std::uint64_t>(nv);
    std::uint64_t* suf = ws.take<std::uint64_t>(nv);
    int levels = 1;
    while ((std::int64_t(1) << levels) <= nblk) ++levels;
    std::uint64_t* tab[40] = {};
    for (int k = 0; k < levels; ++k) tab[k] = ws.take<std::uint64_t>(nblk);
    std::uint64_t** dtab = ws.take<std::uint64_t*>(40);
    if (!A || !pre || !suf || !dtab || !tab[levels - 1]) return cudaErrorMemoryAllocation;
    rmq_base<<<grid_blocks(nblk * 32, 256), 256, 0, st>>>(f->svec, f->depth, nv, A, pre, suf, tab[0]);
    for (int k = 1; k < levels; ++k)
        rmq_level<<<grid_blocks(nblk, 256), 256, 0, st>>>(tab[k - 1], nblk, std::int64_t(1) << (k - 1), tab[k]);
    cudaMemcpyAsync(dtab, tab, sizeof(tab), cudaMemcpyHostToDevice, st);

    std::uint64_t* k0 = ws.take<std::uint64_t>(n);
    std::uint32_t* v0 = ws.take<std::uint32_t>(n);
    std::uint64_t* k1 = ws.take<std::uint64_t>(n);
    std::uint32_t* v1 = ws.take<std::uint32_t>(n);
    std::uint32_t* leaf = ws.take<std::uint32_t>(n);
    if (!k0 || !v0 || !k1 || !v1 || !leaf) return cudaErrorMemoryAllocation;
    const int leaf_bits = bits_for(static_cast<std::uint64_t>(n - 1) | 1);
    Rmq R{A, pre, suf, dtab, levels};
    cudaMemsetAsync(f->derr + 2, 0, sizeof(unsigned long long), st);
    topo_heights<<<nb, 256, 0, st>>>(g, f->mask, f->sv_start, f->sv_size, f->depth, R, f->height, leaf, f->derr + 2);
    // The number of radix passes depends on the tallest level: read it back.
    cudaMemcpyAsync(&f->herr[2], f->derr + 2, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    const std::uint64_t maxh = f->herr[2];
    f->max_height = static_cast<std::int64_t>(maxh);
    topo_keys<<<nb, 256, 0, st>>>(g, f->mask, f->height, leaf, leaf_bits, maxh, k0, v0);
    const int bits = leaf_bits + bits_for(maxh + 1);
    const int cur = radix_sort_pairs(k0, v0, k1, v1, n, bits, ws, st, &e);
    if (e != cudaSuccess) return e;
    topo_store<<<grid_blocks(nv, 256), 256, 0, st>>>(cur ? v1 : v0, nv, f->topo, f->topo_pos);
    ws.used = mark;
    return cudaGetLastError();
}


// ---------------------------------------------------------------------------
// accumulate (src/cpu/lsdtt_flowinfo_cpu.cpp:1979-2046)
//
// The reference seeds every valid cell with its weight and pushes
// acc[rec] += acc[flat] in topological order, so a receiver's total is its
// weight plus its donors' totals added in the donors' topological order.
// When every partial sum is exactly representable (default weights dx^2 with
// dx^2 = m*2^e and n_valid*m < 2^53) the order cannot matter and the total is
// size*dx^2 exactly: one pass. Otherwise the totals are formed level by level
// (height 0 first) with each cell adding its donors in topological order --
// the reference's additions in the reference's order.
// ---------------------------------------------------------------------------
namespace
{

__global__ void accum_exact(Grid g, const std::uint8_t* __restrict__ mask, const std::uint64_t* __restrict__ size,
                            double w, double* __restrict__ out)
{
    LSDTT_COUNT();
    const std::int64_t c = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= g.n) return;
    out[c] = mask[c] ? static_cast<double>(size[c]) * w : 0.0;
}

__global__ void accum_seed(Grid g, const std::uint8_t* __restrict__ mask, const double* __restrict__ w, double dw,
                           double* __restrict__ out)
{
    LSDTT_COUNT();
    const std::int64_t c = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= g.n) return;
    out[c] = mask[c] ? (w ? w[c] : dw) : 0.0;
}

__global__ void accum_level(Grid g, const std::uint8_t* __restrict__ mask, const std::uint8_t* __restrict__ dir,
                            const std::int64_t* __restrict__ topo, const std::uint32_t* __restrict__ topo_pos,
                            std::int64_t lo, std::int64_t hi, double* __restrict__ acc)
{
    LSDTT_COUNT();
    const std::int64_t i = lo + static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= hi) return;
    const std::int64_t c = topo[i];
    std::int64_t d[8];
    const int k = donor_list(g, mask, dir, c, d);
    // Order donors by topological position.
    std::uint32_t p[8];
    for (int a = 0; a < k; ++a) p[a] = topo_pos[d[a]];
    for (int a = 1; a < k; ++a)
    {
        const std::uint32_t pk = p[a];
        const std::int64_t dk = d[a];
        int j = a;
        while (j > 0 && p[j - 1] > pk) { p[j] = p[j - 1]; d[j] = d[j - 1]; --j; }
        p[j] = pk;
        d[j] = dk;
    }
    double s = acc[c];
    for (int a = 0; a < k; ++a) s = __dadd_rn(s, acc[d[a]]);
    acc[c] = s;
}

__global__ void level_bounds(const std::int64_t* __restrict__ topo, const std::int32_t* __restrict__ height,
                             std::int64_t nv, std::int64_t* __restrict__ start)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const std::int32_t h = height[topo[i]];
    if (i == 0 || height[topo[i - 1]] != h) start[h] = i;
    if (i == nv - 1) start[h + 1] = nv;
}

bool exact_by_count(double dw, std::int64_t nv)
{
    // dw = m * 2^e with m odd; exact iff nv * m < 2^53.
    if (!(dw > 0.0) || !std::isfinite(dw)) return false;
    int e = 0;
    double fr = std::frexp(dw, &e);  // dw = fr * 2^e, fr in [0.5, 1)
    std::uint64_t m = static_cast<std::uint64_t>(std::ldexp(fr, 53));
    while (m && !(m & 1)) m >>= 1;
    const long double prod = static_cast<long double>(m) * static_cast<long double>(nv);
    return prod < 9007199254740992.0L;
}

}  // namespace

cudaError_t accumulate(lsdtt_gpu_flow* f, const double* w, double* out, cudaStream_t st, bool* exact_path)
{
    const Grid& g = f->g;
    const unsigned nb = grid_blocks(g.n, 256);
    const double dw = g.cell * g.cell;
    if (!w && exact_by_count(dw, f->n_valid))
    {
        *exact_path = true;
        accum_exact<<<nb, 256, 0, st>>>(g, f->mask, f->sv_size, dw, out);
        return cudaGetLastError();
    }
    *exact_path = false;
    accum_seed<<<nb, 256, 0, st>>>(g, f->mask, w, dw, out);
    const std::int64_t nv = f->n_valid;
    if (nv == 0) return cudaGetLastError();
    const std::int64_t nlev = f->max_height + 1;
    Scratch& ws = f->ws;
    const std::size_t mark = ws.used;
    std::int64_t* start = ws.take<std::int64_t>(static_cast<std::size_t>(nlev) + 1);
    if (!start) return cudaErrorMemoryAllocation;
    level_bounds<<<grid_blocks(nv, 256), 256, 0, st>>>(f->topo, f->height, nv, start);
    std::int64_t* hstart = static_cast<std::int64_t*>(std::malloc(sizeof(std::int64_t) * (nlev + 1)));
    if (!hstart) return cudaErrorMemoryAllocation;
    cudaMemcpyAsync(hstart, start, sizeof(std::int64_t) * (nlev + 1), cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess)
        for (std::int64_t k = 1; k < nlev; ++k)  // level 0 cells have no donors
        {
            const std::int64_t lo = hstart[k], hi = hstart[k + 1];
            if (hi > lo) accum_level<<<grid_blocks(hi - lo, 128), 128, 0, st>>>(g, f->mask, f->dir, f->topo,
                                                                               f->topo_pos, lo, hi, out);
        }
    std::free(hstart);
    ws.used = mark;
    return e != cudaSuccess ? e : cudaGetLastError();
}

}  // namespace lsdtt_gb300

namespace lsdtt_gb300
{
LSDTT_DEFINE_LAUNCH_READER(stack)
}  // namespace lsdtt_gb300
