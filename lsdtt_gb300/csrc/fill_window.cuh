// fill_window.cuh -- the epsilon fill in the reference's exact order, by
// independent value windows: the replay of one window by one warp.
//
// The reference (priority_flood_core, lsdtt_raster_flow_preprocessing_cpu.cpp
// :416-511) pops cells from a heap keyed by value and from one FIFO of raised
// cells; the FIFO front is taken whenever its value is at most the heap top.
// A cell takes its value from its first-popped neighbour, so the result
// depends on that global order. An "episode" is a stretch of the run with a
// non-empty FIFO; between episodes the heap pops in plain value order and no
// cell is raised.
//
// Windows. An episode can only start when a heap pop meets an unqueued
// neighbour at or below its own value; that happens only at an epsilon-0 pour
// level: a value P = F0(c) of a cell c with z(c) <= F0(c) next to a cell b
// with z(b) = F0(b) = P, F0 being the epsilon-0 fill (exact, order-free).
// Cut the value axis at those levels. If the FIFO is empty when the heap top
// first reaches a cut S, the state of the run at that moment is known without
// replaying anything before it: a cell has been popped exactly when F0 < S,
// and the heap holds exactly the cells with F0 >= S that have a neighbour
// with F0 < S (or are seeds), each at its own elevation (F0 = z for them).
// So the run from S onwards can be replayed from S alone: the window's
// "list" is the F0-sorted array from S on, filtered to those cells, merged
// with a small heap of the cells the window discovers itself and the
// window's own FIFO. The replay stops at the first moment its FIFO is empty
// and no cut lies between the heap top and the largest value it popped; the
// next cut above that value is then a valid window start of its own.
//
// Every candidate window is replayed at once (one warp each); the windows
// that start at a valid cut form a chain from the lowest cut (valid by
// construction), each one naming the next, and only the chain's raised
// values are kept. A replay that reaches a cut that is not a candidate
// carries on through it, so which cuts are candidates decides how much work
// is wasted, never the result.
//
// Ties between heap entries of equal value are taken in (value, cell index)
// order. The reference's std::priority_queue orders them by its internal
// layout, which no parallel method can reproduce; its output then is not a
// function of the algorithm, and the two differ only where such a tie
// decides a discovery.
#pragma once

#include <cmath>
#include <cstdint>

#include "common.cuh"
#include "fill_tile.cuh"

namespace lsdtt_gb300
{
namespace
{

constexpr std::uint32_t kWinNone = 0xffffffffu;
constexpr int kWinOk = 0, kWinOverflow = 1;

// Order-preserving map of a float to an unsigned key (NaN not expected).
__host__ __device__ __forceinline__ std::uint32_t float_order_key(float v)
{
    std::uint32_t b;
    memcpy(&b, &v, 4);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

__host__ __device__ __forceinline__ float float_from_order_key(std::uint32_t k)
{
    const std::uint32_t b = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    float v;
    memcpy(&v, &b, 4);
    return v;
}

// One grid (or one ensemble member) as the window replay sees it; every
// pointer and cell index is member-local. Per cell one 16-byte record
// {z, F0 (epsilon-0 fill), mnb (min F0 over valid neighbours; -inf for
// seeds, +inf for cells never queued), class (0 invalid or NaN, 1 valid)};
// per sorted position {F0, mnb, cell, -} over the valid cells by
// (F0, index): one load gives a replay all it needs of a cell.
struct WinGrid
{
    int nr, nc;
    bool per_ns, per_ew;
    float L, Ld, eps;
    const float4* rec;
    const float4* ordRec;
    std::int64_t nsorted;
    const float* cuts;          // sorted distinct pour levels
    const std::uint8_t* cand;   // candidate window start per cut
    int ncut;
};

// first sorted position with F0 >= v (n if none)
__device__ __forceinline__ std::int64_t win_lower_bound(const float4* a, std::int64_t n, float v)
{
    std::int64_t lo = 0, hi = n;
    while (lo < hi)
    {
        const std::int64_t mid = (lo + hi) >> 1;
        if (a[mid].x < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// first k with a[k] > v
__device__ __forceinline__ std::int64_t win_upper_bound(const float* a, std::int64_t n, float v)
{
    std::int64_t lo = 0, hi = n;
    while (lo < hi)
    {
        const std::int64_t mid = (lo + hi) >> 1;
        if (a[mid] <= v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ bool win_key_less(float za, std::uint32_t ia, float zb, std::uint32_t ib)
{
    return za < zb || (za == zb && ia < ib);
}

// Storage of one replay. Small tiers keep everything in shared memory (the
// seen set as an open-addressing hash); the large tier keeps the FIFO and
// heap in global memory and marks seen cells with a per-cell stamp. FIFO
// entries are {value bits, cell} and heap entries {order key of the value,
// cell} in one 64-bit word each, so that one load moves an entry and one
// compare orders two heap entries by (value, cell).
struct WinStore
{
    std::uint64_t* fq;    // FIFO (ring)
    std::uint32_t fcap;   // power of two
    std::uint64_t* hk;    // heap, 1-based (hk[1] the minimum); hcap + 2 entries, 16-byte aligned
    std::uint32_t hcap;
    std::uint32_t* hs;    // seen hash (small tiers) or null
    std::uint32_t hscap;  // power of two
    std::uint32_t* stamp; // per-cell stamps (large tier) or null
    std::uint32_t stamp_id;
    std::uint32_t* oc;    // raised outputs (small tiers) or null: written to out_F directly
    float* ov;
    std::uint32_t ocap;
    float* out_F;         // large tier: the fill itself (member-local)
};

// Heap entry of a cell at value z. Both zeros share one key (they compare
// equal, so the cell index decides); the value read back is then +0, which
// no replay can tell from -0: it only compares it and raises from it with a
// positive minimum slope.
__device__ __forceinline__ std::uint64_t win_hkey(float z, std::uint32_t cell)
{
    return (static_cast<std::uint64_t>(float_order_key(z == 0.0f ? 0.0f : z)) << 32) | cell;
}

__device__ __forceinline__ float win_hkey_value(std::uint64_t k)
{
    return float_from_order_key(static_cast<std::uint32_t>(k >> 32));
}

__device__ __forceinline__ std::uint64_t win_fentry(float v, std::uint32_t cell)
{
    return (static_cast<std::uint64_t>(__float_as_uint(v)) << 32) | cell;
}

// Binary heap on the 64-bit keys (distinct: one entry per cell), one
// thread, 1-based so that the two children of a node share one 16-byte load.
__device__ __forceinline__ void win_heap_push(const WinStore& s, std::uint32_t& size, std::uint64_t key)
{
    std::uint32_t i = ++size;
    while (i > 1)
    {
        const std::uint32_t p = i >> 1;
        const std::uint64_t pk = s.hk[p];
        if (key >= pk) break;
        s.hk[i] = pk;
        i = p;
    }
    s.hk[i] = key;
}

__device__ __forceinline__ void win_heap_pop(const WinStore& s, std::uint32_t& size)
{
    const std::uint32_t n = --size;  // entries left
    if (n == 0) return;
    const std::uint64_t key = s.hk[n + 1];
    std::uint32_t i = 1;
    for (;;)
    {
        std::uint32_t c = 2 * i;
        if (c > n) break;
        const ulonglong2 pr = *reinterpret_cast<const ulonglong2*>(s.hk + c);
        std::uint64_t ck = pr.x;
        if (c < n && pr.y < ck)
        {
            ck = pr.y;
            ++c;
        }
        if (key <= ck) break;
        s.hk[i] = ck;
        i = c;
    }
    s.hk[i] = key;
}

// Row of a cell index (exact: a float estimate corrected by whole rows).
__device__ __forceinline__ int win_row(std::uint32_t cell, int nc, float inv_nc)
{
    int r = __float2int_rz(__uint2float_rz(cell) * inv_nc);
    int c = static_cast<int>(cell - static_cast<std::uint32_t>(r) * static_cast<std::uint32_t>(nc));
    while (c < 0)
    {
        --r;
        c += nc;
    }
    while (c >= nc)
    {
        ++r;
        c -= nc;
    }
    return r;
}

__device__ __forceinline__ std::uint32_t win_hash(std::uint32_t x, std::uint32_t mask)
{
    return (x * 2654435761u) & mask;
}

// Insert `cell` into the shared-memory seen set; false if it was there
// already (or every slot was probed: *full is set). The caller counts the
// insertions warp-wide and keeps the set at most three quarters full.
__device__ __forceinline__ bool win_seen_insert(const WinStore& s, std::uint32_t cell, bool* full)
{
    const std::uint32_t mask = s.hscap - 1;
    std::uint32_t h = win_hash(cell, mask);
    for (std::uint32_t probe = 0; probe < s.hscap; ++probe)
    {
        const std::uint32_t prev = atomicCAS(&s.hs[h], kWinNone, cell);
        if (prev == kWinNone) return true;
        if (prev == cell) return false;
        h = (h + 1) & mask;
    }
    *full = true;
    return false;
}

struct WinResult
{
    int status;          // kWinOk / kWinOverflow
    int next;            // next window start (cut index; ncut = none)
    std::uint32_t nout;  // raised outputs (small tiers)
};

// Replay the window starting at cut w, by one full warp (all 32 lanes call
// it with the same arguments). `pop_limit` bounds the pops (0: none). Every
// loop iteration takes one entry from the list, the heap or the FIFO or
// leaves; each cell enters the heap or the FIFO at most once (the seen set),
// so the replay ends after at most nsorted + (cells seen) iterations.
//
// A pop is a chain of dependent steps, so the loop keeps what it can off
// that chain: the neighbour loads are issued before the heap is repaired,
// and the cuts around the running maximum and a block of the sorted list sit
// in registers (one entry per lane).
__device__ WinResult win_replay(const WinGrid& G, int w, const WinStore& s, std::uint64_t pop_limit)
{
    const int lane = threadIdx.x & 31;
    const unsigned full = 0xffffffffu;
    const float S = G.cuts[w];
    std::uint32_t seen = 0;  // cells in the seen set (warp-uniform)
    const std::uint32_t seen_cap = (s.hscap >> 1) + (s.hscap >> 2);
    if (s.hs)
        for (std::uint32_t k = lane; k < s.hscap; k += 32) s.hs[k] = kWinNone;
    __syncwarp();
    // two directions reach the same cell only through the periodic wrap of
    // a grid one or two cells across
    const bool dedupe = (G.per_ns && G.nr <= 2) || (G.per_ew && G.nc <= 2);
    // cuts cb .. cb+31, one per lane (+inf past the last), with their
    // candidate flags; cb <= cnext - 1 and cnext - cb <= 31 (or cnext = ncut)
    int cb = w;
    float cut_l = INFINITY;
    bool cand_l = true;
    if (cb + lane < G.ncut)
    {
        cut_l = G.cuts[cb + lane];
        cand_l = G.cand[cb + lane] != 0;
    }
    // the sorted list from lb on, one position per lane; the list head is
    // the first position >= p queued at the window start (mnb < S)
    const float4 lsent = make_float4(0.0f, INFINITY, 0.0f, 0.0f);
    std::int64_t p = win_lower_bound(G.ordRec, G.nsorted, S);
    std::int64_t lb = p;
    float4 lo = lb + lane < G.nsorted ? G.ordRec[lb + lane] : lsent;
    const float inv_nc = 1.0f / static_cast<float>(G.nc);
    bool rescan = true;  // the list head below is stale
    bool have_l = false;
    float lz = INFINITY;
    std::uint32_t lc = kWinNone;
    std::uint32_t head = 0, tail = 0, hsize = 0, nout = 0;
    float V = S;
    int cnext = w + 1;  // first cut > V
    std::uint64_t pops = 0;
    WinResult res{kWinOk, G.ncut, 0};
    const std::uint32_t fmask = s.fcap - 1;
    for (;;)
    {
        if (rescan)
        {
            have_l = false;
            for (;;)
            {
                const unsigned b = __ballot_sync(full, lb + lane >= p && lo.y < S);
                if (b)
                {
                    const int k = __ffs(b) - 1;
                    p = lb + k;
                    lz = __shfl_sync(full, lo.x, k);
                    lc = __float_as_uint(__shfl_sync(full, lo.z, k));
                    have_l = true;
                    break;
                }
                if (lb + 32 >= G.nsorted)
                {
                    p = G.nsorted;
                    break;
                }
                lb += 32;
                lo = lb + lane < G.nsorted ? G.ordRec[lb + lane] : lsent;
            }
            if (!have_l)
            {
                lz = INFINITY;
                lc = kWinNone;
            }
            rescan = false;
        }
        // heap minimum (list head or discovered heap top)
        float hmz = lz;
        std::uint32_t hmc = lc;
        bool from_list = have_l;
        if (hsize > 0)
        {
            const std::uint64_t t = s.hk[1];
            const float tz = win_hkey_value(t);
            const std::uint32_t tc = static_cast<std::uint32_t>(t);
            if (!have_l || win_key_less(tz, tc, lz, lc))
            {
                hmz = tz;
                hmc = tc;
                from_list = false;
            }
        }
        const bool have_h = have_l || hsize > 0;
        const bool fifo_ne = tail != head;
        int src;  // 0 list, 1 heap, 2 FIFO
        float cur_v;
        std::uint32_t cur_c;
        if (fifo_ne)
        {
            const std::uint64_t f = s.fq[head & fmask];
            const float fz = __uint_as_float(static_cast<std::uint32_t>(f >> 32));
            if (!have_h || fz <= hmz)
            {
                src = 2;
                cur_v = fz;
                cur_c = static_cast<std::uint32_t>(f);
            }
            else
            {
                src = from_list ? 0 : 1;
                cur_v = hmz;
                cur_c = hmc;
            }
        }
        else
        {
            if (!have_h)
            {
                res.next = G.ncut;
                break;
            }
            // FIFO empty: a pop can start an episode only at a cut in [hmz, V]
            const float cprev = __shfl_sync(full, cut_l, cnext - 1 - cb);
            const bool candn = __shfl_sync(full, cand_l, cnext - cb);
            const bool trig = hmz <= V && cprev >= hmz;
            if (!trig && (cnext >= G.ncut || candn))
            {
                res.next = cnext;
                break;
            }
            src = from_list ? 0 : 1;
            cur_v = hmz;
            cur_c = hmc;
        }
        // neighbours, one lane per direction (N, NE, ..., NW): the loads go
        // out first
        const int r = win_row(cur_c, G.nc, inv_nc);
        const int c = static_cast<int>(cur_c - static_cast<std::uint32_t>(r) * G.nc);
        std::uint32_t j = kWinNone;
        float4 q = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        std::uint32_t sv = 0;  // the cell's stamp (large tier), loaded beside its record
        if (lane < 8)
        {
            int rr, cc;
            if (fill_nb(G.nr, G.nc, G.per_ns, G.per_ew, r, c, lane, rr, cc))
            {
                j = static_cast<std::uint32_t>(rr) * G.nc + cc;
                q = G.rec[j];
                if (s.stamp) sv = s.stamp[j];
            }
        }
        // take it
        if (src == 2)
        {
            ++head;
            if (s.oc)
            {
                if (nout >= s.ocap)
                {
                    res.status = kWinOverflow;
                    break;
                }
                if (lane == 0)
                {
                    s.oc[nout] = cur_c;
                    s.ov[nout] = cur_v;
                }
                ++nout;
            }
            else if (lane == 0)
                s.out_F[cur_c] = cur_v;
        }
        else if (src == 0)
        {
            ++p;
            rescan = true;
        }
        else
        {
            if (lane == 0) win_heap_pop(s, hsize);
            else --hsize;
        }
        __syncwarp();
        if (cur_v > V)
        {
            V = cur_v;
            // first cut > V (the cuts are sorted; lanes past the last hold +inf)
            for (;;)
            {
                const unsigned b = __ballot_sync(full, cut_l > V);
                if (b)
                {
                    cnext = min(cb + __ffs(b) - 1, G.ncut);
                    break;
                }
                if (cb + 32 >= G.ncut)
                {
                    cnext = G.ncut;
                    break;
                }
                cb += 31;
                cut_l = INFINITY;
                cand_l = true;
                if (cb + lane < G.ncut)
                {
                    cut_l = G.cuts[cb + lane];
                    cand_l = G.cand[cb + lane] != 0;
                }
            }
        }
        if (pop_limit && ++pops > pop_limit)
        {
            res.status = kWinOverflow;
            break;
        }
        // open: valid, not popped before the window (F0 >= S), not queued
        // at its start (mnb >= S)
        if (j != kWinNone && !(q.w != 0.0f && q.y >= S && !(q.z < S))) j = kWinNone;
        const float zj = q.x;
        // a neighbour reached twice through a periodic wrap counts once
        if (dedupe)
            for (int k = 0; k < 7; ++k)
            {
                const std::uint32_t other = __shfl_sync(full, j, k);
                if (lane > k && j != kWinNone && other == j) j = kWinNone;
            }
        bool fresh = false, probe_full = false;
        if (j != kWinNone)
        {
            if (s.stamp)
            {
                fresh = sv != s.stamp_id;
                if (fresh) s.stamp[j] = s.stamp_id;
            }
            else
                fresh = win_seen_insert(s, j, &probe_full);
        }
        const bool raised = fresh && zj <= cur_v;
        const unsigned rb = __ballot_sync(full, raised);
        const unsigned hb = __ballot_sync(full, fresh && !raised);
        if (s.hs)
        {
            seen += __popc(rb | hb);
            if (__any_sync(full, probe_full) || seen > seen_cap)
            {
                res.status = kWinOverflow;
                break;
            }
        }
        if (tail - head + __popc(rb) > s.fcap || hsize + __popc(hb) > s.hcap)
        {
            res.status = kWinOverflow;
            break;
        }
        if (raised)
        {
            const float nz = raise_from(cur_v, G.eps, (lane & 1) ? G.Ld : G.L);
            const std::uint32_t slot = (tail + __popc(rb & ((1u << lane) - 1u))) & fmask;
            s.fq[slot] = win_fentry(nz, j);
        }
        tail += __popc(rb);
        // heap pushes, each by the lane that found the cell, in lane order
        // (every lane keeps the heap size)
        const std::uint64_t my_key = win_hkey(zj, j);
        unsigned m = hb;
        while (m)
        {
            const int k = __ffs(m) - 1;
            m &= m - 1;
            if (lane == k) win_heap_push(s, hsize, my_key);
            else ++hsize;
            __syncwarp();
        }
        __syncwarp();
    }
    res.nout = nout;
    return res;
}

}  // namespace
}  // namespace lsdtt_gb300
