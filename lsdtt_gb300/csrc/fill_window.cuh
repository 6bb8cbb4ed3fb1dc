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
// heap in global memory and marks seen cells with a per-cell stamp.
struct WinStore
{
    float* fv;            // FIFO values (ring)
    std::uint32_t* fc;    // FIFO cells
    std::uint32_t fcap;   // power of two
    float* hz;            // heap keys
    std::uint32_t* hc;    // heap cells
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

// Binary heap on (key, cell), one thread.
__device__ __forceinline__ void win_heap_push(const WinStore& s, std::uint32_t& size, float key, std::uint32_t cell)
{
    std::uint32_t i = size++;
    while (i > 0)
    {
        const std::uint32_t p = (i - 1) >> 1;
        const float pk = s.hz[p];
        const std::uint32_t pc = s.hc[p];
        if (!win_key_less(key, cell, pk, pc)) break;
        s.hz[i] = pk;
        s.hc[i] = pc;
        i = p;
    }
    s.hz[i] = key;
    s.hc[i] = cell;
}

__device__ __forceinline__ void win_heap_pop(const WinStore& s, std::uint32_t& size)
{
    const std::uint32_t n = --size;
    if (n == 0) return;
    const float key = s.hz[n];
    const std::uint32_t cell = s.hc[n];
    std::uint32_t i = 0;
    for (;;)
    {
        std::uint32_t c = 2 * i + 1;
        if (c >= n) break;
        float ck = s.hz[c];
        std::uint32_t cc = s.hc[c];
        if (c + 1 < n && win_key_less(s.hz[c + 1], s.hc[c + 1], ck, cc))
        {
            ++c;
            ck = s.hz[c];
            cc = s.hc[c];
        }
        if (!win_key_less(ck, cc, key, cell)) break;
        s.hz[i] = ck;
        s.hc[i] = cc;
        i = c;
    }
    s.hz[i] = key;
    s.hc[i] = cell;
}

__device__ __forceinline__ std::uint32_t win_hash(std::uint32_t x, std::uint32_t mask)
{
    return (x * 2654435761u) & mask;
}

// Insert `cell` into the shared-memory seen set; false if it was there
// already (or the set is full: *full is set).
__device__ __forceinline__ bool win_seen_insert(const WinStore& s, std::uint32_t cell, std::uint32_t* count,
                                                bool* full)
{
    const std::uint32_t mask = s.hscap - 1;
    std::uint32_t h = win_hash(cell, mask);
    for (std::uint32_t probe = 0; probe < s.hscap; ++probe)
    {
        const std::uint32_t prev = atomicCAS(&s.hs[h], kWinNone, cell);
        if (prev == kWinNone)
        {
            if (atomicAdd(count, 1u) + 1 > (s.hscap >> 1) + (s.hscap >> 2)) *full = true;
            return true;
        }
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
__device__ WinResult win_replay(const WinGrid& G, int w, const WinStore& s, std::uint64_t pop_limit)
{
    const int lane = threadIdx.x & 31;
    const float S = G.cuts[w];
    __shared__ std::uint32_t sh_seen_count[32];  // one per warp of the block
    __shared__ bool sh_full[32];
    const int wib = threadIdx.x >> 5;
    if (lane == 0)
    {
        sh_seen_count[wib] = 0;
        sh_full[wib] = false;
    }
    if (s.hs)
        for (std::uint32_t k = lane; k < s.hscap; k += 32) s.hs[k] = kWinNone;
    __syncwarp();
    std::int64_t p = win_lower_bound(G.ordRec, G.nsorted, S);
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
        // the list head: next sorted cell queued at the window start (kept
        // in registers until the list is popped)
        if (rescan)
        {
            have_l = false;
            while (p < G.nsorted)
            {
                const std::int64_t q = p + lane;
                float4 o = make_float4(0.0f, INFINITY, 0.0f, 0.0f);
                if (q < G.nsorted) o = G.ordRec[q];
                const unsigned b = __ballot_sync(0xffffffffu, o.y < S);
                if (b)
                {
                    const int k = __ffs(b) - 1;
                    p += k;
                    lz = __shfl_sync(0xffffffffu, o.x, k);
                    lc = __float_as_uint(__shfl_sync(0xffffffffu, o.z, k));
                    have_l = true;
                    break;
                }
                p += 32;
            }
            if (p > G.nsorted) p = G.nsorted;
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
            const float tz = s.hz[0];
            const std::uint32_t tc = s.hc[0];
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
            const float fz = s.fv[head & fmask];
            if (!have_h || fz <= hmz)
            {
                src = 2;
                cur_v = fz;
                cur_c = s.fc[head & fmask];
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
            const bool trig = hmz <= V && cnext > 0 && G.cuts[cnext - 1] >= hmz;
            if (!trig && (cnext >= G.ncut || G.cand[cnext]))
            {
                res.next = cnext;
                break;
            }
            src = from_list ? 0 : 1;
            cur_v = hmz;
            cur_c = hmc;
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
            while (cnext < G.ncut && G.cuts[cnext] <= V) ++cnext;
        }
        if (pop_limit && ++pops > pop_limit)
        {
            res.status = kWinOverflow;
            break;
        }
        // neighbours, one lane per direction (N, NE, ..., NW)
        const int r = static_cast<int>(cur_c / static_cast<std::uint32_t>(G.nc));
        const int c = static_cast<int>(cur_c - static_cast<std::uint32_t>(r) * G.nc);
        std::uint32_t j = kWinNone;
        bool fresh = false;
        float zj = 0.0f;
        std::uint32_t sv = 0;  // the cell's stamp (large tier), loaded beside its record
        if (lane < 8)
        {
            int rr, cc;
            if (fill_nb(G.nr, G.nc, G.per_ns, G.per_ew, r, c, lane, rr, cc))
            {
                const std::uint32_t jj = static_cast<std::uint32_t>(rr) * G.nc + cc;
                const float4 q = G.rec[jj];
                if (s.stamp) sv = s.stamp[jj];
                zj = q.x;
                // open: valid, not popped before the window (F0 >= S), not
                // queued at its start (mnb >= S)
                if (q.w != 0.0f && q.y >= S && !(q.z < S)) j = jj;
            }
        }
        // a neighbour reached twice through a periodic wrap counts once
        for (int k = 0; k < 7; ++k)
        {
            const std::uint32_t other = __shfl_sync(0xffffffffu, j, k);
            if (lane > k && j != kWinNone && other == j) j = kWinNone;
        }
        if (j != kWinNone)
        {
            if (s.stamp)
            {
                fresh = sv != s.stamp_id;
                if (fresh) s.stamp[j] = s.stamp_id;
            }
            else
                fresh = win_seen_insert(s, j, &sh_seen_count[wib], &sh_full[wib]);
        }
        __syncwarp();
        if (sh_full[wib])
        {
            res.status = kWinOverflow;
            break;
        }
        const bool raised = fresh && zj <= cur_v;
        const unsigned rb = __ballot_sync(0xffffffffu, raised);
        const unsigned hb = __ballot_sync(0xffffffffu, fresh && !raised);
        if (tail - head + __popc(rb) > s.fcap || hsize + __popc(hb) > s.hcap)
        {
            res.status = kWinOverflow;
            break;
        }
        if (raised)
        {
            const float nz = raise_from(cur_v, G.eps, (lane & 1) ? G.Ld : G.L);
            const std::uint32_t slot = (tail + __popc(rb & ((1u << lane) - 1u))) & fmask;
            s.fv[slot] = nz;
            s.fc[slot] = j;
        }
        tail += __popc(rb);
        // heap pushes by lane 0
        unsigned m = hb;
        while (m)
        {
            const int k = __ffs(m) - 1;
            m &= m - 1;
            const float kz = __shfl_sync(0xffffffffu, zj, k);
            const std::uint32_t kc = __shfl_sync(0xffffffffu, j, k);
            if (lane == 0) win_heap_push(s, hsize, kz, kc);
            else ++hsize;
        }
        __syncwarp();
    }
    res.nout = nout;
    return res;
}

}  // namespace
}  // namespace lsdtt_gb300
