// fill_sweep.cuh -- one value window of the epsilon fill (fill_window.cuh)
// replayed by a whole thread block, one FIFO sweep at a time.
//
// A sweep is the reference's processing of the FIFO entries f_1..f_m present
// when the previous sweep ended, with the heap pops interleaved between them.
// Within a sweep every pop has a time T: the FIFO entry f_g pops at
// (g, 1); a heap cell of value k and index i pops at (g, 0, k, i), where g
// is its gap -- the first FIFO index at or after the moment it was queued
// whose value exceeds k (before f_g the heap pops everything below v_g, in
// value order). A cell queued before the sweep has gap NG(1, k); one that a
// pop discovers inherits the gap of its discoverer (the next gap after a
// FIFO entry), advanced to the next FIFO value above k. A cell not yet
// queued is discovered by the neighbour that pops first, i.e. with the
// smallest T, in that neighbour's direction order; it is raised (next
// sweep's FIFO, ordered by (T of the discoverer, direction)) when it is not
// above the discoverer's value, and otherwise queued as a heap cell (a pop
// of this sweep if its gap exists). Those rules define every T of the sweep
// as a fixed point, found in rounds: each round re-evaluates the cells next
// to the pops that changed in the previous one (a changed pop can only move
// the cells next to it). Between sweeps, when the FIFO runs empty, the block
// takes single heap pops by the sequential rules of win_replay.
//
// The replay is latency-bound (one sweep after another), so each round costs
// a few dependent loads: one 16-byte event record per cell, the round's
// lists in shared memory, every neighbour's record loaded at once.
#pragma once

#include <cstdint>

#include "fill_window.cuh"

namespace lsdtt_gb300
{
namespace
{

constexpr int kSwThreads = 512;
// (the chain block has a whole SM to itself: its registers fill it, so the
// shared memory is sized to hold the widest FIFO generations of large basins)
constexpr int kSwFQ = 4096;  // FIFO entries of one sweep (a power of two)
constexpr int kSwL = 4096;   // entries of each per-sweep list (changed pops, discovered cells)
constexpr int kSwLv = 4;     // levels of the heap cells at or above the near threshold

// A cell's pop in the current sweep: valid when st is the sweep's id.
struct __align__(16) SwEv
{
    std::uint64_t hi;  // (gap << 33) | (kind << 32) | value key; kind 1 = FIFO entry
    std::uint32_t st;
    float val;
};

// A cell's discoverer in the current sweep (valid when te_st is the sweep's id).
struct __align__(16) SwTe
{
    std::uint64_t hi;   // discoverer's T
    std::uint32_t lo;   // its tie word (its cell for heap pops, 0 for FIFO entries)
    float val;          // its value
};

// Per-member scratch of the block replay (member-local, one entry per cell
// unless stated). Stamps make every array valid without clearing: a value
// counts only when it carries the current window's or sweep's id.
struct SweepBufs
{
    std::uint32_t* cst;      // (window id << 2) | 1 heap, 2 FIFO, 3 popped
    SwEv* ev;
    SwTe* te;
    std::uint32_t* te_st;    // sweep id: the discoverer in te is valid
    std::uint8_t* te_k;      // direction from the discoverer
    std::uint32_t* mk_c;     // round id: re-evaluated in this round (one thread per cell);
                             // a value at or below the sweep's id: not yet in this sweep
    std::uint32_t *dc, *dc2; // heap cells discovered earlier, not popped, with a value
    float *dk, *dk2;         //   below the threshold T ("near", two buffers)
    std::uint32_t* lc;       // the same at or above T, in kSwLv levels of lstride entries:
    float* lk;               //   level 0 below Lb[1], level k in [Lb[k], Lb[k+1]), the last
    std::size_t lstride;     //   unbounded; the bands grow 16-fold, a level is gathered and
                             //   spread again only when T reaches its lower bound (a radix heap)
    std::uint32_t* sc;       // spare list the gathering goes through
    float* sk;
};

struct SweepShared
{
    std::uint32_t fc[kSwFQ];
    float fv[kSwFQ];
    std::uint16_t ng[kSwFQ + 2];
    std::uint32_t nc[kSwFQ];
    float nv[kSwFQ];
    std::uint64_t nhi[kSwFQ];
    std::uint32_t nlo[kSwFQ];
    std::uint8_t nk[kSwFQ];
    std::uint32_t la[kSwL], lb[kSwL], lt[kSwL];
    std::uint32_t cnt[12];
    float red_v[kSwThreads / 32];
    std::uint32_t red_i[kSwThreads / 32];
    std::uint32_t red_s[kSwThreads / 32];
    std::int64_t red_p;
};

__device__ __forceinline__ std::uint64_t sw_hi(std::uint32_t g, std::uint32_t kind, float key)
{
    return (static_cast<std::uint64_t>(g) << 33) | (static_cast<std::uint64_t>(kind) << 32) | float_order_key(key);
}

// FIFOs up to this length are searched entry by entry; longer ones through
// the next-greater table ng
constexpr std::uint32_t kSwScan = 64;

// first FIFO index >= g0 (1-based) whose value exceeds key; m + 1 if none
__device__ __forceinline__ std::uint32_t sw_ng(const SweepShared& sh, std::uint32_t m, std::uint32_t g0, float key)
{
    std::uint32_t g = g0;
    if (m <= kSwScan)
        while (g <= m && !(sh.fv[g - 1] > key)) ++g;
    else
        while (g <= m && !(sh.fv[g - 1] > key)) g = sh.ng[g];
    return g;
}

// Block replay of window w (every thread of a kSwThreads block calls it).
// *ctr is the member's id counter (stamps), advanced here. Returns kWinOk
// with *next set, or kWinOverflow (a sweep's FIFO or lists above their
// shared-memory size, or no fixed point within its round limit) -- then
// nothing of the window is final and the caller replays it by the
// sequential rules.
__device__ int win_sweep_replay(const WinGrid& G, int w, const SweepBufs& B, float* out_F, std::uint32_t* ctr,
                                SweepShared& sh, int* next)
{
    const int tid = threadIdx.x;
    const float S = G.cuts[w];
    __shared__ std::uint32_t s_ctr, s_m, s_nd, s_win, s_sweep, s_status, s_last_move;
    __shared__ std::uint32_t s_nl[kSwLv];
    __shared__ std::int64_t s_p;
    __shared__ float s_V, s_Vmax, s_T, s_D;
    __shared__ float s_Lb[kSwLv];
    __shared__ int s_j;
    __shared__ int s_cnext, s_next, s_stop;
    if (tid == 0)
    {
        s_ctr = *ctr;
        s_win = ++s_ctr;
        s_p = win_lower_bound(G.ordRec, G.nsorted, S);
        s_V = S;
        s_cnext = w + 1;
        s_m = 0;
        s_nd = 0;
        // near threshold T: four diagonal raise steps above the start
        // (adapted as the window goes); level bounds 16, 256, 4096 bands on
        s_D = fmaxf(4.0f * G.eps * G.Ld, 1e-6f * fabsf(S) + 1e-30f);
        s_T = S + s_D;
        float wb = 16.0f * s_D;
        s_Lb[0] = s_T;
        for (int k = 0; k < kSwLv; ++k) s_nl[k] = 0;
        for (int k = 1; k < kSwLv; ++k)
        {
            s_Lb[k] = s_T + wb;
            wb *= 16.0f;
        }
        s_last_move = 0;
        s_status = kWinOk;
        s_next = G.ncut;
        s_stop = 0;
    }
    __syncthreads();
    const std::uint32_t win = s_win;
    // not queued yet: valid, not popped before the window, not queued at its
    // start, not queued by this window
    auto open_cell = [&](std::uint32_t j, float& zj) -> bool {
        const float4 q = G.rec[j];
        const std::uint32_t c = B.cst[j];
        zj = q.x;
        return q.w != 0.0f && q.y >= S && !(q.z < S) && (c >> 2) != win;
    };
    std::uint32_t* dc = B.dc;
    std::uint32_t* dc2 = B.dc2;
    float* dk = B.dk;
    float* dk2 = B.dk2;
    // level of a heap cell's key at or above T
    auto level_of = [&](float key) -> int {
        int k = 0;
        while (k + 1 < kSwLv && !(key < s_Lb[k + 1])) ++k;
        return k;
    };
    auto lvc = [&](int k) { return B.lc + static_cast<std::size_t>(k) * B.lstride; };
    auto lvk = [&](int k) { return B.lk + static_cast<std::size_t>(k) * B.lstride; };
    // every pass pops at least one cell (a background pop or a sweep's
    // FIFO), so more passes than cells means the replay has gone wrong: it
    // is then left to the sequential rules
    const std::uint64_t pass_cap = static_cast<std::uint64_t>(G.nr) * static_cast<std::uint64_t>(G.nc) + 2;
    std::uint64_t passes = 0;
    for (;;)
    {
        if (++passes > pass_cap)
        {
            if (tid == 0) s_status = kWinOverflow;
            __syncthreads();
            break;
        }
        if (s_m == 0)
        {
            // ---- FIFO empty: one heap pop by the sequential rules ----
            if (tid == 0)
            {
                std::int64_t p = s_p;
                while (p < G.nsorted && !(G.ordRec[p].y < S)) ++p;
                s_p = p;
            }
            // the least discovered heap cell: in the first non-empty list
            // (every near key is below T, and every level's keys below the
            // next level's)
            int which = -1;
            if (!s_nd)
            {
                which = kSwLv - 1;
                for (int k = kSwLv - 2; k >= 0; --k)
                    if (s_nl[k]) which = k;
            }
            const std::uint32_t* lc = which < 0 ? dc : lvc(which);
            const float* lk = which < 0 ? dk : lvk(which);
            const std::uint32_t ln = which < 0 ? s_nd : s_nl[which];
            float bz = INFINITY;
            std::uint32_t bi = kWinNone, bslot = kWinNone;
            for (std::uint32_t t = tid; t < ln; t += kSwThreads)
                if (win_key_less(lk[t], lc[t], bz, bi))
                {
                    bz = lk[t];
                    bi = lc[t];
                    bslot = t;
                }
            for (int o = 16; o > 0; o >>= 1)
            {
                const float oz = __shfl_down_sync(0xffffffffu, bz, o);
                const std::uint32_t oi = __shfl_down_sync(0xffffffffu, bi, o);
                const std::uint32_t os = __shfl_down_sync(0xffffffffu, bslot, o);
                if (win_key_less(oz, oi, bz, bi))
                {
                    bz = oz;
                    bi = oi;
                    bslot = os;
                }
            }
            if ((tid & 31) == 0)
            {
                sh.red_v[tid >> 5] = bz;
                sh.red_i[tid >> 5] = bi;
                sh.red_s[tid >> 5] = bslot;
            }
            __syncthreads();
            if (tid == 0)
            {
                for (int k = 1; k < kSwThreads / 32; ++k)
                    if (win_key_less(sh.red_v[k], sh.red_i[k], bz, bi))
                    {
                        bz = sh.red_v[k];
                        bi = sh.red_i[k];
                        bslot = sh.red_s[k];
                    }
                const bool have_l = s_p < G.nsorted;
                float hz = INFINITY;
                std::uint32_t hc = kWinNone;
                bool from_list = false;
                if (have_l)
                {
                    const float4 o = G.ordRec[s_p];
                    hz = o.x;
                    hc = __float_as_uint(o.z);
                    from_list = true;
                }
                if (bi != kWinNone && (!have_l || win_key_less(bz, bi, hz, hc)))
                {
                    hz = bz;
                    hc = bi;
                    from_list = false;
                }
                if (hc == kWinNone)
                {
                    s_next = G.ncut;
                    s_stop = 1;
                }
                else
                {
                    const float V = s_V;
                    // first cut above V (sweeps leave it to this point)
                    {
                        int lo = s_cnext, hi = G.ncut;
                        while (lo < hi)
                        {
                            const int mid = (lo + hi) >> 1;
                            if (G.cuts[mid] <= V) lo = mid + 1;
                            else hi = mid;
                        }
                        s_cnext = lo;
                    }
                    const int cn = s_cnext;
                    const bool trig = hz <= V && cn > 0 && G.cuts[cn - 1] >= hz;
                    if (!trig && (cn >= G.ncut || G.cand[cn]))
                    {
                        s_next = cn;
                        s_stop = 1;
                    }
                    else
                    {
                        if (from_list) ++s_p;
                        else
                        {
                            if (which < 0)
                            {
                                const std::uint32_t last = --s_nd;
                                dc[bslot] = dc[last];
                                dk[bslot] = dk[last];
                            }
                            else
                            {
                                const std::uint32_t last = --s_nl[which];
                                std::uint32_t* wc = lvc(which);
                                float* wk = lvk(which);
                                wc[bslot] = wc[last];
                                wk[bslot] = wk[last];
                            }
                            B.cst[hc] = (win << 2) | 3u;
                        }
                        if (hz > s_V)
                        {
                            s_V = hz;
                            while (s_cnext < G.ncut && G.cuts[s_cnext] <= s_V) ++s_cnext;
                        }
                        const int r = static_cast<int>(hc / static_cast<std::uint32_t>(G.nc));
                        const int c = static_cast<int>(hc - static_cast<std::uint32_t>(r) * G.nc);
                        std::uint32_t m = 0;
                        for (int d = 0; d < 8; ++d)
                        {
                            int rr, cc;
                            if (!fill_nb(G.nr, G.nc, G.per_ns, G.per_ew, r, c, d, rr, cc)) continue;
                            const std::uint32_t j = static_cast<std::uint32_t>(rr) * G.nc + cc;
                            float zj;
                            if (!open_cell(j, zj)) continue;
                            if (zj <= hz)
                            {
                                sh.fc[m] = j;
                                sh.fv[m] = raise_from(hz, G.eps, (d & 1) ? G.Ld : G.L);
                                ++m;
                                B.cst[j] = (win << 2) | 2u;
                            }
                            else
                            {
                                if (zj < s_T)
                                {
                                    dc[s_nd] = j;
                                    dk[s_nd] = zj;
                                    ++s_nd;
                                }
                                else
                                {
                                    const int k = level_of(zj);
                                    lvc(k)[s_nl[k]] = j;
                                    lvk(k)[s_nl[k]] = zj;
                                    ++s_nl[k];
                                }
                                B.cst[j] = (win << 2) | 1u;
                            }
                        }
                        s_m = m;
                    }
                }
            }
            __syncthreads();
            if (s_stop) break;
            continue;
        }
        // ---- one sweep ----
        const std::uint32_t m = s_m;
        if (tid == 0)
        {
            // the sweep's id, then ids for its rounds (sweep + 1 .. sweep + 64)
            s_sweep = ++s_ctr;
            s_ctr += 64;
            // cnt: [0] changed (la), [1] changed next (lb), [2] discovered
            // (lt), [3] surviving heap cells, [4] next FIFO, [5] overflow,
            // [6..10] moves and appends to the near list and the levels
            for (int k = 0; k < 12; ++k) sh.cnt[k] = 0;
        }
        {
            // the FIFO's largest value, and the next greater FIFO value after
            // each index (1-based, m + 1: none): every thread looks up to 32
            // entries ahead; one thread finishes the rest right to left with
            // pointer jumps (entries g + 1 .. g + 32 are known not greater)
            float lv = -INFINITY;
            for (std::uint32_t g = tid; g < m; g += kSwThreads) lv = fmaxf(lv, sh.fv[g]);
            if (m > kSwScan)
                for (std::uint32_t g = 1 + tid; g <= m; g += kSwThreads)
                {
                    const float v = sh.fv[g - 1];
                    const std::uint32_t lim = min(m + 1, g + 33);
                    std::uint32_t n = g + 1;
                    while (n < lim && !(sh.fv[n - 1] > v)) ++n;
                    sh.ng[g] = static_cast<std::uint16_t>((n < lim || lim == m + 1) ? n : 0u);
                }
            for (int o = 16; o > 0; o >>= 1) lv = fmaxf(lv, __shfl_down_sync(0xffffffffu, lv, o));
            if ((tid & 31) == 0) sh.red_v[tid >> 5] = lv;
            __syncthreads();
            if (tid == 0)
            {
                float vmax = -INFINITY;
                for (int k = 0; k < kSwThreads / 32; ++k) vmax = fmaxf(vmax, sh.red_v[k]);
                s_Vmax = vmax;
                if (m > kSwScan)
                {
                    sh.ng[m + 1] = static_cast<std::uint16_t>(m + 1);
                    for (std::uint32_t g = m; g >= 1; --g)
                        if (sh.ng[g] == 0)
                        {
                            std::uint32_t n = g + 33;
                            while (n <= m && !(sh.fv[n - 1] > sh.fv[g - 1])) n = sh.ng[n];
                            sh.ng[g] = static_cast<std::uint16_t>(n);
                        }
                }
            }
        }
        __syncthreads();
        const std::uint32_t sweep = s_sweep;
        const float Vmax = s_Vmax;
        if (Vmax >= s_T)
        {
            // the FIFO reaches T: raise it; the levels whose lower bound it
            // has reached (0 .. j) are gathered and spread again, below T to
            // the near list, the rest under new bounds (kept below level
            // j + 1's); each cell goes down a level at a time
            if (tid == 0)
            {
                // T moved again within 4 sweeps: widen the band; not within
                // 64: narrow it (a sweep's id advances by 65)
                if (sweep - s_last_move < 4u * 65u) s_D *= 2.0f;
                else if (sweep - s_last_move > 64u * 65u) s_D *= 0.5f;
                s_last_move = sweep;
                s_T = Vmax + s_D;
                s_Lb[0] = s_T;
                int jl = 0;
                for (int k = 1; k < kSwLv; ++k)
                    if (!(s_T < s_Lb[k])) jl = k;
                if (jl > 0)
                {
                    const float cap = jl + 1 < kSwLv ? s_Lb[jl + 1] : INFINITY;
                    float wb = 16.0f * s_D;
                    for (int k = 1; k <= jl; ++k)
                    {
                        s_Lb[k] = fminf(s_T + wb, cap);
                        wb *= 16.0f;
                    }
                }
                s_j = jl;
                for (int k = 6; k < 12; ++k) sh.cnt[k] = 0;
            }
            __syncthreads();
            const int jl = s_j;
            std::uint32_t ng_all = 0;
            for (int k = 0; k <= jl; ++k)
            {
                const std::uint32_t nk = s_nl[k];
                const std::uint32_t* src_c = lvc(k);
                const float* src_k = lvk(k);
                for (std::uint32_t t = tid; t < nk; t += kSwThreads)
                {
                    B.sc[ng_all + t] = src_c[t];
                    B.sk[ng_all + t] = src_k[t];
                }
                ng_all += nk;
            }
            __syncthreads();
            const float T = s_T;
            const std::uint32_t nd0 = s_nd;
            const int lane = tid & 31;
            auto warp_append = [&](bool want, std::uint32_t* dst_c, float* dst_k, std::uint32_t* ctr, std::uint32_t c,
                                   float key) {
                const unsigned b = __ballot_sync(0xffffffffu, want);
                if (!b) return;
                const int lead = __ffs(b) - 1;
                std::uint32_t base = 0;
                if (lane == lead) base = atomicAdd(ctr, static_cast<std::uint32_t>(__popc(b)));
                base = __shfl_sync(0xffffffffu, base, lead);
                if (want)
                {
                    const std::uint32_t k2 = base + __popc(b & ((1u << lane) - 1u));
                    dst_c[k2] = c;
                    dst_k[k2] = key;
                }
            };
            for (std::uint32_t t0 = 0; t0 < ng_all; t0 += kSwThreads)
            {
                const std::uint32_t t = t0 + tid;
                const bool in = t < ng_all;
                const std::uint32_t c = in ? B.sc[t] : 0u;
                const float key = in ? B.sk[t] : INFINITY;
                const int dest = !in ? -2 : (key < T ? -1 : level_of(key));
                warp_append(dest == -1, dc + nd0, dk + nd0, &sh.cnt[6], c, key);
                for (int k = 0; k <= jl; ++k) warp_append(dest == k, lvc(k), lvk(k), &sh.cnt[7 + k], c, key);
            }
            __syncthreads();
            if (tid == 0)
            {
                s_nd = nd0 + sh.cnt[6];
                for (int k = 0; k <= jl; ++k) s_nl[k] = sh.cnt[7 + k];
                for (int k = 0; k < 12; ++k) sh.cnt[k] = 0;
            }
            __syncthreads();
        }
        auto push_list = [&](std::uint32_t* list, int which, std::uint32_t c) {
            const std::uint32_t k = atomicAdd(&sh.cnt[which], 1u);
            if (k < static_cast<std::uint32_t>(kSwL)) list[k] = c;
            else sh.cnt[5] = 1;
        };
        // the same for a whole warp at once (lanes with `want`): one atomic
        auto push_warp = [&](std::uint32_t* list, int which, bool want, std::uint32_t c) {
            const unsigned b = __ballot_sync(0xffffffffu, want);
            if (!b) return;
            const int lane = tid & 31;
            const int lead = __ffs(b) - 1;
            std::uint32_t base = 0;
            if (lane == lead) base = atomicAdd(&sh.cnt[which], static_cast<std::uint32_t>(__popc(b)));
            base = __shfl_sync(0xffffffffu, base, lead);
            if (want)
            {
                const std::uint32_t k = base + __popc(b & ((1u << lane) - 1u));
                if (k < static_cast<std::uint32_t>(kSwL)) list[k] = c;
                else sh.cnt[5] = 1;
            }
        };
        // FIFO entries: pops (g, 1)
        for (std::uint32_t g0 = 0; g0 < m; g0 += kSwThreads)
        {
            const std::uint32_t g = g0 + tid;
            std::uint32_t c = 0;
            if (g < m)
            {
                c = sh.fc[g];
                B.ev[c] = SwEv{sw_hi(g + 1, 1, 0.0f), sweep, sh.fv[g]};
            }
            push_warp(sh.la, 0, g < m, c);
        }
        // heap cells discovered earlier: those below Vmax pop in this sweep
        {
            const std::uint32_t nd = s_nd;
            constexpr int kU = 4;
            for (std::uint32_t t0 = 0; t0 < nd; t0 += kSwThreads * kU)
            {
                std::uint32_t cs[kU];
                float ks[kU];
#pragma unroll
                for (int u = 0; u < kU; ++u)
                {
                    const std::uint32_t t = t0 + u * kSwThreads + tid;
                    cs[u] = t < nd ? dc[t] : 0u;
                    ks[u] = t < nd ? dk[t] : INFINITY;
                }
#pragma unroll
                for (int u = 0; u < kU; ++u)
                {
                    const bool in = t0 + u * kSwThreads + tid < nd;
                    const bool pops = in && ks[u] < Vmax;
                    if (pops)
                    {
                        B.ev[cs[u]] = SwEv{sw_hi(sw_ng(sh, m, 1, ks[u]), 0, ks[u]), sweep, ks[u]};
                        B.cst[cs[u]] = (win << 2) | 3u;
                    }
                    push_warp(sh.la, 0, pops, cs[u]);
                    // survivors: compacted with one atomic per warp
                    const bool keep = in && !pops;
                    const unsigned b = __ballot_sync(0xffffffffu, keep);
                    if (b)
                    {
                        const int lane = tid & 31, lead = __ffs(b) - 1;
                        std::uint32_t base = 0;
                        if (lane == lead) base = atomicAdd(&sh.cnt[3], static_cast<std::uint32_t>(__popc(b)));
                        base = __shfl_sync(0xffffffffu, base, lead);
                        if (keep)
                        {
                            const std::uint32_t k2 = base + __popc(b & ((1u << lane) - 1u));
                            dc2[k2] = cs[u];
                            dk2[k2] = ks[u];
                        }
                    }
                }
            }
        }
        // list cells below Vmax (the sorted list from s_p on) pop too
        for (;;)
        {
            const std::int64_t p0 = s_p;
            const std::int64_t q = p0 + tid;
            bool past = q >= G.nsorted;
            bool pops = false;
            std::uint32_t c = 0;
            if (!past)
            {
                const float4 o = G.ordRec[q];
                if (!(o.x < Vmax)) past = true;
                else if (o.y < S)
                {
                    c = __float_as_uint(o.z);
                    B.ev[c] = SwEv{sw_hi(sw_ng(sh, m, 1, o.x), 0, o.x), sweep, o.x};
                    pops = true;
                }
            }
            push_warp(sh.la, 0, pops, c);
            if (tid == 0) sh.red_p = G.nsorted + 1;
            __syncthreads();
            if (past) atomicMin(reinterpret_cast<unsigned long long*>(&sh.red_p), static_cast<unsigned long long>(q));
            __syncthreads();
            const std::int64_t stop = sh.red_p;
            __syncthreads();
            if (stop <= G.nsorted)
            {
                if (tid == 0) s_p = stop;
                break;
            }
            if (tid == 0) s_p = p0 + kSwThreads;
            __syncthreads();
        }
        __syncthreads();
        // rounds: re-evaluate the not-yet-queued cells next to changed pops
        std::uint32_t* la = sh.la;
        std::uint32_t* lb = sh.lb;
        int rounds = 0;
        for (;;)
        {
            const std::uint32_t nch = min(sh.cnt[0], static_cast<std::uint32_t>(kSwL));
            if (nch == 0 || sh.cnt[5]) break;
            // a sweep settles in two or three rounds; one that has not after
            // 64 leaves the window to the sequential rules
            if (++rounds > 64)
            {
                __syncthreads();
                if (tid == 0) sh.cnt[5] = 1;
                __syncthreads();
                break;
            }
            const std::uint32_t round = sweep + static_cast<std::uint32_t>(rounds);
            for (std::uint32_t t = tid; t < nch * 8; t += kSwThreads)
            {
                const std::uint32_t c = la[t >> 3];
                const int dd = static_cast<int>(t & 7);
                const int r0 = static_cast<int>(c / static_cast<std::uint32_t>(G.nc));
                const int c0 = static_cast<int>(c - static_cast<std::uint32_t>(r0) * G.nc);
                int rr, cc;
                if (!fill_nb(G.nr, G.nc, G.per_ns, G.per_ew, r0, c0, dd, rr, cc)) continue;
                const std::uint32_t j = static_cast<std::uint32_t>(rr) * G.nc + cc;
                // every load the evaluation needs, issued before any is used:
                // j's record and state, the records of its eight neighbours
                std::uint32_t nbs[8];
#pragma unroll
                for (int d = 0; d < 8; ++d)
                {
                    int r2, c2;
                    nbs[d] = fill_nb(G.nr, G.nc, G.per_ns, G.per_ew, rr, cc, d, r2, c2)
                                 ? static_cast<std::uint32_t>(r2) * G.nc + c2
                                 : kWinNone;
                }
                const float4 qj = G.rec[j];
                const std::uint32_t cj = B.cst[j];
                SwEv evs[8];
#pragma unroll
                for (int d = 0; d < 8; ++d) evs[d] = B.ev[nbs[d] != kWinNone ? nbs[d] : j];
                const SwEv self = B.ev[j];
                const float zj = qj.x;
                if (!(qj.w != 0.0f && qj.y >= S && !(qj.z < S) && (cj >> 2) != win)) continue;
                // one thread per cell and round: the cell's records have a
                // single writer within the round (an older mark: first
                // visit in this sweep, listed for the finalisation)
                const std::uint32_t prev_mark = atomicExch(&B.mk_c[j], round);
                if (prev_mark == round) continue;
                if (prev_mark <= sweep) push_list(sh.lt, 2, j);
                // the neighbour of j that pops first, and its direction to j
                std::uint64_t bh = ~0ull;
                std::uint32_t bl = ~0u;
                float bval = 0.0f;
                int bk = 8;
#pragma unroll
                for (int d = 0; d < 8; ++d)
                {
                    if (nbs[d] == kWinNone || evs[d].st != sweep) continue;
                    const std::uint64_t h = evs[d].hi;
                    const std::uint32_t l = ((h >> 32) & 1u) ? 0u : nbs[d];
                    const int k = (d + 4) & 7;
                    if (h < bh || (h == bh && (l < bl || (l == bl && k < bk))))
                    {
                        bh = h;
                        bl = l;
                        bk = k;
                        bval = evs[d].val;
                    }
                }
                const bool was_ev = self.st == sweep;
                if (bk == 8)
                {
                    // no pop next to it any more: not discovered in this sweep
                    B.te_st[j] = 0;
                    if (was_ev)
                    {
                        B.ev[j].st = 0;
                        push_list(lb, 1, j);
                    }
                    continue;
                }
                B.te[j] = SwTe{bh, bl, bval};
                B.te_k[j] = static_cast<std::uint8_t>(bk);
                B.te_st[j] = sweep;
                bool ev = false;
                std::uint64_t nh = 0;
                if (!(zj <= bval))
                {
                    const std::uint32_t gd = static_cast<std::uint32_t>(bh >> 33);
                    const std::uint32_t gpush = ((bh >> 32) & 1u) ? gd + 1 : gd;
                    const std::uint32_t g = sw_ng(sh, m, gpush, zj);
                    if (g <= m)
                    {
                        ev = true;
                        nh = sw_hi(g, 0, zj);
                    }
                }
                if (ev)
                {
                    if (!was_ev || self.hi != nh)
                    {
                        B.ev[j] = SwEv{nh, sweep, zj};
                        push_list(lb, 1, j);
                    }
                }
                else if (was_ev)
                {
                    B.ev[j].st = 0;
                    push_list(lb, 1, j);
                }
            }
            __syncthreads();
            if (tid == 0)
            {
                sh.cnt[0] = sh.cnt[1];
                sh.cnt[1] = 0;
            }
            std::uint32_t* t = la;
            la = lb;
            lb = t;
            __syncthreads();
        }
        __syncthreads();
        if (sh.cnt[5] || sh.cnt[2] > static_cast<std::uint32_t>(kSwL))
        {
            if (tid == 0) s_status = kWinOverflow;
            __syncthreads();
            break;
        }
        // finalize: pops, next FIFO, heap cells
        float vmax_pop = -INFINITY;
        for (std::uint32_t g = tid; g < m; g += kSwThreads)
        {
            const std::uint32_t c = sh.fc[g];
            out_F[c] = sh.fv[g];
            B.cst[c] = (win << 2) | 3u;
            vmax_pop = fmaxf(vmax_pop, sh.fv[g]);
        }
        const std::uint32_t nt = sh.cnt[2];
        for (std::uint32_t t = tid; t < nt; t += kSwThreads)
        {
            const std::uint32_t j = sh.lt[t];
            const std::uint32_t tst = B.te_st[j];
            const float zj = G.rec[j].x;
            const SwEv e = B.ev[j];
            const SwTe d = B.te[j];
            const int dk_dir = B.te_k[j];
            if (tst != sweep) continue;
            if (e.st == sweep)
            {
                B.cst[j] = (win << 2) | 3u;
                vmax_pop = fmaxf(vmax_pop, zj);
            }
            else if (zj <= d.val)
            {
                const std::uint32_t s2 = atomicAdd(&sh.cnt[4], 1u);
                if (s2 < static_cast<std::uint32_t>(kSwFQ))
                {
                    const int k = dk_dir;
                    sh.nc[s2] = j;
                    sh.nv[s2] = raise_from(d.val, G.eps, (k & 1) ? G.Ld : G.L);
                    sh.nhi[s2] = d.hi;
                    sh.nlo[s2] = d.lo;
                    sh.nk[s2] = static_cast<std::uint8_t>(k);
                }
                B.cst[j] = (win << 2) | 2u;
            }
            else
            {
                if (zj < s_T)
                {
                    const std::uint32_t s2 = atomicAdd(&sh.cnt[3], 1u);
                    dc2[s2] = j;
                    dk2[s2] = zj;
                }
                else
                {
                    const int k = level_of(zj);
                    const std::uint32_t s2 = s_nl[k] + atomicAdd(&sh.cnt[7 + k], 1u);
                    lvc(k)[s2] = j;
                    lvk(k)[s2] = zj;
                }
                B.cst[j] = (win << 2) | 1u;
            }
        }
        // the largest value popped: the FIFO's (list and earlier heap pops
        // are below Vmax, the FIFO's largest) or a discovered cell's
        for (int o = 16; o > 0; o >>= 1) vmax_pop = fmaxf(vmax_pop, __shfl_down_sync(0xffffffffu, vmax_pop, o));
        if ((tid & 31) == 0) sh.red_v[tid >> 5] = vmax_pop;
        __syncthreads();
        const std::uint32_t mn = sh.cnt[4];
        if (tid == 0)
        {
            float v = s_V;
            for (int k = 0; k < kSwThreads / 32; ++k) v = fmaxf(v, sh.red_v[k]);
            s_V = v;
            s_nd = sh.cnt[3];
            for (int k = 0; k < kSwLv; ++k) s_nl[k] += sh.cnt[7 + k];
            if (mn > static_cast<std::uint32_t>(kSwFQ)) s_status = kWinOverflow;
        }
        __syncthreads();
        if (s_status != kWinOk) break;
        // the next FIFO in push order (discoverer's T, direction): each entry
        // counts the entries before it (keys are distinct); up to 32 entries
        // within warp 0 by shuffles, past 64 by a bitonic sort of indices
        // (ng is free until the next sweep builds it)
        if (mn > 64)
        {
            const std::uint32_t P = 1u << (32 - __clz(mn - 1));
            for (std::uint32_t t = tid; t < P; t += kSwThreads) sh.ng[t] = static_cast<std::uint16_t>(t);
            __syncthreads();
            // a after b in push order (indices past mn last)
            auto after = [&](std::uint32_t a, std::uint32_t b) {
                if (a >= mn) return b < mn || a > b;
                if (b >= mn) return false;
                const std::uint64_t ah = sh.nhi[a], bh = sh.nhi[b];
                if (ah != bh) return ah > bh;
                const std::uint32_t al = sh.nlo[a], bl = sh.nlo[b];
                if (al != bl) return al > bl;
                return sh.nk[a] > sh.nk[b];
            };
            for (std::uint32_t k = 2; k <= P; k <<= 1)
                for (std::uint32_t j = k >> 1; j > 0; j >>= 1)
                {
                    for (std::uint32_t i = tid; i < P; i += kSwThreads)
                    {
                        const std::uint32_t l = i ^ j;
                        if (l > i)
                        {
                            const std::uint32_t a = sh.ng[i], b = sh.ng[l];
                            if (after(a, b) == ((i & k) == 0))
                            {
                                sh.ng[i] = static_cast<std::uint16_t>(b);
                                sh.ng[l] = static_cast<std::uint16_t>(a);
                            }
                        }
                    }
                    __syncthreads();
                }
            for (std::uint32_t r = tid; r < mn; r += kSwThreads)
            {
                const std::uint32_t a = sh.ng[r];
                sh.fc[r] = sh.nc[a];
                sh.fv[r] = sh.nv[a];
            }
        }
        else if (mn <= 32)
        {
            if (tid < 32)
            {
                const bool in = static_cast<std::uint32_t>(tid) < mn;
                const std::uint64_t ah = in ? sh.nhi[tid] : ~0ull;
                const std::uint32_t al = in ? sh.nlo[tid] : ~0u;
                const std::uint32_t ak = in ? sh.nk[tid] : 255u;
                const std::uint32_t ac = in ? sh.nc[tid] : 0u;
                const float av = in ? sh.nv[tid] : 0.0f;
                std::uint32_t rank = 0;
                for (int b = 0; b < 32; ++b)
                {
                    const std::uint64_t bh = __shfl_sync(0xffffffffu, ah, b);
                    const std::uint32_t bl = __shfl_sync(0xffffffffu, al, b);
                    const std::uint32_t bk = __shfl_sync(0xffffffffu, ak, b);
                    if (static_cast<std::uint32_t>(b) < mn &&
                        (bh < ah || (bh == ah && (bl < al || (bl == al && bk < ak)))))
                        ++rank;
                }
                if (in)
                {
                    sh.fc[rank] = ac;
                    sh.fv[rank] = av;
                }
            }
        }
        else
        for (std::uint32_t a = tid; a < mn; a += kSwThreads)
        {
            const std::uint64_t ah = sh.nhi[a];
            const std::uint32_t al = sh.nlo[a];
            const std::uint8_t ak = sh.nk[a];
            std::uint32_t rank = 0;
            for (std::uint32_t b = 0; b < mn; ++b)
            {
                const std::uint64_t bh = sh.nhi[b];
                if (bh < ah || (bh == ah && (sh.nlo[b] < al || (sh.nlo[b] == al && sh.nk[b] < ak)))) ++rank;
            }
            sh.fc[rank] = sh.nc[a];
            sh.fv[rank] = sh.nv[a];
        }
        __syncthreads();
        if (tid == 0) s_m = mn;
        {
            std::uint32_t* t1 = dc;
            dc = dc2;
            dc2 = t1;
            float* t2 = dk;
            dk = dk2;
            dk2 = t2;
        }
        __syncthreads();
    }
    if (tid == 0) *ctr = s_ctr;
    __syncthreads();
    *next = s_next;  // every thread: the caller's control flow stays uniform
    const int status = static_cast<int>(s_status);
    __syncthreads();  // s_* are reused by the next call
    return status;
}

}  // namespace
}  // namespace lsdtt_gb300
