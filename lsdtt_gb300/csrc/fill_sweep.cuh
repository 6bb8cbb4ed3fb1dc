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
// as a fixed point, found by re-evaluating the cells next to changed pops
// until nothing changes (a changed pop can only move the cells next to it).
// Between sweeps and when the FIFO runs empty the block falls back to the
// sequential rules of win_replay (one pop at a time).
#pragma once

#include <cstdint>

#include "fill_window.cuh"

namespace lsdtt_gb300
{
namespace
{

constexpr int kSwThreads = 256;
constexpr int kSwFQ = 2048;  // FIFO entries per sweep held in shared memory

// Per-member scratch of the block replay (member-local, one entry per cell
// unless stated). Stamps make every array valid without clearing: a value
// counts only when it carries the current window's, sweep's or round's id.
struct SweepBufs
{
    std::uint32_t* cst;      // (window id << 2) | 1 heap, 2 FIFO, 3 popped
    std::uint32_t* ev_st;    // sweep id of the cell's pop in this sweep
    std::uint64_t* ev_hi;    // (gap << 33) | (kind << 32) | value key
    float* ev_val;
    std::uint32_t* mk_c;     // round id: listed as a candidate this round
    std::uint32_t* mk_t;     // sweep id: discovered (tentatively) in this sweep
    std::uint32_t* te_st;    // sweep id: tentative discoverer below is valid
    std::uint64_t* te_hi;    // discoverer's T (hi word)
    std::uint32_t* te_lo;    //   and tie word (its cell for heap pops, 0 for FIFO)
    float* te_val;           //   and value
    std::uint8_t* te_k;      //   and direction
    std::uint32_t *la, *lb;  // changed-cell lists
    std::uint32_t* lc;       // candidates of a round
    std::uint32_t* lt;       // cells discovered in this sweep
    std::uint32_t *dc, *dc2; // heap cells discovered earlier, not popped (two buffers)
    float *dk, *dk2;         //   and their values
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
    std::uint32_t cnt[8];
    float red_v[kSwThreads / 32];
    std::uint32_t red_i[kSwThreads / 32];
    std::int64_t red_p;
};

__device__ __forceinline__ std::uint64_t sw_hi(std::uint32_t g, std::uint32_t kind, float key)
{
    return (static_cast<std::uint64_t>(g) << 33) | (static_cast<std::uint64_t>(kind) << 32) | float_order_key(key);
}

// first FIFO index >= g0 (1-based) whose value exceeds key; m + 1 if none
__device__ __forceinline__ std::uint32_t sw_ng(const SweepShared& sh, std::uint32_t m, std::uint32_t g0, float key)
{
    std::uint32_t g = g0;
    while (g <= m && !(sh.fv[g - 1] > key)) g = sh.ng[g];
    return g;
}

// Block replay of window w (every thread of a kSwThreads block calls it).
// *ctr is the member's id counter (stamps), advanced here. Returns kWinOk
// with *next set, or kWinOverflow (a sweep's FIFO above kSwFQ, or no fixed
// point within its round limit) -- then nothing of the window is final and
// the caller replays it by the sequential rules.
__device__ int win_sweep_replay(const WinGrid& G, int w, const SweepBufs& B, float* out_F, std::uint32_t* ctr,
                                SweepShared& sh, int* next)
{
    const int tid = threadIdx.x;
    const float S = G.cuts[w];
    __shared__ std::uint32_t s_ctr, s_m, s_nd, s_win, s_sweep, s_round, s_status;
    __shared__ std::int64_t s_p;
    __shared__ float s_V, s_Vmax;
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
        s_status = kWinOk;
        s_next = G.ncut;
        s_stop = 0;
    }
    __syncthreads();
    const std::uint32_t win = s_win;
    auto open_cell = [&](std::uint32_t j, float4& q) -> bool {
        q = G.rec[j];
        return q.w != 0.0f && q.y >= S && !(q.z < S) && (B.cst[j] >> 2) != win;
    };
    std::uint32_t* dc = B.dc;
    std::uint32_t* dc2 = B.dc2;
    float* dk = B.dk;
    float* dk2 = B.dk2;
    for (;;)
    {
        if (s_m == 0)
        {
            // ---- FIFO empty: one heap pop by the sequential rules ----
            // the list head (thread 0) and the least discovered heap cell
            if (tid == 0)
            {
                std::int64_t p = s_p;
                while (p < G.nsorted && !(G.ordRec[p].y < S)) ++p;
                s_p = p;
            }
            float bz = INFINITY;
            std::uint32_t bi = kWinNone, bslot = kWinNone;
            for (std::uint32_t t = tid; t < s_nd; t += kSwThreads)
                if (win_key_less(dk[t], dc[t], bz, bi))
                {
                    bz = dk[t];
                    bi = dc[t];
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
            __shared__ std::uint32_t s_slot[kSwThreads / 32];
            if ((tid & 31) == 0)
            {
                sh.red_v[tid >> 5] = bz;
                sh.red_i[tid >> 5] = bi;
                s_slot[tid >> 5] = bslot;
            }
            __syncthreads();
            if (tid == 0)
            {
                for (int k = 1; k < kSwThreads / 32; ++k)
                    if (win_key_less(sh.red_v[k], sh.red_i[k], bz, bi))
                    {
                        bz = sh.red_v[k];
                        bi = sh.red_i[k];
                        bslot = s_slot[k];
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
                            // remove from the discovered heap cells
                            const std::uint32_t last = --s_nd;
                            dc[bslot] = dc[last];
                            dk[bslot] = dk[last];
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
                            float4 q;
                            if (!open_cell(j, q)) continue;
                            if (q.x <= hz)
                            {
                                sh.fc[m] = j;
                                sh.fv[m] = raise_from(hz, G.eps, (d & 1) ? G.Ld : G.L);
                                ++m;
                                B.cst[j] = (win << 2) | 2u;
                            }
                            else
                            {
                                dc[s_nd] = j;
                                dk[s_nd] = q.x;
                                ++s_nd;
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
            s_sweep = ++s_ctr;
            // next greater FIFO value after each index (1-based, m + 1: none),
            // built right to left with pointer jumps
            sh.ng[m + 1] = static_cast<std::uint16_t>(m + 1);
            float vmax = -INFINITY;
            for (std::uint32_t g = m; g >= 1; --g)
            {
                std::uint32_t n = g + 1;
                while (n <= m && !(sh.fv[n - 1] > sh.fv[g - 1])) n = sh.ng[n];
                sh.ng[g] = static_cast<std::uint16_t>(n);
                vmax = fmaxf(vmax, sh.fv[g - 1]);
            }
            s_Vmax = vmax;
            sh.cnt[0] = 0;  // changed list (la)
            sh.cnt[1] = 0;  // next changed list (lb)
            sh.cnt[2] = 0;  // discovered in this sweep (lt)
            sh.cnt[3] = 0;  // surviving heap cells (dc2)
            sh.cnt[4] = 0;  // next FIFO
        }
        __syncthreads();
        const std::uint32_t sweep = s_sweep;
        const float Vmax = s_Vmax;
        // FIFO entries: pops (g, 1)
        for (std::uint32_t g = tid; g < m; g += kSwThreads)
        {
            const std::uint32_t c = sh.fc[g];
            B.ev_st[c] = sweep;
            B.ev_hi[c] = sw_hi(g + 1, 1, 0.0f);
            B.ev_val[c] = sh.fv[g];
            B.la[atomicAdd(&sh.cnt[0], 1u)] = c;
        }
        // heap cells discovered earlier: those below Vmax pop in this sweep
        for (std::uint32_t t = tid; t < s_nd; t += kSwThreads)
        {
            const std::uint32_t c = dc[t];
            const float k = dk[t];
            if (k < Vmax)
            {
                B.ev_st[c] = sweep;
                B.ev_hi[c] = sw_hi(sw_ng(sh, m, 1, k), 0, k);
                B.ev_val[c] = k;
                B.la[atomicAdd(&sh.cnt[0], 1u)] = c;
            }
            else
            {
                const std::uint32_t s2 = atomicAdd(&sh.cnt[3], 1u);
                dc2[s2] = c;
                dk2[s2] = k;
            }
        }
        // list cells below Vmax (the sorted list from s_p on) pop too
        for (;;)
        {
            const std::int64_t p0 = s_p;
            const std::int64_t q = p0 + tid;
            bool past = q >= G.nsorted;
            if (!past)
            {
                const float4 o = G.ordRec[q];
                if (!(o.x < Vmax)) past = true;
                else if (o.y < S)
                {
                    const std::uint32_t c = __float_as_uint(o.z);
                    B.ev_st[c] = sweep;
                    B.ev_hi[c] = sw_hi(sw_ng(sh, m, 1, o.x), 0, o.x);
                    B.ev_val[c] = o.x;
                    B.la[atomicAdd(&sh.cnt[0], 1u)] = c;
                }
            }
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
        std::uint32_t* la = B.la;
        std::uint32_t* lb = B.lb;
        int rounds = 0;
        for (;;)
        {
            const std::uint32_t nch = sh.cnt[0];
            if (nch == 0) break;
            if (++rounds > 4096)
            {
                if (tid == 0) s_status = kWinOverflow;
                break;
            }
            if (tid == 0)
            {
                s_round = ++s_ctr;
                sh.cnt[5] = 0;  // candidates of this round
            }
            __syncthreads();
            const std::uint32_t round = s_round;
            // candidates: open neighbours of changed cells, once each
            for (std::uint32_t t = tid; t < nch * 8; t += kSwThreads)
            {
                const std::uint32_t c = la[t >> 3];
                const int d = static_cast<int>(t & 7);
                const int r = static_cast<int>(c / static_cast<std::uint32_t>(G.nc));
                const int cc0 = static_cast<int>(c - static_cast<std::uint32_t>(r) * G.nc);
                int rr, cc;
                if (!fill_nb(G.nr, G.nc, G.per_ns, G.per_ew, r, cc0, d, rr, cc)) continue;
                const std::uint32_t j = static_cast<std::uint32_t>(rr) * G.nc + cc;
                float4 q;
                if (!open_cell(j, q)) continue;
                if (atomicExch(&B.mk_c[j], round) == round) continue;
                B.lc[atomicAdd(&sh.cnt[5], 1u)] = j;
            }
            __syncthreads();
            const std::uint32_t ncand = sh.cnt[5];
            if (tid == 0) sh.cnt[1] = 0;
            __syncthreads();
            for (std::uint32_t t = tid; t < ncand; t += kSwThreads)
            {
                const std::uint32_t j = B.lc[t];
                const int r = static_cast<int>(j / static_cast<std::uint32_t>(G.nc));
                const int c = static_cast<int>(j - static_cast<std::uint32_t>(r) * G.nc);
                // the neighbour that pops first, and its direction towards j
                std::uint64_t bh = ~0ull;
                std::uint32_t bl = ~0u, be = kWinNone;
                int bk = 8;
                for (int d = 0; d < 8; ++d)
                {
                    int rr, cc;
                    if (!fill_nb(G.nr, G.nc, G.per_ns, G.per_ew, r, c, d, rr, cc)) continue;
                    const std::uint32_t e = static_cast<std::uint32_t>(rr) * G.nc + cc;
                    if (B.ev_st[e] != sweep) continue;
                    const std::uint64_t h = B.ev_hi[e];
                    const std::uint32_t l = ((h >> 32) & 1u) ? 0u : e;
                    const int k = (d + 4) & 7;
                    if (h < bh || (h == bh && (l < bl || (l == bl && k < bk))))
                    {
                        bh = h;
                        bl = l;
                        be = e;
                        bk = k;
                    }
                }
                const bool was_ev = B.ev_st[j] == sweep;
                if (be == kWinNone)
                {
                    // no pop next to it any more: not discovered in this sweep
                    B.te_st[j] = 0;
                    if (was_ev)
                    {
                        B.ev_st[j] = 0;
                        lb[atomicAdd(&sh.cnt[1], 1u)] = j;
                    }
                    continue;
                }
                const float dval = B.ev_val[be];
                B.te_st[j] = sweep;
                B.te_hi[j] = bh;
                B.te_lo[j] = bl;
                B.te_val[j] = dval;
                B.te_k[j] = static_cast<std::uint8_t>(bk);
                if (atomicExch(&B.mk_t[j], sweep) != sweep) B.lt[atomicAdd(&sh.cnt[2], 1u)] = j;
                const float zj = G.rec[j].x;
                bool ev = false;
                std::uint64_t nh = 0;
                if (!(zj <= dval))
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
                    if (!was_ev || B.ev_hi[j] != nh)
                    {
                        B.ev_hi[j] = nh;
                        B.ev_val[j] = zj;
                        B.ev_st[j] = sweep;
                        lb[atomicAdd(&sh.cnt[1], 1u)] = j;
                    }
                }
                else if (was_ev)
                {
                    B.ev_st[j] = 0;
                    lb[atomicAdd(&sh.cnt[1], 1u)] = j;
                }
            }
            __syncthreads();
            if (tid == 0) sh.cnt[0] = sh.cnt[1];
            std::uint32_t* t = la;
            la = lb;
            lb = t;
            __syncthreads();
        }
        __syncthreads();
        if (s_status != kWinOk) break;
        // finalize: pops, next FIFO, heap cells
        float vmax_pop = -INFINITY;
        for (std::uint32_t g = tid; g < m; g += kSwThreads)
        {
            const std::uint32_t c = sh.fc[g];
            out_F[c] = sh.fv[g];
            B.cst[c] = (win << 2) | 3u;
            vmax_pop = fmaxf(vmax_pop, sh.fv[g]);
        }
        // heap pops among the cells queued before the sweep
        for (std::uint32_t t = tid; t < s_nd; t += kSwThreads)
            if (dk[t] < Vmax)
            {
                B.cst[dc[t]] = (win << 2) | 3u;
                vmax_pop = fmaxf(vmax_pop, dk[t]);
            }
        const std::uint32_t nt = sh.cnt[2];
        for (std::uint32_t t = tid; t < nt; t += kSwThreads)
        {
            const std::uint32_t j = B.lt[t];
            if (B.te_st[j] != sweep) continue;
            const float zj = G.rec[j].x;
            if (B.ev_st[j] == sweep)
            {
                B.cst[j] = (win << 2) | 3u;
                vmax_pop = fmaxf(vmax_pop, zj);
            }
            else if (zj <= B.te_val[j])
            {
                const std::uint32_t s2 = atomicAdd(&sh.cnt[4], 1u);
                if (s2 < kSwFQ)
                {
                    const int k = B.te_k[j];
                    sh.nc[s2] = j;
                    sh.nv[s2] = raise_from(B.te_val[j], G.eps, (k & 1) ? G.Ld : G.L);
                    sh.nhi[s2] = B.te_hi[j];
                    sh.nlo[s2] = B.te_lo[j];
                    sh.nk[s2] = static_cast<std::uint8_t>(k);
                }
                B.cst[j] = (win << 2) | 2u;
            }
            else
            {
                const std::uint32_t s2 = atomicAdd(&sh.cnt[3], 1u);
                dc2[s2] = j;
                dk2[s2] = zj;
                B.cst[j] = (win << 2) | 1u;
            }
        }
        // list pops' values: the largest is below Vmax; the sweep's largest
        // popped value is at least its largest FIFO value, which is Vmax
        for (int o = 16; o > 0; o >>= 1) vmax_pop = fmaxf(vmax_pop, __shfl_down_sync(0xffffffffu, vmax_pop, o));
        if ((tid & 31) == 0) sh.red_v[tid >> 5] = vmax_pop;
        __syncthreads();
        const std::uint32_t mn = sh.cnt[4];
        if (tid == 0)
        {
            float v = s_V;
            for (int k = 0; k < kSwThreads / 32; ++k) v = fmaxf(v, sh.red_v[k]);
            s_V = v;
            while (s_cnext < G.ncut && G.cuts[s_cnext] <= s_V) ++s_cnext;
            s_nd = sh.cnt[3];
            if (mn > kSwFQ) s_status = kWinOverflow;
        }
        __syncthreads();
        if (s_status != kWinOk) break;
        // the next FIFO in push order: (discoverer's T, direction); a
        // rank sort (each entry counts the entries before it)
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
        // swap the heap-cell buffers
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
