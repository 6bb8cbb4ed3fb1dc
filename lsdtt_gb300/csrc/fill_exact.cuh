// fill_exact.cuh -- the epsilon fill in the reference's order over packed
// grids (one grid = one member), from the epsilon-0 fill F0 and the
// value-ordered estimate F1 (see fill_window.cuh for the method).
//
// Stages, every launch of a fixed size (no host read-back, so an ensemble
// step can hold them in its CUDA graph):
//   1. per cell: min neighbour F0, sort keys, pour levels;
//   2. distinct pour levels per member, ascending (the cuts);
//   3. candidate window starts: cuts not inside (F0(c), F1(c)] of a cell
//      raised in the estimate;
//   4. the valid cells of each member sorted by (F0, index);
//   5. every candidate replayed by one warp with its state in shared memory
//      (three sizes, each taking the overflows of the one before; the two
//      larger only when the members that fill are fewer than the SMs);
//      raised cells staged in a pool;
//   6. per member, one block follows the chain of valid windows from the
//      lowest cut; a window on it that no size could hold is replayed by
//      the whole block one FIFO sweep at a time (fill_sweep.cuh), or, where
//      a sweep outgrows the block's shared memory, by the sequential rules
//      with the heap and FIFO in shared and then global memory;
//   7. the chain's staged cells committed.
#pragma once

#include <cstdint>

#include "common.cuh"
#include "engine.cuh"
#include "fill_sweep.cuh"
#include "fill_window.cuh"
#include "prims.cuh"

namespace lsdtt_gb300
{
namespace
{

struct ExMember
{
    std::int64_t base;       // first packed cell
    std::int64_t fifo_base;  // first entry of its global-tier FIFO ring
    std::uint32_t fifo_cap;  // power of two >= its cells
    std::int32_t nr, nc;
    float L, Ld, eps, nodata;
    std::int32_t per_ns, per_ew, on;  // on: the epsilon fill is replayed for this member
};

// Device buffers of the exact fill for N packed cells and M members.
struct ExBuffers
{
    float4 *rec, *ordRec;  // per cell and per sorted position (WinGrid)
    std::uint64_t *key0, *key1, *pkey;
    std::uint32_t *val0, *val1;
    float* cuts;
    std::int32_t* cut_member;
    std::uint8_t *cand, *status, *chain;
    std::int32_t* next;
    std::uint32_t *off, *cnt;
    int *diff, *excl;
    std::int32_t *wl, *wl2;
    std::uint32_t* pool_c;
    float* pool_v;
    std::uint64_t *gfq, *ghk;  // the global replay's FIFO and heap (WinStore)
    std::uint32_t* stamp;
    SweepBufs sw;           // the block replay's scratch (global cell indices; offset per member)
    std::uint32_t* sw_ctr;  // [M] stamp counters of the block replay
    std::int32_t* chain_order;  // [M] member of each chain block (largest members first)
    std::int64_t* nsorted;  // [M]
    int *ncut, *cut_base;   // [M], [M + 1]
    unsigned* u;            // [0] total cuts, [1] nwl, [2] work, [3] nwl2, [4] work2, [5] error,
                            // [6] nwl3, [7] work3, [8] pour keys
    unsigned long long* pool_used;
};

inline std::size_t ex_round(std::size_t b) { return (b + 255) & ~std::size_t(255); }

// Bytes of ExBuffers for N cells, M members and a global FIFO of fifo_total
// entries, plus the sort and scan scratch.
inline std::size_t ex_bytes(std::int64_t N, int M, std::int64_t fifo_total)
{
    const std::size_t n = static_cast<std::size_t>(N) + 1, m = static_cast<std::size_t>(M) + 1;
    const std::size_t tiles = static_cast<std::size_t>((N + kSortTile - 1) / kSortTile) + 2;
    std::size_t b = 0;
    for (std::size_t w : {16, 16, 8, 8, 8, 4, 4, 4, 4, 1, 1, 1, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4})
        b += ex_round(w * n);
    b += ex_round(8 * (n + 2));  // global heap
    // block replay: cst, ev, te, te_st, te_k, mk_c, dc, dc2, dk, dk2, sc, sk
    for (std::size_t w : {4, 16, 16, 4, 1, 4, 4, 4, 4, 4, 4, 4}) b += ex_round(w * n);
    b += 2 * ex_round(4 * static_cast<std::size_t>(kSwLv) * n);  // lc, lk
    b += ex_round(4 * m);  // chain order
    b += ex_round(4 * m);
    b += ex_round(8 * static_cast<std::size_t>(fifo_total) + 8);
    b += ex_round(8 * m) + 2 * ex_round(4 * m) + ex_round(64) + ex_round(8);
    b += tiles * 256 * 4 * 2 + tiles * 64 + (256 << 10);  // sort / scan scratch
    return b;
}

// Carve ExBuffers from ws (leaves the rest of ws for the sort and scans).
inline bool ex_carve(Scratch& ws, std::int64_t N, int M, std::int64_t fifo_total, ExBuffers& B)
{
    const std::size_t n = static_cast<std::size_t>(N) + 1, m = static_cast<std::size_t>(M) + 1;
    B.rec = ws.take<float4>(n);
    B.ordRec = ws.take<float4>(n);
    B.key0 = ws.take<std::uint64_t>(n);
    B.key1 = ws.take<std::uint64_t>(n);
    B.pkey = ws.take<std::uint64_t>(n);
    B.val0 = ws.take<std::uint32_t>(n);
    B.val1 = ws.take<std::uint32_t>(n);
    B.cuts = ws.take<float>(n);
    B.cut_member = ws.take<std::int32_t>(n);
    B.cand = ws.take<std::uint8_t>(n);
    B.status = ws.take<std::uint8_t>(n);
    B.chain = ws.take<std::uint8_t>(n);
    B.next = ws.take<std::int32_t>(n);
    B.off = ws.take<std::uint32_t>(n);
    B.cnt = ws.take<std::uint32_t>(n);
    B.diff = ws.take<int>(n);
    B.excl = ws.take<int>(n);
    B.wl = ws.take<std::int32_t>(n);
    B.wl2 = ws.take<std::int32_t>(n);
    B.pool_c = ws.take<std::uint32_t>(n);
    B.pool_v = ws.take<float>(n);
    B.stamp = ws.take<std::uint32_t>(n);
    B.ghk = ws.take<std::uint64_t>(n + 2);
    B.gfq = ws.take<std::uint64_t>(static_cast<std::size_t>(fifo_total) + 1);
    B.sw.cst = ws.take<std::uint32_t>(n);
    B.sw.ev = ws.take<SwEv>(n);
    B.sw.te = ws.take<SwTe>(n);
    B.sw.te_st = ws.take<std::uint32_t>(n);
    B.sw.te_k = ws.take<std::uint8_t>(n);
    B.sw.mk_c = ws.take<std::uint32_t>(n);
    B.sw.dc = ws.take<std::uint32_t>(n);
    B.sw.dc2 = ws.take<std::uint32_t>(n);
    B.sw.dk = ws.take<float>(n);
    B.sw.dk2 = ws.take<float>(n);
    B.sw.sc = ws.take<std::uint32_t>(n);
    B.sw.sk = ws.take<float>(n);
    B.sw.lc = ws.take<std::uint32_t>(static_cast<std::size_t>(kSwLv) * n);
    B.sw.lk = ws.take<float>(static_cast<std::size_t>(kSwLv) * n);
    B.sw.lstride = n;
    B.chain_order = ws.take<std::int32_t>(m);
    B.sw_ctr = ws.take<std::uint32_t>(m);
    B.nsorted = ws.take<std::int64_t>(m);
    B.ncut = ws.take<int>(m);
    B.cut_base = ws.take<int>(m);
    B.u = ws.take<unsigned>(16);
    B.pool_used = ws.take<unsigned long long>(1);
    return B.pool_used != nullptr;
}

__device__ __forceinline__ WinGrid ex_member_grid(const ExMember& M, int m, const float* z, const std::uint8_t* kind,
                                                  const float* F0, const ExBuffers& B)
{
    const int cb = B.cut_base[m];
    return WinGrid{M.nr, M.nc, M.per_ns != 0, M.per_ew != 0, M.L, M.Ld, M.eps, B.rec + M.base, B.ordRec + M.base,
                   B.nsorted[m], B.cuts + cb, B.cand + cb, B.ncut[m]};
}

// 1. Per cell: the replay record {z, F0, smallest F0 among valid neighbours
// (-inf for seeds), valid}, the cell sort key (member, F0; 2^32-1 puts
// invalid and NaN cells last in their member) and, for a pour cell, the
// pour-level key (member, F0), appended to a compact list counted in u[8].
// 256-thread blocks over the packed cells (a block never spans two members).
__global__ void ex_prep(const ExMember* __restrict__ mem, const std::uint16_t* __restrict__ blk_member,
                        std::int64_t N, const float* __restrict__ z, const std::uint8_t* __restrict__ kind,
                        const float* __restrict__ F0, ExBuffers B)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int m = blk_member[blockIdx.x];
    const ExMember M = mem[m];
    const std::uint64_t hi = static_cast<std::uint64_t>(m) << 32;
    const std::int64_t local = i - M.base;
    bool valid = false, has_pour = false;
    std::uint64_t pour_key = 0;
    if (i < N)
    {
        B.val0[i] = static_cast<std::uint32_t>(i);
        float zi = 0.0f;
        if (M.on && local < static_cast<std::int64_t>(M.nr) * M.nc && kind[i] != 0)
        {
            zi = z[i];
            valid = !isnan(zi);
        }
        if (!valid)
        {
            B.rec[i] = make_float4(0.0f, 0.0f, INFINITY, 0.0f);
            B.key0[i] = hi | 0xffffffffull;
        }
        else
        {
            const float f = F0[i];
            B.key0[i] = hi | float_order_key(f);
            const int r = static_cast<int>(local / M.nc), c = static_cast<int>(local - static_cast<std::int64_t>(r) * M.nc);
            float mn = INFINITY;
            bool pour = false;
            for (int d = 0; d < 8; ++d)
            {
                int rr, cc;
                if (!fill_nb(M.nr, M.nc, M.per_ns != 0, M.per_ew != 0, r, c, d, rr, cc)) continue;
                const std::int64_t j = M.base + static_cast<std::int64_t>(rr) * M.nc + cc;
                if (kind[j] == 0) continue;
                const float zj = z[j];
                if (isnan(zj)) continue;
                const float fj = F0[j];
                mn = fminf(mn, fj);
                if (zi <= f && zj == fj && fj == f) pour = true;
            }
            B.rec[i] = make_float4(zi, f, (kind[i] == 2) ? -INFINITY : mn, 1.0f);
            has_pour = pour;
            pour_key = hi | float_order_key(f);
        }
    }
    // the pour keys, compacted (one atomic per warp); their order is undone
    // by the sort
    const unsigned pb = __ballot_sync(0xffffffffu, has_pour);
    if (pb)
    {
        const int lane = threadIdx.x & 31, lead = __ffs(pb) - 1;
        unsigned base = 0;
        if (lane == lead) base = atomicAdd(&B.u[8], static_cast<unsigned>(__popc(pb)));
        base = __shfl_sync(0xffffffffu, base, lead);
        if (has_pour) B.pkey[base + __popc(pb & ((1u << lane) - 1u))] = pour_key;
    }
    const unsigned b = __ballot_sync(0xffffffffu, valid);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(reinterpret_cast<unsigned long long*>(&B.nsorted[m]),
                                                static_cast<unsigned long long>(__popc(b)));
}

// 2. First-of-run flags over the sorted pour-level keys, then the levels.
__global__ void ex_level_flags(const std::uint64_t* __restrict__ key, std::int64_t N,
                               const unsigned* __restrict__ nkeys, std::uint32_t* __restrict__ flag)
{
    LSDTT_COUNT();
    const std::int64_t k = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= N) return;
    if (k >= static_cast<std::int64_t>(*nkeys))
    {
        flag[k] = 0u;
        return;
    }
    const std::uint64_t v = key[k];
    flag[k] = (k == 0 || key[k - 1] != v) ? 1u : 0u;
}

__global__ void ex_level_scatter(const std::uint64_t* __restrict__ key, std::int64_t N,
                                 const std::uint32_t* __restrict__ flag, const std::uint32_t* __restrict__ pos,
                                 ExBuffers B)
{
    LSDTT_COUNT();
    const std::int64_t k = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= N || !flag[k]) return;
    const std::uint64_t v = key[k];
    const int m = static_cast<int>(v >> 32);
    B.cuts[pos[k]] = float_from_order_key(static_cast<std::uint32_t>(v));
    B.cut_member[pos[k]] = m;
    atomicAdd(&B.ncut[m], 1);
}

// 3. A cut in (F0(c), F1(c)] for a cell c raised in the value-ordered fill
// F1 most likely lies inside a running episode (c is still waiting when the
// heap reaches the cut): it is not replayed from. The estimate is used as it
// is: widening it merged valid windows on LEM inputs (epsilon ramps) into a
// few long ones, while a missed invalid cut costs one wasted replay.
__global__ void ex_cover(const ExMember* __restrict__ mem, const std::uint16_t* __restrict__ blk_member,
                         std::int64_t N, const float* __restrict__ z, const std::uint8_t* __restrict__ kind,
                         const float* __restrict__ F0, const float* __restrict__ F1, ExBuffers B)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int m = blk_member[blockIdx.x];
    const ExMember M = mem[m];
    if (i >= N || !M.on || i - M.base >= static_cast<std::int64_t>(M.nr) * M.nc || kind[i] == 0 || isnan(z[i]))
        return;
    const float f0 = F0[i], f1 = F1[i];
    if (!(f1 > f0)) return;
    const int cb = B.cut_base[m], nc = B.ncut[m];
    const int lo = static_cast<int>(win_upper_bound(B.cuts + cb, nc, f0));
    const int hi = static_cast<int>(win_upper_bound(B.cuts + cb, nc, f1));
    if (lo >= hi) return;
    atomicAdd(&B.diff[cb + lo], 1);
    atomicAdd(&B.diff[cb + hi], -1);
}

// Candidate flags (each member's lowest cut always: the first episode starts
// there with an empty FIFO) and the candidate list; every window unreplayed.
__global__ void ex_candidates(std::int64_t N, ExBuffers B)
{
    LSDTT_COUNT();
    const std::int64_t k = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= N || k >= static_cast<std::int64_t>(B.u[0])) return;
    const int m = B.cut_member[k];
    const bool c = k == B.cut_base[m] || B.excl[k] + B.diff[k] == 0;
    B.cand[k] = c ? 1 : 0;
    B.status[k] = 255;
    B.chain[k] = 0;
    if (c) B.wl[atomicAdd(&B.u[1], 1u)] = static_cast<std::int32_t>(k);
}

// 4. Sorted-order records {F0, mnb, member-local cell, 0} per sorted
// position (a member's sorted cells occupy its own packed range).
__global__ void ex_gather(const ExMember* __restrict__ mem, const std::uint16_t* __restrict__ blk_member,
                          std::int64_t N, const std::uint32_t* __restrict__ ord, ExBuffers B)
{
    LSDTT_COUNT();
    const std::int64_t p = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int m = blk_member[blockIdx.x];
    const ExMember M = mem[m];
    if (p >= N || p - M.base >= B.nsorted[m]) return;
    const std::uint32_t c = ord[p];
    const float4 q = B.rec[c];
    B.ordRec[p] = make_float4(q.y, q.z, __uint_as_float(static_cast<std::uint32_t>(c - M.base)), 0.0f);
}

// F before the windows write their raised cells: every valid cell at its own
// elevation (NaN cells stay NaN), invalid cells at the nodata value.
__global__ void ex_base(const ExMember* __restrict__ mem, const std::uint16_t* __restrict__ blk_member,
                        std::int64_t N, const float* __restrict__ z, const std::uint8_t* __restrict__ kind,
                        float* __restrict__ F)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int m = blk_member[blockIdx.x];
    const ExMember M = mem[m];
    if (i >= N || !M.on || i - M.base >= static_cast<std::int64_t>(M.nr) * M.nc) return;
    F[i] = kind[i] == 0 ? M.nodata : z[i];
}

// 5. Replays of the listed windows, one warp per block, the replay state in
// shared memory (FIFO FQ, heap DH, seen set HS, raised outputs OC). A window
// that outgrows any of them is marked kWinOverflow for the next size. Raised
// outputs are staged in the pool and committed only for chain windows.
template <int FQ, int DH, int HS, int OC>
__global__ void __launch_bounds__(32) ex_windows(const ExMember* __restrict__ mem, const float* __restrict__ z,
                                                 const std::uint8_t* __restrict__ kind, const float* __restrict__ F0,
                                                 ExBuffers B, const std::int32_t* __restrict__ wl,
                                                 const unsigned* __restrict__ nwl, unsigned* __restrict__ work,
                                                 unsigned long long pool_cap, unsigned long long pop_limit)
{
    LSDTT_COUNT();
    extern __shared__ __align__(16) unsigned char ex_smem[];
    WinStore s{};
    s.fq = reinterpret_cast<std::uint64_t*>(ex_smem);
    s.fcap = FQ;
    s.hk = s.fq + FQ;
    s.hcap = DH;
    s.hs = reinterpret_cast<std::uint32_t*>(s.hk + DH + 2);
    s.hscap = HS;
    s.oc = s.hs + HS;
    s.ov = reinterpret_cast<float*>(s.oc + OC);
    s.ocap = OC;
    const int lane = threadIdx.x & 31;
    const unsigned total = *nwl;
    for (;;)
    {
        unsigned t = 0;
        if (lane == 0) t = atomicAdd(work, 1u);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= total) break;
        const int g = wl[t];
        const int m = B.cut_member[g];
        const WinGrid G = ex_member_grid(mem[m], m, z, kind, F0, B);
        WinResult r = win_replay(G, g - B.cut_base[m], s, pop_limit);
        unsigned long long base = 0;
        if (r.status == kWinOk && r.nout)
        {
            if (lane == 0) base = atomicAdd(B.pool_used, static_cast<unsigned long long>(r.nout));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base + r.nout > pool_cap) r.status = kWinOverflow;
            else
                for (std::uint32_t k = lane; k < r.nout; k += 32)
                {
                    B.pool_c[base + k] = s.oc[k];
                    B.pool_v[base + k] = s.ov[k];
                }
        }
        if (lane == 0)
        {
            B.next[g] = r.next;
            B.status[g] = static_cast<std::uint8_t>(r.status);
            B.off[g] = static_cast<std::uint32_t>(base);
            B.cnt[g] = r.nout;
        }
        __syncwarp();
    }
}

// Windows of list `src` that one size could not hold, listed for the next.
__global__ void ex_overflow_list(std::int64_t N, const std::int32_t* __restrict__ src, const unsigned* __restrict__ nsrc,
                                 std::int32_t* __restrict__ dst, unsigned* __restrict__ ndst,
                                 const std::uint8_t* __restrict__ status)
{
    LSDTT_COUNT();
    const std::int64_t t = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= N || t >= static_cast<std::int64_t>(*nsrc)) return;
    const int g = src[t];
    if (status[g] == kWinOverflow) dst[atomicAdd(ndst, 1u)] = g;
}

// 6. The chain of each member, one block of kSwThreads per member (block m):
// from the lowest cut each window names the next valid start. A window on
// the chain that no shared-memory size held is replayed here by the
// whole block, one FIFO sweep at a time (fill_sweep.cuh); a sweep whose FIFO
// outgrows the block's shared memory sends the window to the sequential
// rules, run by warp 0 with the heap (DH_C) and FIFO (FQ_C) in the same
// shared memory, or past that in global memory. Either way the window's
// raised cells go straight into F. u[5] records a failure (1: a global
// replay outgrew its arrays; 2: the chain did not advance).
template <int FQ_C, int DH_C>
__global__ void __launch_bounds__(kSwThreads) ex_chain(const ExMember* __restrict__ mem, const float* __restrict__ z,
                                                       const std::uint8_t* __restrict__ kind,
                                                       const float* __restrict__ F0, float* __restrict__ F,
                                                       ExBuffers B)
{
    LSDTT_COUNT();
    extern __shared__ __align__(16) unsigned char ex_csmem[];
    const int tid = threadIdx.x, lane = tid & 31;
    const int m = B.chain_order[blockIdx.x];
    const ExMember M = mem[m];
    if (!M.on) return;
    const WinGrid G = ex_member_grid(M, m, z, kind, F0, B);
    const int cb = B.cut_base[m];
    SweepShared& sh = *reinterpret_cast<SweepShared*>(ex_csmem);
    SweepBufs sb = B.sw;
    {
        const std::int64_t o = M.base;
        sb.cst += o;
        sb.ev += o;
        sb.te += o;
        sb.te_st += o;
        sb.te_k += o;
        sb.mk_c += o;
        sb.dc += o;
        sb.dc2 += o;
        sb.dk += o;
        sb.dk2 += o;
        sb.sc += o;
        sb.sk += o;
        sb.lc += o;
        sb.lk += o;
    }
    WinStore mid{};
    mid.fq = reinterpret_cast<std::uint64_t*>(ex_csmem);
    mid.fcap = FQ_C;
    mid.hk = mid.fq + FQ_C;
    mid.hcap = DH_C;
    mid.stamp = B.stamp + M.base;
    mid.out_F = F + M.base;
    WinStore big = mid;
    big.fq = B.gfq + M.fifo_base;
    big.fcap = M.fifo_cap;
    // (1-based: index nr*nc lands at most on the next member's unused
    // entry 0, and the pair load reads one past it)
    big.hk = B.ghk + M.base;
    big.hcap = static_cast<std::uint32_t>(static_cast<std::int64_t>(M.nr) * M.nc);
    __shared__ std::uint32_t s_ctr;
    __shared__ int s_nx, s_fail;
    if (tid == 0)
    {
        s_ctr = B.sw_ctr[m];
        s_fail = 0;
    }
    __syncthreads();
    int w = 0;
    while (w < G.ncut)
    {
        int nx;
        if (B.status[cb + w] != kWinOk)
        {
            int sn = G.ncut;
            const int rs = win_sweep_replay(G, w, sb, F + M.base, &s_ctr, sh, &sn);
            if (rs == kWinOk)
                nx = sn;
            else
            {
                // the sequential rules, by warp 0 (the same shared memory)
                if (tid < 32)
                {
                    // seen-set stamps unique per window and attempt
                    mid.stamp_id = 2u * static_cast<std::uint32_t>(w) + 1u;
                    WinResult r = win_replay(G, w, mid, 0);
                    if (r.status != kWinOk)
                    {
                        big.stamp_id = 2u * static_cast<std::uint32_t>(w) + 2u;
                        r = win_replay(G, w, big, 0);
                    }
                    if (lane == 0)
                    {
                        s_nx = r.next;
                        s_fail = r.status != kWinOk ? 1 : 0;
                    }
                }
                __syncthreads();
                if (s_fail)
                {
                    if (tid == 0) atomicExch(&B.u[5], 1u);
                    return;
                }
                nx = s_nx;
            }
            if (tid == 0) B.chain[cb + w] = 2;
        }
        else
        {
            nx = B.next[cb + w];
            if (tid == 0) B.chain[cb + w] = 1;
        }
        __syncthreads();
        if (nx <= w)  // a window always ends above its start
        {
            if (tid == 0) atomicExch(&B.u[5], 2u);
            return;
        }
        w = nx;
    }
    if (tid == 0) B.sw_ctr[m] = s_ctr;
}

// 7. Staged raised cells of the chain windows into F, one warp per window.
__global__ void ex_commit(const ExMember* __restrict__ mem, std::int64_t N, float* __restrict__ F, ExBuffers B)
{
    LSDTT_COUNT();
    const int lane = threadIdx.x & 31;
    const std::int64_t warps = static_cast<std::int64_t>(gridDim.x) * (blockDim.x >> 5);
    const std::int64_t total = static_cast<std::int64_t>(B.u[0]);
    for (std::int64_t k = (static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
         k < total && k < N; k += warps)
    {
        if (B.chain[k] != 1) continue;
        float* Fm = F + mem[B.cut_member[k]].base;
        const std::uint32_t o = B.off[k], c = B.cnt[k];
        for (std::uint32_t t = lane; t < c; t += 32) Fm[B.pool_c[o + t]] = B.pool_v[o + t];
    }
}

constexpr int kExA_FQ = 128, kExA_DH = 256, kExA_HS = 1024, kExA_OC = 256;
// (windows past the small size are heap-bound: their FIFO stays short)
constexpr int kExM_FQ = 128, kExM_DH = 1024, kExM_HS = 4096, kExM_OC = 512;
constexpr int kExB_FQ = 128, kExB_DH = 4096, kExB_HS = 8192, kExB_OC = 1024;
constexpr std::size_t kExSmemA = 8 * kExA_FQ + 8 * (kExA_DH + 2) + 4 * kExA_HS + 8 * kExA_OC;
constexpr std::size_t kExSmemM = 8 * kExM_FQ + 8 * (kExM_DH + 2) + 4 * kExM_HS + 8 * kExM_OC;
constexpr std::size_t kExSmemB = 8 * kExB_FQ + 8 * (kExB_DH + 2) + 4 * kExB_HS + 8 * kExB_OC;
constexpr int kExC_FQ = 2048, kExC_DH = 16384;
constexpr std::size_t kExSmemC =
    (8 * kExC_FQ + 8 * (kExC_DH + 2)) > sizeof(SweepShared) ? (8 * kExC_FQ + 8 * (kExC_DH + 2)) : sizeof(SweepShared);

// Opt the larger replay sizes into their shared memory (current device).
inline cudaError_t ex_setup()
{
    cudaError_t e = cudaFuncSetAttribute(ex_windows<kExM_FQ, kExM_DH, kExM_HS, kExM_OC>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kExSmemM));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(ex_windows<kExB_FQ, kExB_DH, kExB_HS, kExB_OC>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kExSmemB));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(ex_chain<kExC_FQ, kExC_DH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(kExSmemC));
    return e;
}

// Enqueue the whole exact fill on st. On entry F holds the value-ordered
// estimate for the members that are on; on return (in stream order) their
// fill in the reference's order. `ws` holds the buffers carved by ex_carve
// and room for the sort and scan scratch. `mbits` = bits of the member index
// (0 for one member). Failures of the replays are left in B.u[5]. With
// profiling on, each stage is timed under its name (`ens`: the ensemble's
// names) with its algorithmic bytes: the records and keys it reads and
// writes once per cell; the replays count one 16-byte record per cell,
// though they are bound by the latency of their dependent steps. `n_on` =
// the members whose fill is on (their chains are the ones that work).
inline cudaError_t ex_run(const ExMember* mem, const std::uint16_t* blk_member, std::int64_t N, int M, int mbits,
                          const float* z, const std::uint8_t* kind, const float* F0, float* F, const ExBuffers& B,
                          Scratch& ws, int sms, cudaStream_t st, bool ens = false, int n_on = -1)
{
    if (n_on < 0) n_on = M;
    static const char* const kNames[2][9] = {
        {"fill_exact_prep", "fill_exact_levels", "fill_exact_candidates", "fill_exact_cell_sort",
         "fill_exact_windows_small", "fill_exact_windows_mid", "fill_exact_windows_large", "fill_exact_chain",
         "fill_exact_commit"},
        {"ens_fill_exact_prep", "ens_fill_exact_levels", "ens_fill_exact_candidates", "ens_fill_exact_cell_sort",
         "ens_fill_exact_windows_small", "ens_fill_exact_windows_mid", "ens_fill_exact_windows_large",
         "ens_fill_exact_chain", "ens_fill_exact_commit"}};
    const char* const* nm = kNames[ens ? 1 : 0];
    const double cells = static_cast<double>(N);
    const unsigned nb = static_cast<unsigned>(N / 256);
    cudaError_t e = cudaMemsetAsync(B.u, 0, 16 * sizeof(unsigned), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.pool_used, 0, sizeof(unsigned long long), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.nsorted, 0, sizeof(std::int64_t) * M, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.ncut, 0, sizeof(int) * M, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.diff, 0, sizeof(int) * (static_cast<std::size_t>(N) + 1), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.stamp, 0, sizeof(std::uint32_t) * static_cast<std::size_t>(N), st);
    // the block replay's stamps and counters start from zero on every run
    for (std::uint32_t* a : {B.sw.cst, B.sw.mk_c, B.sw.te_st})
        if (e == cudaSuccess) e = cudaMemsetAsync(a, 0, sizeof(std::uint32_t) * static_cast<std::size_t>(N), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.sw.ev, 0, sizeof(SwEv) * static_cast<std::size_t>(N), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(B.sw_ctr, 0, sizeof(std::uint32_t) * M, st);
    if (e != cudaSuccess) return e;
    // z 4, kind 1, F0 4 in; record 16, keys 8 + 8, value 4 out
    LSDTT_TIMED(nm[0], 45.0 * cells, st, (ex_prep<<<nb, 256, 0, st>>>(mem, blk_member, N, z, kind, F0, B)));
    const int bits = 32 + mbits;
    // distinct pour levels: the compacted pour keys sorted (the cell keys
    // stay in key0/val0 meanwhile; the values carried by that sort are not
    // used; wl2, off and cnt are free until the replays)
    auto levels = [&]() -> cudaError_t {
        cudaError_t le = cudaSuccess;
        const int r = radix_sort_pairs(B.pkey, reinterpret_cast<std::uint32_t*>(B.wl2), B.key1, B.val1, N, bits, ws,
                                       st, &le, B.u + 8);
        if (le != cudaSuccess) return le;
        const std::uint64_t* lk = r ? B.key1 : B.pkey;
        std::uint32_t* flag = B.off;
        std::uint32_t* pos = B.cnt;
        ex_level_flags<<<nb, 256, 0, st>>>(lk, N, B.u + 8, flag);
        le = exclusive_scan<std::uint32_t, std::uint32_t>(flag, N, pos, B.u, ws, st);
        if (le != cudaSuccess) return le;
        ex_level_scatter<<<nb, 256, 0, st>>>(lk, N, flag, pos, B);
        return exclusive_scan<int, int>(B.ncut, M, B.cut_base, static_cast<int*>(nullptr), ws, st);
    };
    LSDTT_TIMED(nm[1], 24.0 * cells, st, (e = levels()));
    if (e != cudaSuccess) return e;
    // candidate starts: record 16 and F 4 in per cell
    auto candidates = [&]() -> cudaError_t {
        ex_cover<<<nb, 256, 0, st>>>(mem, blk_member, N, z, kind, F0, F, B);
        const cudaError_t ce = exclusive_scan<int, int>(B.diff, N, B.excl, static_cast<int*>(nullptr), ws, st);
        if (ce != cudaSuccess) return ce;
        ex_candidates<<<nb, 256, 0, st>>>(N, B);
        return cudaSuccess;
    };
    LSDTT_TIMED(nm[2], 20.0 * cells, st, (e = candidates()));
    if (e != cudaSuccess) return e;
    // the valid cells of each member by (F0, index): keys and values in and
    // out, the sorted records out
    auto cell_sort = [&]() -> cudaError_t {
        cudaError_t ce = cudaSuccess;
        const int r = radix_sort_pairs(B.key0, B.val0, B.key1, B.val1, N, bits, ws, st, &ce);
        if (ce != cudaSuccess) return ce;
        ex_gather<<<nb, 256, 0, st>>>(mem, blk_member, N, r ? B.val1 : B.val0, B);
        ex_base<<<nb, 256, 0, st>>>(mem, blk_member, N, z, kind, F);
        return cudaSuccess;
    };
    LSDTT_TIMED(nm[3], 40.0 * cells, st, (e = cell_sort()));
    if (e != cudaSuccess) return e;
    // replays: small shared-memory size, then two larger ones for the
    // overflows of the one before (the sizes trade room for warps per SM:
    // 20, 7 and 3); wl is free again once the middle size has its list.
    // The larger sizes pay only where the chains are few: with a filling
    // member per SM or more, the chains' block sweeps replay the windows the
    // small size could not hold -- only those on a chain, where the larger
    // sizes replay every such candidate one pop at a time -- and the step
    // is faster without them (256 members: 358 ms a step with them, 234 ms
    // without; one 2048 x 2048 grid: 498 ms with them, 779 ms without)
    LSDTT_TIMED(nm[4], 16.0 * cells, st,
                (ex_windows<kExA_FQ, kExA_DH, kExA_HS, kExA_OC><<<sms * 20, 32, kExSmemA, st>>>(
                    mem, z, kind, F0, B, B.wl, B.u + 1, B.u + 2, static_cast<unsigned long long>(N), 16ull * kExA_HS)));
    if (n_on < sms)
    {
        LSDTT_TIMED(nm[5], 16.0 * cells, st,
                    (ex_overflow_list<<<nb, 256, 0, st>>>(N, B.wl, B.u + 1, B.wl2, B.u + 3, B.status),
                     ex_windows<kExM_FQ, kExM_DH, kExM_HS, kExM_OC><<<sms * 7, 32, kExSmemM, st>>>(
                         mem, z, kind, F0, B, B.wl2, B.u + 3, B.u + 4, static_cast<unsigned long long>(N),
                         16ull * kExM_HS)));
        LSDTT_TIMED(nm[6], 16.0 * cells, st,
                    (ex_overflow_list<<<nb, 256, 0, st>>>(N, B.wl2, B.u + 3, B.wl, B.u + 6, B.status),
                     ex_windows<kExB_FQ, kExB_DH, kExB_HS, kExB_OC><<<sms * 3, 32, kExSmemB, st>>>(
                         mem, z, kind, F0, B, B.wl, B.u + 6, B.u + 7, static_cast<unsigned long long>(N),
                         16ull * kExB_HS)));
    }
    LSDTT_TIMED(nm[7], 16.0 * cells, st,
                (ex_chain<kExC_FQ, kExC_DH><<<M, kSwThreads, kExSmemC, st>>>(mem, z, kind, F0, F, B)));
    // the staged raised cells: cell 4 + value 4 in, 4 out at most per cell
    LSDTT_TIMED(nm[8], 12.0 * cells, st,
                (ex_commit<<<static_cast<unsigned>(std::max<std::int64_t>(1, std::min<std::int64_t>(N / 8, sms * 64))),
                             256, 0, st>>>(mem, N, F, B)));
    return cudaGetLastError();
}

}  // namespace
}  // namespace lsdtt_gb300
