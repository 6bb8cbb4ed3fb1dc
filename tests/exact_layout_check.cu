// Host-only check of the exact fill's memory accounting
// (lsdtt_gb300/csrc/fill_exact.cuh): for a range of packed sizes, member
// counts and FIFO totals, ex_carve fits every buffer into ex_bytes(...)
// bytes, and what is left holds the largest scratch the radix sorts and
// scans of ex_run take (their Scratch::take calls replayed here). Runs no
// kernel and touches no device memory: the buffer base is a dummy address
// that is never dereferenced.
#include <cstdio>
#include <cstdint>

#include "fill_exact.cuh"

using namespace lsdtt_gb300;

// The takes of exclusive_scan over n items of `sz` bytes (recursive over
// its tile sums); false if one does not fit.
static bool scan_fits(Scratch& ws, std::int64_t n, std::size_t sz)
{
    if (n == 0) return true;
    const std::size_t mark = ws.used;
    const std::int64_t tiles = (n + kScanTile - 1) / kScanTile;
    const bool a = ws.take<unsigned char>(static_cast<std::size_t>(tiles + 1) * sz) != nullptr;
    const bool b = ws.take<unsigned char>(static_cast<std::size_t>(tiles + 1) * sz) != nullptr;
    bool ok = a && b && (tiles == 1 || scan_fits(ws, tiles, sz));
    ws.used = mark;
    return ok;
}

// The takes of radix_sort_pairs over n pairs, with the scan of its histograms.
static bool sort_fits(Scratch& ws, std::int64_t n)
{
    if (n <= 1) return true;
    const std::size_t mark = ws.used;
    const std::int64_t tiles = (n + kSortTile - 1) / kSortTile;
    const bool a = ws.take<std::uint32_t>(static_cast<std::size_t>(tiles) * 256) != nullptr;
    const bool b = ws.take<std::uint32_t>(static_cast<std::size_t>(tiles) * 256) != nullptr;
    const bool ok = a && b && scan_fits(ws, tiles * 256, sizeof(std::uint32_t));
    ws.used = mark;
    return ok;
}

int main()
{
    struct Case
    {
        std::int64_t N;
        int M;
    };
    const Case cases[] = {{256, 1}, {4096, 1}, {65536, 1}, {262144, 1}, {1 << 20, 4}, {89503232, 256},
                          {67108864, 1}, {2560, 10}, {300000 / 256 * 256 + 256, 3}};
    int bad = 0;
    for (const Case& c : cases)
    {
        // FIFO rings: a power of two of at least the member's cells each
        std::int64_t fifo_total = 0;
        const std::int64_t per = c.N / c.M;
        for (int k = 0; k < c.M; ++k)
        {
            std::int64_t cap = 2;
            while (cap < per) cap <<= 1;
            fifo_total += cap;
        }
        const std::size_t bytes = ex_bytes(c.N, c.M, fifo_total);
        Scratch ws{reinterpret_cast<char*>(std::uintptr_t(1) << 20), bytes, 0};
        ExBuffers B{};
        const bool carved = ex_carve(ws, c.N, c.M, fifo_total, B);
        const void* need[] = {B.rec, B.ordRec, B.key0, B.key1, B.pkey, B.val0, B.val1, B.cuts, B.cut_member, B.cand,
                              B.status, B.chain, B.next, B.off, B.cnt, B.diff, B.excl, B.wl, B.wl2, B.pool_c,
                              B.pool_v, B.stamp, B.ghk, B.gfq, B.sw.cst, B.sw.ev, B.sw.te, B.sw.te_st, B.sw.te_k,
                              B.sw.mk_c, B.sw.dc, B.sw.dc2, B.sw.dk, B.sw.dk2, B.sw.sc, B.sw.sk, B.sw.lc, B.sw.lk,
                              B.chain_order, B.sw_ctr, B.nsorted, B.ncut, B.cut_base, B.u, B.pool_used};
        bool all = carved;
        for (const void* p : need) all = all && p != nullptr;
        const bool sorts = sort_fits(ws, c.N);
        const bool scans = scan_fits(ws, c.N + 1, sizeof(int)) && scan_fits(ws, c.N, sizeof(std::uint32_t)) &&
                           scan_fits(ws, c.M, sizeof(int));
        std::printf("N %lld M %d: %zu bytes (%.1f a cell), carved %d, sort scratch %d, scan scratch %d\n",
                    static_cast<long long>(c.N), c.M, bytes, static_cast<double>(bytes) / static_cast<double>(c.N),
                    all ? 1 : 0, sorts ? 1 : 0, scans ? 1 : 0);
        if (!all || !sorts || !scans) ++bad;
    }
    std::printf(bad ? "FAIL\n" : "OK\n");
    return bad ? 1 : 0;
}
