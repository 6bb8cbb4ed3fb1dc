// A CPU restatement of the GPU's epsilon-fill method (lsdtt_gb300/csrc/
// fill_window.cuh, fill_exact.cuh, fill_sweep.cuh), for tests only: value
// windows cut at epsilon-0 pour levels, chained from the lowest cut, each
// replayed either by the sequential rules (the one-warp replay) or by FIFO
// sweeps whose pop times are a fixed point (the block replay). Plain
// containers, no attempt at speed. Seeds as the reference seeds them: the
// valid cells on non-periodic edges, and, when the interior holds nodata,
// the valid cells next to a nodata cell; nodata cells are never queued.
// tests/test_window_model.py holds its result to the oracle's priority flood
// with (row, col) heap ties, bit for bit, and the two replays to each other
// window by window.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <deque>
#include <limits>
#include <map>
#include <queue>
#include <unordered_map>
#include <unordered_set>
#include <utility>
#include <vector>

namespace
{

const int kDr[8] = {-1, -1, 0, 1, 1, 1, 0, -1};  // N, NE, E, SE, S, SW, W, NW
const int kDc[8] = {0, 1, 1, 1, 0, -1, -1, -1};

struct Grid
{
    int nr, nc;
    bool per_ns, per_ew;
    const std::uint8_t* valid;  // null: every cell valid
    std::vector<char> seeds;
    bool ok(std::size_t i) const { return !valid || valid[i] != 0; }
    bool nb(int r, int c, int d, int& rr, int& cc) const
    {
        rr = r + kDr[d];
        cc = c + kDc[d];
        if (per_ns) { if (rr < 0) rr += nr; else if (rr >= nr) rr -= nr; }
        if (per_ew) { if (cc < 0) cc += nc; else if (cc >= nc) cc -= nc; }
        return rr >= 0 && rr < nr && cc >= 0 && cc < nc;
    }
    bool seed(int r, int c) const { return seeds[static_cast<std::size_t>(r) * nc + c] != 0; }
    // the reference's seeding (raster_flow_preprocessing_cpu.cpp:518-589):
    // valid cells on a non-periodic edge, and next to an in-bounds nodata
    // cell when the interior holds any nodata
    void make_seeds()
    {
        seeds.assign(static_cast<std::size_t>(nr) * nc, 0);
        bool interior = false;
        for (int r = 1; r < nr - 1 && !interior; ++r)
            for (int c = 1; c < nc - 1; ++c)
                if (!ok(static_cast<std::size_t>(r) * nc + c)) { interior = true; break; }
        for (int r = 0; r < nr; ++r)
            for (int c = 0; c < nc; ++c)
            {
                const std::size_t i = static_cast<std::size_t>(r) * nc + c;
                if (!ok(i)) continue;
                bool s = (!per_ns && (r == 0 || r == nr - 1)) || (!per_ew && (c == 0 || c == nc - 1));
                for (int d = 0; d < 8 && !s && interior; ++d)
                {
                    const int rr = r + kDr[d], cc = c + kDc[d];
                    if (rr >= 0 && rr < nr && cc >= 0 && cc < nc && !ok(static_cast<std::size_t>(rr) * nc + cc))
                        s = true;
                }
                seeds[i] = s ? 1 : 0;
            }
    }
};

float raise_from(float v, float eps, float d)
{
    return std::max(v + eps * d, std::nextafter(v, std::numeric_limits<float>::infinity()));
}

// (value, cell) order of heap entries
struct Key
{
    float z;
    std::uint32_t i;
};
bool key_less(const Key& a, const Key& b) { return a.z < b.z || (a.z == b.z && a.i < b.i); }
struct KeyGreater
{
    bool operator()(const Key& a, const Key& b) const { return key_less(b, a); }
};
using MinHeap = std::priority_queue<Key, std::vector<Key>, KeyGreater>;

// Priority flood with (value, cell) ties; `value_order`: raised cells go to
// the heap (the value-ordered estimate) instead of the FIFO.
std::vector<float> flood(const float* z, const Grid& g, float L, float eps, bool value_order)
{
    const float Ld = L * 1.41421356237309504880f;
    const std::size_t n = static_cast<std::size_t>(g.nr) * g.nc;
    std::vector<float> F(z, z + n);
    std::vector<char> state(n, 0);  // 0 open, 1 queued, 2 popped
    MinHeap heap;
    std::deque<Key> fifo;
    for (int r = 0; r < g.nr; ++r)
        for (int c = 0; c < g.nc; ++c)
            if (g.seed(r, c))
            {
                const std::uint32_t i = static_cast<std::uint32_t>(r * g.nc + c);
                heap.push({F[i], i});
                state[i] = 1;
            }
    while (!heap.empty() || !fifo.empty())
    {
        Key cur;
        if (!fifo.empty() && (heap.empty() || fifo.front().z <= heap.top().z))
        {
            cur = fifo.front();
            fifo.pop_front();
        }
        else
        {
            cur = heap.top();
            heap.pop();
        }
        if (state[cur.i] == 2) continue;
        state[cur.i] = 2;
        const int r = static_cast<int>(cur.i) / g.nc, c = static_cast<int>(cur.i) % g.nc;
        for (int d = 0; d < 8; ++d)
        {
            int rr, cc;
            if (!g.nb(r, c, d, rr, cc)) continue;
            const std::uint32_t j = static_cast<std::uint32_t>(rr * g.nc + cc);
            if (state[j] || !g.ok(j)) continue;
            if (F[j] <= cur.z)
            {
                F[j] = eps > 0.0f ? raise_from(cur.z, eps, (d & 1) ? Ld : L) : cur.z;
                if (value_order) heap.push({F[j], j});
                else fifo.push_back({F[j], j});
            }
            else
                heap.push({F[j], j});
            state[j] = 1;
        }
    }
    return F;
}

// What every window needs: F0, min neighbour F0 (-inf for seeds), the cuts
// and their candidate flags, the cells sorted by (F0, cell).
struct Setup
{
    Grid g;
    const float* z;
    float L, Ld, eps;
    std::size_t n;
    std::vector<float> F0, mnb, cuts;
    std::vector<char> cand;
    std::vector<std::uint32_t> sorted;
};

Setup setup(const float* z, const Grid& g, float L, float eps)
{
    Setup X{g, z, L, L * 1.41421356237309504880f, eps, static_cast<std::size_t>(g.nr) * g.nc, {}, {}, {}, {}, {}};
    X.F0 = flood(z, g, L, 0.0f, false);
    const std::vector<float> F1 = flood(z, g, L, eps, true);
    X.mnb.assign(X.n, std::numeric_limits<float>::infinity());
    for (int r = 0; r < g.nr; ++r)
        for (int c = 0; c < g.nc; ++c)
        {
            const std::size_t i = static_cast<std::size_t>(r) * g.nc + c;
            if (!g.ok(i)) continue;  // never queued (mnb stays +inf)
            float m = std::numeric_limits<float>::infinity();
            bool pour = false;
            for (int d = 0; d < 8; ++d)
            {
                int rr, cc;
                if (!g.nb(r, c, d, rr, cc)) continue;
                const std::size_t b = static_cast<std::size_t>(rr) * g.nc + cc;
                if (!g.ok(b)) continue;
                m = std::min(m, X.F0[b]);
                // a pour level: c at or below F0(c), next to b with z(b) = F0(b) = F0(c)
                if (z[i] <= X.F0[i] && z[b] == X.F0[b] && X.F0[b] == X.F0[i]) pour = true;
            }
            X.mnb[i] = g.seed(r, c) ? -std::numeric_limits<float>::infinity() : m;
            if (pour) X.cuts.push_back(X.F0[i]);
        }
    std::sort(X.cuts.begin(), X.cuts.end());
    X.cuts.erase(std::unique(X.cuts.begin(), X.cuts.end()), X.cuts.end());
    // candidates: the lowest cut, and cuts inside no (F0(c), F1(c)] of a raised cell
    const int ncut = static_cast<int>(X.cuts.size());
    std::vector<int> diff(ncut + 1, 0);
    for (std::size_t i = 0; i < X.n; ++i)
        if (F1[i] > X.F0[i])
        {
            const int lo = static_cast<int>(std::upper_bound(X.cuts.begin(), X.cuts.end(), X.F0[i]) - X.cuts.begin());
            const int hi = static_cast<int>(std::upper_bound(X.cuts.begin(), X.cuts.end(), F1[i]) - X.cuts.begin());
            if (lo < hi)
            {
                ++diff[lo];
                --diff[hi];
            }
        }
    X.cand.assign(ncut, 0);
    int acc = 0;
    for (int k = 0; k < ncut; ++k)
    {
        acc += diff[k];
        X.cand[k] = (k == 0 || acc == 0) ? 1 : 0;
    }
    for (std::size_t i = 0; i < X.n; ++i)
        if (g.ok(i)) X.sorted.push_back(static_cast<std::uint32_t>(i));
    std::sort(X.sorted.begin(), X.sorted.end(),
              [&](std::uint32_t a, std::uint32_t b) { return key_less({X.F0[a], a}, {X.F0[b], b}); });
    return X;
}

using Outputs = std::vector<std::pair<std::uint32_t, float>>;

// The window's running maximum and the first cut above it.
struct Front
{
    const Setup& X;
    float V;
    int cnext;
    void pop(float v)
    {
        if (v > V)
        {
            V = v;
            while (cnext < static_cast<int>(X.cuts.size()) && X.cuts[cnext] <= V) ++cnext;
        }
    }
    // with the FIFO empty and `hm` the heap minimum: the window stops unless
    // a cut lies in [hm, V] or the next cut is no candidate
    bool stops(float hm) const
    {
        const bool trig = hm <= V && X.cuts[cnext - 1] >= hm;
        return !trig && (cnext >= static_cast<int>(X.cuts.size()) || X.cand[cnext]);
    }
};

// The sorted list from the window start S: the cells queued at S
// (F0 >= S with a neighbour below S, or seeds).
struct List
{
    const Setup& X;
    float S;
    std::size_t p;
    bool head(Key& k)
    {
        while (p < X.sorted.size() && !(X.mnb[X.sorted[p]] < S)) ++p;
        if (p >= X.sorted.size()) return false;
        k = {X.F0[X.sorted[p]], X.sorted[p]};
        return true;
    }
};

// The sequential rules (the one-warp replay); returns the next window start.
int replay_sequential(const Setup& X, int w, Outputs& out)
{
    const float S = X.cuts[w];
    List list{X, S, static_cast<std::size_t>(
                        std::lower_bound(X.sorted.begin(), X.sorted.end(), S,
                                         [&](std::uint32_t a, float v) { return X.F0[a] < v; }) -
                        X.sorted.begin())};
    Front front{X, S, w + 1};
    std::unordered_set<std::uint32_t> seen;
    MinHeap heap;
    std::deque<Key> fifo;
    for (;;)
    {
        Key lh{}, hm{std::numeric_limits<float>::infinity(), ~0u};
        const bool have_l = list.head(lh);
        bool from_list = false;
        if (have_l)
        {
            hm = lh;
            from_list = true;
        }
        if (!heap.empty() && (!have_l || key_less(heap.top(), lh)))
        {
            hm = heap.top();
            from_list = false;
        }
        const bool have_h = have_l || !heap.empty();
        Key cur;
        bool from_fifo = false;
        if (!fifo.empty() && (!have_h || fifo.front().z <= hm.z))
        {
            cur = fifo.front();
            fifo.pop_front();
            from_fifo = true;
        }
        else
        {
            if (fifo.empty() && (!have_h || front.stops(hm.z)))
                return have_h ? front.cnext : static_cast<int>(X.cuts.size());
            cur = hm;
            if (from_list) ++list.p;
            else heap.pop();
        }
        if (from_fifo) out.push_back({cur.i, cur.z});
        front.pop(cur.z);
        const int r = static_cast<int>(cur.i) / X.g.nc, c = static_cast<int>(cur.i) % X.g.nc;
        for (int d = 0; d < 8; ++d)
        {
            int rr, cc;
            if (!X.g.nb(r, c, d, rr, cc)) continue;
            const std::uint32_t j = static_cast<std::uint32_t>(rr * X.g.nc + cc);
            if (!X.g.ok(j) || X.F0[j] < S || X.mnb[j] < S || !seen.insert(j).second) continue;
            if (X.z[j] <= cur.z) fifo.push_back({raise_from(cur.z, X.eps, (d & 1) ? X.Ld : X.L), j});
            else heap.push({X.z[j], j});
        }
    }
}

// Pop time within a sweep: FIFO entry g at (g, 1); a heap cell of value k
// at (g, 0, k, cell), g the first FIFO index at or after its queueing whose
// value exceeds k.
struct Time
{
    std::uint32_t g, kind;
    float k;
    std::uint32_t i;
};
bool time_less(const Time& a, const Time& b)
{
    if (a.g != b.g) return a.g < b.g;
    if (a.kind != b.kind) return a.kind < b.kind;
    if (a.k != b.k) return a.k < b.k;
    return a.i < b.i;
}

// The block rules: one FIFO sweep at a time, its pop times a fixed point.
int replay_sweeps(const Setup& X, int w, Outputs& out, long long* sweeps)
{
    const float S = X.cuts[w];
    List list{X, S, static_cast<std::size_t>(
                        std::lower_bound(X.sorted.begin(), X.sorted.end(), S,
                                         [&](std::uint32_t a, float v) { return X.F0[a] < v; }) -
                        X.sorted.begin())};
    Front front{X, S, w + 1};
    std::unordered_map<std::uint32_t, int> state;  // 1 heap, 2 FIFO, 3 popped (list cells: by p)
    auto st = [&](std::uint32_t j) { const auto it = state.find(j); return it == state.end() ? 0 : it->second; };
    auto open = [&](std::uint32_t j) { return X.g.ok(j) && X.F0[j] >= S && !(X.mnb[j] < S) && st(j) == 0; };
    MinHeap heap;  // discovered heap cells (stale entries skipped by state)
    auto heap_top = [&](Key& k) {
        while (!heap.empty() && st(heap.top().i) != 1) heap.pop();
        if (heap.empty()) return false;
        k = heap.top();
        return true;
    };
    std::vector<std::pair<std::uint32_t, float>> fifo;  // the current sweep's FIFO
    for (;;)
    {
        if (fifo.empty())
        {
            // FIFO empty: one heap pop by the sequential rules
            Key lh{}, dh{}, hm{std::numeric_limits<float>::infinity(), ~0u};
            const bool have_l = list.head(lh), have_d = heap_top(dh);
            if (!have_l && !have_d) return static_cast<int>(X.cuts.size());
            bool from_list = have_l;
            hm = have_l ? lh : dh;
            if (have_d && (!have_l || key_less(dh, lh)))
            {
                hm = dh;
                from_list = false;
            }
            if (front.stops(hm.z)) return front.cnext;
            if (from_list) ++list.p;
            else
            {
                heap.pop();
                state[hm.i] = 3;
            }
            front.pop(hm.z);
            const int r = static_cast<int>(hm.i) / X.g.nc, c = static_cast<int>(hm.i) % X.g.nc;
            for (int d = 0; d < 8; ++d)
            {
                int rr, cc;
                if (!X.g.nb(r, c, d, rr, cc)) continue;
                const std::uint32_t j = static_cast<std::uint32_t>(rr * X.g.nc + cc);
                if (!open(j)) continue;
                if (X.z[j] <= hm.z)
                {
                    state[j] = 2;
                    fifo.push_back({j, raise_from(hm.z, X.eps, (d & 1) ? X.Ld : X.L)});
                }
                else
                {
                    state[j] = 1;
                    heap.push({X.z[j], j});
                }
            }
            continue;
        }
        ++*sweeps;
        const std::uint32_t m = static_cast<std::uint32_t>(fifo.size());
        std::vector<float> v(m), sufmax(m + 2, -std::numeric_limits<float>::infinity());
        for (std::uint32_t g = 0; g < m; ++g) v[g] = fifo[g].second;
        for (std::uint32_t g = m; g >= 1; --g) sufmax[g] = std::max(v[g - 1], sufmax[g + 1]);
        // first FIFO index >= g0 (1-based) whose value exceeds k; m + 1: none
        auto NG = [&](std::uint32_t g0, float k) {
            if (g0 > m || !(sufmax[g0] > k)) return m + 1;
            std::uint32_t g = g0;
            while (!(v[g - 1] > k)) ++g;
            return g;
        };
        const float vmax = sufmax[1];
        // pops fixed by the sweep's start: the FIFO, and the heap and list
        // cells below its largest value
        std::unordered_map<std::uint32_t, std::pair<Time, float>> fixed;
        for (std::uint32_t g = 0; g < m; ++g) fixed[fifo[g].first] = {Time{g + 1, 1, 0.0f, 0}, v[g]};
        for (Key k; list.head(k) && k.z < vmax; ++list.p) fixed[k.i] = {Time{NG(1, k.z), 0, k.z, k.i}, k.z};
        for (Key k; heap_top(k) && k.z < vmax;)
        {
            heap.pop();
            state[k.i] = 3;
            fixed[k.i] = {Time{NG(1, k.z), 0, k.z, k.i}, k.z};
        }
        // cells first discovered in this sweep: discoverer = the neighbouring
        // pop with the least time; a discovered heap cell pops in the sweep at
        // the first FIFO value above it after its discoverer -- to a fixed point
        struct Disc
        {
            Time t;
            int d;  // direction from the discoverer
            std::uint32_t by;
        };
        std::map<std::uint32_t, Disc> disc;
        std::map<std::uint32_t, std::pair<Time, float>> derived;
        for (int round = 0;; ++round)
        {
            if (round > 100000) return -1;
            std::map<std::uint32_t, Disc> nd;
            auto visit = [&](std::uint32_t e, const Time& te) {
                const int r = static_cast<int>(e) / X.g.nc, c = static_cast<int>(e) % X.g.nc;
                for (int d = 0; d < 8; ++d)
                {
                    int rr, cc;
                    if (!X.g.nb(r, c, d, rr, cc)) continue;
                    const std::uint32_t j = static_cast<std::uint32_t>(rr * X.g.nc + cc);
                    if (!open(j)) continue;
                    const auto it = nd.find(j);
                    if (it == nd.end() || time_less(te, it->second.t) ||
                        (!time_less(it->second.t, te) && d < it->second.d))
                        nd[j] = Disc{te, d, e};
                }
            };
            for (const auto& kv : fixed) visit(kv.first, kv.second.first);
            for (const auto& kv : derived) visit(kv.first, kv.second.first);
            std::map<std::uint32_t, std::pair<Time, float>> nder;
            for (const auto& kv : nd)
            {
                const std::uint32_t cell = kv.first;
                const Disc& dd = kv.second;
                const float dval = fixed.count(dd.by) ? fixed.at(dd.by).second : derived.at(dd.by).second;
                if (X.z[cell] <= dval) continue;  // raised: into the next FIFO
                const std::uint32_t gpush = dd.t.kind == 1 ? dd.t.g + 1 : dd.t.g;
                const std::uint32_t g = NG(gpush, X.z[cell]);
                if (g <= m) nder[cell] = {Time{g, 0, X.z[cell], cell}, X.z[cell]};
            }
            bool same = nder.size() == derived.size();
            for (auto a = nder.begin(), b = derived.begin(); same && a != nder.end(); ++a, ++b)
                same = a->first == b->first && !time_less(a->second.first, b->second.first) &&
                       !time_less(b->second.first, a->second.first);
            derived.swap(nder);
            disc.swap(nd);
            if (same) break;
        }
        // finish the sweep: its pops, the next FIFO in push order, heap cells
        for (std::uint32_t g = 0; g < m; ++g)
        {
            out.push_back(fifo[g]);
            state[fifo[g].first] = 3;
            front.pop(v[g]);
        }
        for (const auto& kv : fixed)
            if (kv.second.first.kind == 0) front.pop(kv.second.second);
        for (const auto& kv : derived)
        {
            state[kv.first] = 3;
            front.pop(kv.second.second);
        }
        struct Next
        {
            Time t;
            int d;
            std::uint32_t cell;
            float v;
        };
        std::vector<Next> next;
        for (const auto& kv : disc)
        {
            if (derived.count(kv.first)) continue;
            const Disc& dd = kv.second;
            const float dval = fixed.count(dd.by) ? fixed.at(dd.by).second : derived.at(dd.by).second;
            if (X.z[kv.first] <= dval)
            {
                // pushed in the order its discoverer meets its neighbours
                next.push_back({dd.t, dd.d, kv.first, raise_from(dval, X.eps, (dd.d & 1) ? X.Ld : X.L)});
                state[kv.first] = 2;
            }
            else
            {
                state[kv.first] = 1;
                heap.push({X.z[kv.first], kv.first});
            }
        }
        std::sort(next.begin(), next.end(), [](const Next& a, const Next& b) {
            if (time_less(a.t, b.t)) return true;
            if (time_less(b.t, a.t)) return false;
            return a.d < b.d;
        });
        fifo.clear();
        for (const Next& x : next) fifo.push_back({x.cell, x.v});
    }
}

}  // namespace

// The fill by chained windows (`valid` null: every cell valid; nodata cells
// keep their input). mode 0: sequential replays; 1: sweeps; 2: both,
// compared window by window (stats[3] counts windows that differ).
// stats: [0] cuts, [1] candidates, [2] windows on the chain, [3] windows
// whose two replays differ, [4] sweeps. Returns 0, or 1 if a chain did not
// advance, 2 if a sweep found no fixed point.
extern "C" int window_model_fill(const float* z, const std::uint8_t* valid, int nr, int nc, int per_ns, int per_ew,
                                 float L, float eps, int mode, float* out, long long* stats)
{
    Grid g{nr, nc, per_ns != 0, per_ew != 0, valid, {}};
    g.make_seeds();
    const Setup X = setup(z, g, L, eps);
    std::memcpy(out, z, sizeof(float) * X.n);
    const int ncut = static_cast<int>(X.cuts.size());
    long long cands = 0, chain = 0, differ = 0, sweeps = 0;
    for (char c : X.cand) cands += c;
    for (int w = 0; w < ncut;)
    {
        Outputs a, b;
        int nx = 0;
        if (mode != 1) nx = replay_sequential(X, w, a);
        if (mode != 0)
        {
            const int nb = replay_sweeps(X, w, b, &sweeps);
            if (nb < 0) return 2;
            if (mode == 1) nx = nb;
            else
            {
                std::sort(a.begin(), a.end());
                std::sort(b.begin(), b.end());
                bool same = nb == nx && a.size() == b.size();
                for (std::size_t k = 0; same && k < a.size(); ++k)
                    same = a[k].first == b[k].first && std::memcmp(&a[k].second, &b[k].second, 4) == 0;
                if (!same) ++differ;
            }
        }
        for (const auto& o : (mode == 1 ? b : a)) out[o.first] = o.second;
        ++chain;
        if (nx <= w) return 1;
        w = nx;
    }
    stats[0] = ncut;
    stats[1] = cands;
    stats[2] = chain;
    stats[3] = differ;
    stats[4] = sweeps;
    return 0;
}
