// prims.cuh -- data-parallel building blocks used by the routing kernels:
// exclusive scan, order-preserving compaction and a stable LSD radix sort.
// All are written for one GPU and one stream, sized in multiples of the SM
// count by the caller's grid choice, and allocate nothing: the caller passes
// a workspace (Scratch) carved from the engine's pool.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace lsdtt_gb300
{

// Bump allocator over one device buffer owned by an engine. Reset per build.
struct Scratch
{
    char* base = nullptr;
    std::size_t cap = 0;
    std::size_t used = 0;
    template <class T>
    T* take(std::size_t count)
    {
        std::size_t off = (used + 255) & ~std::size_t(255);
        std::size_t bytes = count * sizeof(T);
        if (off + bytes > cap) return nullptr;
        used = off + bytes;
        return reinterpret_cast<T*>(base + off);
    }
};

constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;                       // per thread
constexpr int kScanTile = kScanThreads * kScanItems;  // 4096

template <class T>
__device__ inline T block_exclusive_scan(T v, T* smem_warp, T& total)
{
    // Warp-level inclusive scan then a scan of warp totals.
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        T y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) smem_warp[warp] = x;
    __syncthreads();
    const int nw = blockDim.x >> 5;
    if (warp == 0)
    {
        T w = (lane < nw) ? smem_warp[lane] : T(0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            T y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nw) smem_warp[lane] = w;
    }
    __syncthreads();
    T warp_prefix = (warp > 0) ? smem_warp[warp - 1] : T(0);
    total = smem_warp[nw - 1];
    __syncthreads();
    return warp_prefix + x - v;
}

// Per-tile sums (each block reduces one tile of kScanTile inputs).
template <class TIn, class T>
__global__ void scan_tile_sums(const TIn* __restrict__ in, std::int64_t n, T* __restrict__ sums)
{
    LSDTT_COUNT();
    __shared__ T sw[32];
    const std::int64_t base = static_cast<std::int64_t>(blockIdx.x) * kScanTile;
    T acc = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
    {
        const std::int64_t k = base + static_cast<std::int64_t>(i) * kScanThreads + threadIdx.x;
        if (k < n) acc += static_cast<T>(in[k]);
    }
    T total;
    block_exclusive_scan<T>(acc, sw, total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// Exclusive scan of each tile plus the tile's offset. Each thread owns
// kScanItems consecutive elements so the output order is the input order.
template <class TIn, class T>
__global__ void scan_tile_apply(const TIn* __restrict__ in, std::int64_t n, const T* __restrict__ offs,
                                T* __restrict__ out)
{
    LSDTT_COUNT();
    __shared__ T sw[32];
    const std::int64_t base = static_cast<std::int64_t>(blockIdx.x) * kScanTile +
                              static_cast<std::int64_t>(threadIdx.x) * kScanItems;
    T v[kScanItems];
    T acc = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
    {
        const std::int64_t k = base + i;
        v[i] = (k < n) ? static_cast<T>(in[k]) : T(0);
        acc += v[i];
    }
    T total;
    T pre = block_exclusive_scan<T>(acc, sw, total) + offs[blockIdx.x];
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
    {
        const std::int64_t k = base + i;
        if (k < n) out[k] = pre;
        pre += v[i];
    }
}

// Host: exclusive scan of n values into out (out may alias nothing), and the
// grand total written to *total_dev (device). Workspace: ~n/4096*2 T.
template <class TIn, class T>
inline cudaError_t exclusive_scan(const TIn* in, std::int64_t n, T* out, T* total_dev, Scratch& ws,
                                  cudaStream_t st)
{
    const std::int64_t tiles = (n + kScanTile - 1) / kScanTile;
    if (n == 0)
    {
        if (total_dev) return cudaMemsetAsync(total_dev, 0, sizeof(T), st);
        return cudaSuccess;
    }
    const std::size_t mark = ws.used;
    T* sums = ws.take<T>(static_cast<std::size_t>(tiles) + 1);
    T* offs = ws.take<T>(static_cast<std::size_t>(tiles) + 1);
    if (!sums || !offs) return cudaErrorMemoryAllocation;
    scan_tile_sums<TIn, T><<<static_cast<unsigned>(tiles), kScanThreads, 0, st>>>(in, n, sums);
    if (tiles == 1)
    {
        cudaMemsetAsync(offs, 0, sizeof(T), st);
        if (total_dev) cudaMemcpyAsync(total_dev, sums, sizeof(T), cudaMemcpyDeviceToDevice, st);
    }
    else
    {
        cudaError_t e = exclusive_scan<T, T>(sums, tiles, offs, total_dev, ws, st);
        if (e != cudaSuccess) return e;
    }
    scan_tile_apply<TIn, T><<<static_cast<unsigned>(tiles), kScanThreads, 0, st>>>(in, n, offs, out);
    ws.used = mark;
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Stable LSD radix sort of (uint64 key, uint32 value) pairs over the low
// `bits` bits of the key, 8 bits per pass. Ping-pongs between (k0,v0) and
// (k1,v1); returns the buffer index (0 or 1) holding the result. With a
// device count `dn`, only the first min(n, *dn) pairs are sorted (the
// launches stay sized for n; tiles past the count do nothing).
// ---------------------------------------------------------------------------
constexpr int kSortThreads = 256;  // 8 warps
constexpr int kSortWarpItems = 512;  // per warp: 16 rounds of 32
constexpr int kSortTile = kSortWarpItems * (kSortThreads / 32);  // 4096

static __global__ void radix_hist(const std::uint64_t* __restrict__ keys, std::int64_t n, int shift,
                           std::uint32_t* __restrict__ hist, int n_tiles, const unsigned* __restrict__ dn)
{
    LSDTT_COUNT();
    if (dn && static_cast<std::int64_t>(*dn) < n) n = static_cast<std::int64_t>(*dn);
    __shared__ std::uint32_t h[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const std::int64_t base = static_cast<std::int64_t>(blockIdx.x) * kSortTile;
    for (int i = threadIdx.x; i < kSortTile; i += blockDim.x)
    {
        const std::int64_t k = base + i;
        if (k < n) atomicAdd(&h[(keys[k] >> shift) & 255u], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 256; i += blockDim.x)
        hist[static_cast<std::int64_t>(i) * n_tiles + blockIdx.x] = h[i];  // digit-major
}

static __global__ void radix_scatter(const std::uint64_t* __restrict__ kin, const std::uint32_t* __restrict__ vin,
                              std::int64_t n, int shift, const std::uint32_t* __restrict__ offs, int n_tiles,
                              std::uint64_t* __restrict__ kout, std::uint32_t* __restrict__ vout,
                              const unsigned* __restrict__ dn)
{
    LSDTT_COUNT();
    if (dn && static_cast<std::int64_t>(*dn) < n) n = static_cast<std::int64_t>(*dn);
    __shared__ std::uint32_t wcount[kSortThreads / 32][256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = lane; i < 256; i += 32) wcount[warp][i] = 0;
    __syncwarp();
    const std::int64_t wbase = static_cast<std::int64_t>(blockIdx.x) * kSortTile +
                               static_cast<std::int64_t>(warp) * kSortWarpItems;
    std::uint32_t rank[kSortWarpItems / 32];
    std::uint32_t dig[kSortWarpItems / 32];
#pragma unroll
    for (int r = 0; r < kSortWarpItems / 32; ++r)
    {
        const std::int64_t k = wbase + r * 32 + lane;
        const bool ok = k < n;
        const std::uint32_t d = ok ? static_cast<std::uint32_t>((kin[k] >> shift) & 255u) : 256u + lane;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const unsigned lower = peers & ((1u << lane) - 1u);
        std::uint32_t before = 0;
        if (ok) before = wcount[warp][d];
        rank[r] = before + __popc(lower);
        dig[r] = d;
        __syncwarp();
        // The highest lane of each peer group bumps the shared counter.
        if (ok && (peers >> lane) == 1u) wcount[warp][d] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // Exclusive prefix over warps, per digit: warp w's base for digit d.
    for (int d = threadIdx.x; d < 256; d += blockDim.x)
    {
        std::uint32_t acc = 0;
        for (int w = 0; w < kSortThreads / 32; ++w)
        {
            const std::uint32_t c = wcount[w][d];
            wcount[w][d] = acc;
            acc += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kSortWarpItems / 32; ++r)
    {
        const std::int64_t k = wbase + r * 32 + lane;
        if (k < n)
        {
            const std::uint32_t d = dig[r];
            const std::uint64_t pos = static_cast<std::uint64_t>(offs[static_cast<std::int64_t>(d) * n_tiles + blockIdx.x]) +
                                      wcount[warp][d] + rank[r];
            kout[pos] = kin[k];
            vout[pos] = vin[k];
        }
    }
}

inline int radix_sort_pairs(std::uint64_t* k0, std::uint32_t* v0, std::uint64_t* k1, std::uint32_t* v1,
                            std::int64_t n, int bits, Scratch& ws, cudaStream_t st, cudaError_t* err,
                            const unsigned* dn = nullptr)
{
    *err = cudaSuccess;
    if (n <= 1) return 0;
    const int tiles = static_cast<int>((n + kSortTile - 1) / kSortTile);
    const std::size_t mark = ws.used;
    std::uint32_t* hist = ws.take<std::uint32_t>(static_cast<std::size_t>(tiles) * 256);
    std::uint32_t* offs = ws.take<std::uint32_t>(static_cast<std::size_t>(tiles) * 256);
    if (!hist || !offs) { *err = cudaErrorMemoryAllocation; return 0; }
    int cur = 0;
    for (int shift = 0; shift < bits; shift += 8)
    {
        std::uint64_t* ki = cur ? k1 : k0;
        std::uint32_t* vi = cur ? v1 : v0;
        std::uint64_t* ko = cur ? k0 : k1;
        std::uint32_t* vo = cur ? v0 : v1;
        radix_hist<<<tiles, kSortThreads, 0, st>>>(ki, n, shift, hist, tiles, dn);
        *err = exclusive_scan<std::uint32_t, std::uint32_t>(hist, static_cast<std::int64_t>(tiles) * 256, offs,
                                                            static_cast<std::uint32_t*>(nullptr), ws, st);
        if (*err != cudaSuccess) return cur;
        radix_scatter<<<tiles, kSortThreads, 0, st>>>(ki, vi, n, shift, offs, tiles, ko, vo, dn);
        cur ^= 1;
    }
    ws.used = mark;
    *err = cudaGetLastError();
    return cur;
}

}  // namespace lsdtt_gb300
