// unet.cu -- the learned preconditioner for the implicit hillslope solves.
//
// A 4-level U-Net with additive skips maps a residual r to an approximate
// correction e ~ A^-1 r. It has no counterpart in the reference; the
// network is defined, with its rounding points, by the CPU restatement
// oracle/unet.py, which is also the oracle for these kernels:
//
//   x0 = bf16(r/rms(r));  e0 = relu(conv 1->16); e1 = relu(conv(pool) 16->32)
//   e2 = relu(conv(pool) 32->64); e3 = relu(conv(pool) 64->64)
//   d2 = relu(conv(up e3) 64->64) + e2; d1 = relu(conv(up d2) 64->32) + e1
//   d0 = relu(conv(up d1) 32->16) + e0; y = rms * conv(d0) 16->1
//
// Activations are bf16 in NHWC layout, weights bf16 [Cout][3][3][Cin] with
// an FP32 master copy, every accumulation FP32. The 3x3 convolutions with
// 16..64 input channels run as implicit GEMMs on the tensor cores (bf16
// mma.sync m16n8k16, FP32 accumulators): M = 16 output pixels per warp,
// N = Cout, K = 9*Cin gathered straight from the NHWC activations (zero
// padding at the borders, nearest-neighbour upsampling folded into the
// gather). The one-channel input and output layers and the backward pass
// (data and weight gradients, FP32) run on the CUDA cores; Adam updates the
// FP32 master weights and re-packs bf16 copies.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_bf16.h>

#include "engine.cuh"

namespace lsdtt_gb300
{
namespace
{

constexpr int kLayers = 8;
__host__ __device__ constexpr int layer_cin(int l)
{
    return l == 0 ? 1 : (l == 1 ? 16 : (l == 2 ? 32 : (l == 3 ? 64 : (l == 4 ? 64 : (l == 5 ? 64 : (l == 6 ? 32 : 16))))));
}
__host__ __device__ constexpr int layer_cout(int l)
{
    return l == 0 ? 16 : (l == 1 ? 32 : (l == 2 ? 64 : (l == 3 ? 64 : (l == 4 ? 64 : (l == 5 ? 32 : (l == 6 ? 16 : 1))))));
}

__device__ __forceinline__ float bfr(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

// ---------------------------------------------------------------------------
// forward
// ---------------------------------------------------------------------------
// Grid-wide sums are taken in a fixed order, so that the same inputs give the
// same bits on every run: each of the kRedBlocks blocks of a reduction covers
// a fixed grid-strided share of the cells and writes its own partial (warp
// shuffle tree, then the block's warps in index order); one block then adds
// the partials in a fixed tree (red_partials).
constexpr int kRedBlocks = 152 * 4;
// Pixel shares of one weight-gradient entry (k_conv_bwd_w's grid x).
constexpr int kWgradBlocks = 64;

// The block's sum of v (all threads take part), valid in thread 0.
__device__ __forceinline__ double block_sum_ordered(double v)
{
    __shared__ double sh_red[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();  // a previous call may still be reading
    if ((threadIdx.x & 31) == 0) sh_red[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < static_cast<int>(blockDim.x >> 5); ++k) t += sh_red[k];
    return t;
}

// out[j] = sum over b of part[j * np + b], one block per j, fixed order.
__global__ void red_partials(const double* __restrict__ part, int np, double* __restrict__ out)
{
    LSDTT_COUNT();
    const double* p = part + static_cast<std::int64_t>(blockIdx.x) * np;
    double s = 0.0;
    for (int b = threadIdx.x; b < np; b += blockDim.x) s += p[b];
    s = block_sum_ordered(s);
    if (threadIdx.x == 0) out[blockIdx.x] = s;
}

// part[blockIdx.x] = this block's share of sum r^2
__global__ void k_sumsq(const float* __restrict__ r, std::int64_t n, double* __restrict__ part)
{
    LSDTT_COUNT();
    std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    double s = 0.0;
    for (; i < n; i += static_cast<std::int64_t>(gridDim.x) * blockDim.x) s += static_cast<double>(r[i]) * r[i];
    s = block_sum_ordered(s);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// rms from the kRedBlocks partials of sum r^2 over n cells, summed in a fixed
// order (FP64 is scarce on this part: one block)
__global__ void k_rms(std::int64_t n, const double* __restrict__ part, float* __restrict__ rms_out)
{
    LSDTT_COUNT();
    double s = 0.0;
    for (int b = threadIdx.x; b < kRedBlocks; b += blockDim.x) s += part[b];
    s = block_sum_ordered(s);
    if (threadIdx.x != 0) return;
    float rms = static_cast<float>(sqrt(s / static_cast<double>(n)));
    if (!(rms > 0.0f)) rms = 1.0f;
    *rms_out = rms;
}

// x0 = bf16(r / rms)
__global__ void k_prep(const float* __restrict__ r, std::int64_t n, const float* __restrict__ rms_in,
                       __nv_bfloat16* __restrict__ x0)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const float rms = *rms_in;
    if (i < n) x0[i] = __float2bfloat16_rn(r[i] / rms);
}

// Layer 0 (1 -> 16 channels on CUDA cores: bias first, then the nine taps
// in order, ReLU, BF16) fused with the first 2x2 mean pool: thread (i, j) of
// the (H/2) x (W/2) grid computes e0 at its four pixels (2i + a, 2j + b) and
// p0(i, j) = (((a + b) + c) + d) x 0.25 of their BF16 values, the order
// k_pool uses, so e0 is written once and not read back.
__global__ void k_conv_in_pool(int H, int W, const __nv_bfloat16* __restrict__ x0, const float* __restrict__ wg,
                               const float* __restrict__ bg, __nv_bfloat16* __restrict__ e0,
                               __nv_bfloat16* __restrict__ p0)
{
    LSDTT_COUNT();
    __shared__ float w[16 * 9], b[16];
    for (int k = threadIdx.x; k < 16 * 9; k += blockDim.x) w[k] = wg[k];
    if (threadIdx.x < 16) b[threadIdx.x] = bg[threadIdx.x];
    __syncthreads();
    const int h = H / 2, wd = W / 2;
    const std::int64_t t = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= static_cast<std::int64_t>(h) * wd) return;
    const int i = static_cast<int>(t / wd), j = static_cast<int>(t % wd);
    float v[4][4];  // x0 rows 2i-1 .. 2i+2, columns 2j-1 .. 2j+2 (0 outside)
#pragma unroll
    for (int rr = 0; rr < 4; ++rr)
#pragma unroll
        for (int cc = 0; cc < 4; ++cc)
        {
            const int yy = 2 * i - 1 + rr, xx = 2 * j - 1 + cc;
            v[rr][cc] = (yy >= 0 && yy < H && xx >= 0 && xx < W)
                            ? __bfloat162float(x0[static_cast<std::int64_t>(yy) * W + xx])
                            : 0.f;
        }
    float pool[16];
#pragma unroll
    for (int q = 0; q < 4; ++q)
    {
        const int a = q >> 1, bq = q & 1;  // pixels (0,0), (0,1), (1,0), (1,1): k_pool's order
        alignas(16) __nv_bfloat16 o16[16];
#pragma unroll
        for (int co = 0; co < 16; ++co)
        {
            float s = b[co];
#pragma unroll
            for (int tp = 0; tp < 9; ++tp) s = __fadd_rn(s, __fmul_rn(v[a + tp / 3][bq + tp % 3], w[co * 9 + tp]));
            o16[co] = __float2bfloat16_rn(fmaxf(s, 0.f));
            const float e = __bfloat162float(o16[co]);
            pool[co] = (q == 0) ? e : pool[co] + e;
        }
        __nv_bfloat16* dst = e0 + (static_cast<std::int64_t>(2 * i + a) * W + 2 * j + bq) * 16;
        *reinterpret_cast<uint4*>(dst) = *reinterpret_cast<const uint4*>(o16);
        *reinterpret_cast<uint4*>(dst + 8) = *reinterpret_cast<const uint4*>(o16 + 8);
    }
    alignas(16) __nv_bfloat16 p16[16];
#pragma unroll
    for (int co = 0; co < 16; ++co) p16[co] = __float2bfloat16_rn(pool[co] * 0.25f);
    __nv_bfloat16* pd = p0 + t * 16;
    *reinterpret_cast<uint4*>(pd) = *reinterpret_cast<const uint4*>(p16);
    *reinterpret_cast<uint4*>(pd + 8) = *reinterpret_cast<const uint4*>(p16 + 8);
}

// 2x2 mean, bf16 -> bf16 (H, W are the OUTPUT sizes), eight channels per
// thread with 16-byte loads and stores (C a multiple of 8)
__global__ void k_pool(int H, int W, int C, const __nv_bfloat16* __restrict__ in, __nv_bfloat16* __restrict__ out)
{
    LSDTT_COUNT();
    const int G = C / 8;
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= static_cast<std::int64_t>(H) * W * G) return;
    const int c = static_cast<int>(i % G) * 8;
    const std::int64_t p = i / G;
    const int y = static_cast<int>(p / W), x = static_cast<int>(p % W);
    const int W2 = 2 * W;
    auto at = [&](int yy, int xx, __nv_bfloat16 (&v)[8]) {
        *reinterpret_cast<uint4*>(v) = *reinterpret_cast<const uint4*>(in + (static_cast<std::int64_t>(yy) * W2 + xx) * C + c);
    };
    alignas(16) __nv_bfloat16 a[8], b[8], d[8], e[8], o[8];
    at(2 * y, 2 * x, a);
    at(2 * y, 2 * x + 1, b);
    at(2 * y + 1, 2 * x, d);
    at(2 * y + 1, 2 * x + 1, e);
#pragma unroll
    for (int k = 0; k < 8; ++k)
    {
        const float s = ((__bfloat162float(a[k]) + __bfloat162float(b[k])) + __bfloat162float(d[k])) +
                        __bfloat162float(e[k]);
        o[k] = __float2bfloat16_rn(s * 0.25f);
    }
    *reinterpret_cast<uint4*>(out + p * C + c) = *reinterpret_cast<const uint4*>(o);
}

// Tensor-core 3x3 convolution, Cin and Cout multiples of 16 (Cin) / 8 (Cout).
// One warp: 16 consecutive output pixels of one row x all Cout.
//   mode 0: out = bf16(relu(acc + b))
//   mode 1: pre = bf16(acc + b) stored; out = bf16(relu(acc + b) + skip)
// `up`: the input is at half resolution (nearest upsampling folded in).
template <int CIN, int COUT>
__global__ void __launch_bounds__(128) k_conv_tc(int H, int W, int up, const __nv_bfloat16* __restrict__ in,
                                                 const __nv_bfloat16* __restrict__ wpk, const float* __restrict__ bias,
                                                 int mode, const __nv_bfloat16* __restrict__ skip,
                                                 __nv_bfloat16* __restrict__ pre, __nv_bfloat16* __restrict__ out)
{
    LSDTT_COUNT();
    constexpr int NT = COUT / 8;  // n tiles
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int tiles_per_row = (W + 15) / 16;
    const int y = warp / tiles_per_row;
    const int x0 = (warp % tiles_per_row) * 16;
    if (y >= H) return;
    const int g = lane >> 2, tig = lane & 3;
    const int Win = up ? (W >> 1) : W, Hin = up ? (H >> 1) : H;
    float acc[NT][4];
#pragma unroll
    for (int t = 0; t < NT; ++t)
        acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.f;
    const int xa = x0 + g, xb = x0 + g + 8;  // the two pixel rows of the A fragment
#pragma unroll 1
    for (int tap = 0; tap < 9; ++tap)
    {
        const int yy = y + tap / 3 - 1;
        const int xa2 = xa + tap % 3 - 1, xb2 = xb + tap % 3 - 1;
        const bool va = yy >= 0 && yy < H && xa2 >= 0 && xa2 < W && xa < W;
        const bool vb = yy >= 0 && yy < H && xb2 >= 0 && xb2 < W && xb < W;
        const int sy = up ? (yy >> 1) : yy;
        const std::int64_t ra = va ? (static_cast<std::int64_t>(sy) * Win + (up ? (xa2 >> 1) : xa2)) * CIN : 0;
        const std::int64_t rb = vb ? (static_cast<std::int64_t>(sy) * Win + (up ? (xb2 >> 1) : xb2)) * CIN : 0;
        (void)Hin;
#pragma unroll
        for (int kc = 0; kc < CIN / 16; ++kc)
        {
            const int c0 = kc * 16 + tig * 2;
            const unsigned a0 = va ? *reinterpret_cast<const unsigned*>(in + ra + c0) : 0u;
            const unsigned a1 = vb ? *reinterpret_cast<const unsigned*>(in + rb + c0) : 0u;
            const unsigned a2 = va ? *reinterpret_cast<const unsigned*>(in + ra + c0 + 8) : 0u;
            const unsigned a3 = vb ? *reinterpret_cast<const unsigned*>(in + rb + c0 + 8) : 0u;
#pragma unroll
            for (int nt = 0; nt < NT; ++nt)
            {
                const int co = nt * 8 + g;
                const __nv_bfloat16* wp = wpk + (static_cast<std::int64_t>(co) * 9 + tap) * CIN + c0;
                const unsigned b0 = *reinterpret_cast<const unsigned*>(wp);
                const unsigned b1 = *reinterpret_cast<const unsigned*>(wp + 8);
                asm volatile(
                    "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
                    "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};\n"
                    : "+f"(acc[nt][0]), "+f"(acc[nt][1]), "+f"(acc[nt][2]), "+f"(acc[nt][3])
                    : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
            }
        }
    }
    // Epilogue: c0,c1 -> pixel xa, channels nt*8 + tig*2 + {0,1}; c2,c3 -> pixel xb.
#pragma unroll
    for (int nt = 0; nt < NT; ++nt)
    {
        const int co = nt * 8 + tig * 2;
#pragma unroll
        for (int h = 0; h < 2; ++h)
        {
            const int xx = h ? xb : xa;
            if (xx >= W) continue;
            const std::int64_t o = (static_cast<std::int64_t>(y) * W + xx) * COUT + co;
#pragma unroll
            for (int q = 0; q < 2; ++q)
            {
                const float a = __fadd_rn(acc[nt][h * 2 + q], bias[co + q]);
                if (mode == 0)
                    out[o + q] = __float2bfloat16_rn(fmaxf(a, 0.f));
                else
                {
                    if (pre) pre[o + q] = __float2bfloat16_rn(a);  // kept for the backward pass only
                    out[o + q] = __float2bfloat16_rn(__fadd_rn(fmaxf(a, 0.f), __bfloat162float(skip[o + q])));
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// The same convolutions on the 5th-generation tensor cores (tcgen05).
//
// One CTA (8 warps) works through tiles of kTcM = 128 consecutive output
// pixels of one row; each tile is one UMMA of M = 128, N = COUT per K-step,
// K = 9 taps x CIN in steps of 16, BF16 operands from shared memory, FP32
// accumulator in tensor memory (TMEM), issued by one thread.
//
// Shared memory, canonical K-major layouts without swizzle (8-row x 16-byte
// core matrices):
//   halo: the 3 x 130 input pixels the tile reads (zero outside the image,
//         nearest upsampling folded in), stored per row as CIN/8 chunks of
//         130 contiguous 16-byte pixel rows. The A operand of tap (dy, dx)
//         is then a descriptor into it: start = row dy + dx pixels, the
//         8-row groups 128 B apart (SBO), the K chunks one chunk apart (LBO).
//   B:    the layer's weights for all 9 taps, per tap [COUT/8 groups][CIN/8
//         chunks][8 rows x 16 B], staged once per CTA.
// The epilogue reads the accumulator with tcgen05.ld (warp w owns TMEM lanes
// = tile pixels 32(w % 4)..+31; warps w and w + 4 split the columns) and
// fuses bias, ReLU, the decoder skip and the BF16 store. Every wait on the MMA barrier is bounded: on expiry the kernel
// records an error, waits once more (bounded) for its MMAs, frees its TMEM
// and returns.
constexpr int kTcM = 128;
constexpr int kHaloW = kTcM + 2;
constexpr int kChunkBytes = kHaloW * 16;
constexpr int kTcSpin = 1 << 22;

template <int CIN, int COUT>
struct Tc5Layout
{
    static constexpr int kChunks = CIN / 8;
    static constexpr int kRowBytes = kChunks * kChunkBytes;
    static constexpr int kHaloBytes = 3 * kRowBytes;      // one halo buffer (two are kept)
    static constexpr int kSboB = kChunks * 128;
    static constexpr int kTapBytes = (COUT / 8) * kSboB;
    static constexpr int kBBytes = 9 * kTapBytes;
    static constexpr int kBOff = 2 * kHaloBytes;
    static constexpr int kBarOff = kBOff + kBBytes;        // two mbarriers (16 B) then the TMEM address
    // At least 64 KB: the A descriptors span 16 groups x 2080 B if their two
    // byte offsets were read the other way round; keep any such read inside.
    static constexpr int kSmem = (kBarOff + 64) > 65536 ? (kBarOff + 64) : 65536;
    static constexpr int kAccCols = COUT < 32 ? 32 : COUT;
    static constexpr int kTmemCols = 2 * kAccCols;         // two accumulators
    static_assert(CIN % 16 == 0 && COUT % 16 == 0 && COUT <= 256, "UMMA shape");
    static_assert(kSmem <= 227 * 1024, "shared memory");
};

// Shared-memory matrix descriptor: start, leading (K) and stride (M/N) byte
// offsets in 16-byte units, descriptor version 1, no swizzle.
__device__ __forceinline__ std::uint64_t tc5_desc(std::uint32_t addr, std::uint32_t lbo, std::uint32_t sbo)
{
    return static_cast<std::uint64_t>((addr >> 4) & 0x3FFFu) |
           (static_cast<std::uint64_t>((lbo >> 4) & 0x3FFFu) << 16) |
           (static_cast<std::uint64_t>((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N = COUT, M = 128.
template <int N>
__device__ __forceinline__ constexpr std::uint32_t tc5_idesc()
{
    return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<std::uint32_t>(N >> 3) << 17) |
           (static_cast<std::uint32_t>(kTcM >> 4) << 24);
}

__device__ __forceinline__ bool tc5_wait(std::uint32_t mbar, std::uint32_t phase)
{
    for (int spin = 0; spin < kTcSpin; ++spin)
    {
        std::uint32_t ok;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(mbar), "r"(phase)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// Stage the 3 x 130-pixel input halo of tile (y, x0) with 16-byte cp.async
// copies (zero-filled outside the image; nearest upsampling folded in).
template <int CIN>
__device__ __forceinline__ void tc5_stage(std::uint32_t halo_s, const __nv_bfloat16* __restrict__ in, int H, int W,
                                          int Win, int up, int y, int x0)
{
    constexpr int kCh = CIN / 8;
    for (int q = threadIdx.x; q < 3 * kHaloW * kCh; q += blockDim.x)
    {
        const int kc = q % kCh;
        const int rest = q / kCh;
        const int j = rest % kHaloW, dy = rest / kHaloW;
        const int yy = y + dy - 1, xx = x0 - 1 + j;
        const bool inside = yy >= 0 && yy < H && xx >= 0 && xx < W;
        const int sy = inside ? (up ? (yy >> 1) : yy) : 0, sx = inside ? (up ? (xx >> 1) : xx) : 0;
        const __nv_bfloat16* src = in + (static_cast<std::int64_t>(sy) * Win + sx) * CIN + kc * 8;
        const std::uint32_t dst = halo_s + dy * (kCh * kChunkBytes) + kc * kChunkBytes + j * 16;
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(inside ? 16 : 0)
                     : "memory");
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}

// One kind::f16 UMMA (M = 128) into tmem_acc; `accum` 0 overwrites the
// accumulator, 1 adds to it.
__device__ __forceinline__ void umma_f16(std::uint32_t tmem_acc, std::uint64_t ad, std::uint64_t bd,
                                         std::uint32_t idesc, std::uint32_t accum)
{
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_acc),
        "l"(ad), "l"(bd), "r"(idesc), "r"(accum)
        : "memory");
}

// A shared-memory descriptor's start field is the byte address >> 4 in its
// low 14 bits, so a descriptor for an address `off` bytes further on is the
// same descriptor plus off >> 4 (shared addresses stay below 2^18, so the
// field never carries). The issuing thread adds constants instead of
// rebuilding 64-bit descriptors for each of up to 36 UMMAs a tile.
__device__ __forceinline__ std::uint64_t desc_plus(std::uint64_t d, std::uint32_t off)
{
    return d + static_cast<std::uint64_t>(off >> 4);
}

// Issue the 9 x CIN/16 UMMAs of one tile into accumulator column `acc`, then
// commit to the tile's barrier (one thread).
template <int CIN, int COUT>
__device__ __forceinline__ void tc5_issue(std::uint32_t tmem_acc, std::uint32_t halo_s, std::uint32_t b_s,
                                          std::uint32_t mbar_s)
{
    using Lt = Tc5Layout<CIN, COUT>;
    constexpr std::uint32_t idesc = tc5_idesc<COUT>();
    const std::uint64_t ad0 = tc5_desc(halo_s, kChunkBytes, 128);
    const std::uint64_t bd0 = tc5_desc(b_s, 128, Lt::kSboB);
#pragma unroll
    for (int t = 0; t < 9; ++t)
    {
        const int dy = t / 3, dx = t - dy * 3;
#pragma unroll
        for (int ks = 0; ks < CIN / 16; ++ks)
            umma_f16(tmem_acc, desc_plus(ad0, dy * Lt::kRowBytes + 2 * ks * kChunkBytes + dx * 16),
                     desc_plus(bd0, t * Lt::kTapBytes + 2 * ks * 128), idesc, (t | ks) ? 1u : 0u);
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar_s)
                 : "memory");
}

// Epilogue of one 128-pixel tile of output row y at x0 from the FP32
// accumulator at TMEM column tmem_acc: warp w reads TMEM lanes 32 (w % 4) ..
// (its tile pixels); warps w and w + 4 take alternate column chunks (8 wide
// for 16 output channels, so that both halves work, else 16). Bias, ReLU
// (mode 0) or ReLU plus the decoder skip (mode 1, pre-activation to `pre`
// when given), BF16 stores. `skip_row` points at the skip values of the
// tile's first pixel (COUT per pixel), in global or shared memory.
template <int COUT>
__device__ __forceinline__ void tc_epilogue(std::uint32_t tmem_acc, int y, int x0, int W, const float* __restrict__ bias,
                                            int mode, const __nv_bfloat16* skip_row,
                                            __nv_bfloat16* __restrict__ pre, __nv_bfloat16* __restrict__ out)
{
    constexpr int CW = COUT == 16 ? 8 : 16;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int quarter = warp & 3, half = warp >> 2;
    const int m = quarter * 32 + lane;
    const int x = x0 + m;
    const std::int64_t o = (static_cast<std::int64_t>(y) * W + x) * COUT;
    const std::uint32_t lane_col = tmem_acc + (static_cast<std::uint32_t>(quarter * 32) << 16);
#pragma unroll
    for (int n0 = CW * half; n0 < COUT; n0 += 2 * CW)
    {
        std::uint32_t r[CW];
        if constexpr (CW == 8)
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n"
                         : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                           "=r"(r[7])
                         : "r"(lane_col + static_cast<std::uint32_t>(n0)));
        else
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                "%14, %15}, [%16];\n"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15])
                : "r"(lane_col + static_cast<std::uint32_t>(n0)));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (x < W)
        {
            alignas(16) __nv_bfloat16 ov[CW];
            alignas(16) __nv_bfloat16 pv[CW];
            alignas(16) __nv_bfloat16 sv[CW];
            if (mode == 1)
            {
#pragma unroll
                for (int k = 0; k < CW; k += 8)
                    *reinterpret_cast<uint4*>(sv + k) =
                        *reinterpret_cast<const uint4*>(skip_row + m * COUT + n0 + k);
            }
#pragma unroll
            for (int j = 0; j < CW; ++j)
            {
                const float a = __fadd_rn(__uint_as_float(r[j]), bias[n0 + j]);
                if (mode == 0)
                    ov[j] = __float2bfloat16_rn(fmaxf(a, 0.f));
                else
                {
                    pv[j] = __float2bfloat16_rn(a);
                    ov[j] = __float2bfloat16_rn(__fadd_rn(fmaxf(a, 0.f), __bfloat162float(sv[j])));
                }
            }
#pragma unroll
            for (int k = 0; k < CW; k += 8)
                *reinterpret_cast<uint4*>(out + o + n0 + k) = *reinterpret_cast<const uint4*>(ov + k);
            if (mode == 1 && pre)
            {
#pragma unroll
                for (int k = 0; k < CW; k += 8)
                    *reinterpret_cast<uint4*>(pre + o + n0 + k) = *reinterpret_cast<const uint4*>(pv + k);
            }
        }
    }
}

// Pipelined over a CTA's tiles: while the tensor core works on tile i, the
// CTA stages tile i + 1 (second halo buffer) and then drains tile i's
// accumulator (second TMEM accumulator) through the epilogue.
template <int CIN, int COUT>
__global__ void __launch_bounds__(256) k_conv_tc5(int H, int W, int up, const __nv_bfloat16* __restrict__ in,
                                                  const __nv_bfloat16* __restrict__ wpk,
                                                  const float* __restrict__ bias, int mode,
                                                  const __nv_bfloat16* __restrict__ skip,
                                                  __nv_bfloat16* __restrict__ pre, __nv_bfloat16* __restrict__ out,
                                                  unsigned* __restrict__ err)
{
    LSDTT_COUNT();
    using Lt = Tc5Layout<CIN, COUT>;
    extern __shared__ __align__(1024) unsigned char tc5_smem[];
    const int tid = threadIdx.x, warp = tid >> 5;
    const std::uint32_t base_s = static_cast<std::uint32_t>(__cvta_generic_to_shared(tc5_smem));
    const std::uint32_t b_s = base_s + Lt::kBOff;
    const std::uint32_t mbar_s = base_s + Lt::kBarOff;  // [0], [8]: per accumulator
    const std::uint32_t tslot_s = mbar_s + 16;
    const std::uint32_t* tslot = reinterpret_cast<const std::uint32_t*>(tc5_smem + Lt::kBarOff + 16);
    unsigned char* bsm = tc5_smem + Lt::kBOff;

    for (int q = tid; q < 9 * COUT * Lt::kChunks; q += blockDim.x)
    {
        const int kc = q % Lt::kChunks;
        const int rest = q / Lt::kChunks;
        const int n = rest % COUT, t = rest / COUT;
        const uint4 v = *reinterpret_cast<const uint4*>(wpk + (static_cast<std::int64_t>(n) * 9 + t) * CIN + kc * 8);
        *reinterpret_cast<uint4*>(bsm + t * Lt::kTapBytes + (n >> 3) * Lt::kSboB + kc * 128 + (n & 7) * 16) = v;
    }
    if (warp == 0)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tslot_s),
                     "r"(Lt::kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0)
    {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar_s) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar_s + 8) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    const int Win = up ? (W >> 1) : W;
    const int tpr = (W + kTcM - 1) / kTcM;
    const int tiles = H * tpr;
    int tile = blockIdx.x;
    // prologue: stage the first tile
    if (tile < tiles) tc5_stage<CIN>(base_s, in, H, W, Win, up, tile / tpr, (tile % tpr) * kTcM);
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const std::uint32_t tmem = *tslot;
    if (tid == 0 && tile < tiles) tc5_issue<CIN, COUT>(tmem, base_s, b_s, mbar_s);

    std::uint32_t phase[2] = {0u, 0u};
    bool failed = false;
    for (int it = 0; tile < tiles && !failed; ++it, tile += gridDim.x)
    {
        const int cur = it & 1, nxt = cur ^ 1;
        const int ntile = tile + static_cast<int>(gridDim.x);
        // stage the next tile into the other halo buffer while the tensor
        // core works on this one (its MMAs read only halo[cur])
        if (ntile < tiles)
            tc5_stage<CIN>(base_s + nxt * Lt::kHaloBytes, in, H, W, Win, up, ntile / tpr, (ntile % tpr) * kTcM);
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        // this tile's MMAs
        const bool ok = tc5_wait(mbar_s + 8 * cur, phase[cur]);
        if (__syncthreads_or(ok ? 0 : 1))  // block-uniform: every thread leaves together
        {
            if (tid == 0) atomicOr(err, 1u);
            if (!ok) tc5_wait(mbar_s + 8 * cur, phase[cur]);  // once more for the MMAs in flight
            failed = true;
            break;
        }
        phase[cur] ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // next tile's MMAs into the other accumulator (the barrier above also
        // ordered every thread's staging of halo[nxt] before them)
        if (tid == 0 && ntile < tiles)
            tc5_issue<CIN, COUT>(tmem + nxt * Lt::kAccCols, base_s + nxt * Lt::kHaloBytes, b_s, mbar_s + 8 * nxt);
        // epilogue of this tile
        {
            const int ty = tile / tpr, tx0 = (tile % tpr) * kTcM;
            const __nv_bfloat16* skip_row = mode == 1 ? skip + (static_cast<std::int64_t>(ty) * W + tx0) * COUT : nullptr;
            tc_epilogue<COUT>(tmem + cur * Lt::kAccCols, ty, tx0, W, bias, mode, skip_row, pre, out);
        }
        // accumulator[cur] and halo[cur] are free once every warp is past here
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(Lt::kTmemCols)
                     : "memory");
}

// Rolling-row form of the tcgen05 convolution. Each persistent CTA walks
// down a vertical segment of one 128-pixel band of the image, so tile y+1
// needs one new input row (tile y's rows y-1..y+1 hold two of its three).
// Input rows live in a ring of D + 4 row slots (same per-row layout as
// k_conv_tc5: CIN/8 chunks of 130 contiguous 16-byte pixel rows); input rows
// are staged D + 1 rows ahead of the tile that first reads them, so copies,
// MMAs and the epilogue overlap. Decoder layers (kSkip) stage their skip rows
// into a second ring. Waits are bounded as in k_conv_tc5.
__host__ __device__ constexpr int tc6_smem_bytes(int cin, int cout, int d, bool skip)
{
    // B (9 taps of cout x cin BF16), input ring, skip ring, barriers
    return (9 * cout * cin * 2 + 127) / 128 * 128 + (d + 4) * (cin / 8) * kChunkBytes +
           (skip ? (d + 3) * kTcM * cout * 2 : 0) + 64;
}

template <int CIN, int COUT, int D, bool kSkip>
struct Tc6Layout
{
    static constexpr int kRing = D + 4;                  // input rows: tile y's three, the next D + 1
    static constexpr int kSkipRing = kSkip ? D + 3 : 1;  // skip rows: y .. y + D + 1, and one still being read
    static constexpr int kChunks = CIN / 8;
    static constexpr int kRowBytes = kChunks * kChunkBytes;
    static constexpr int kSboB = kChunks * 128;
    static constexpr int kTapBytes = (COUT / 8) * kSboB;
    static constexpr int kBBytes = 9 * kTapBytes;
    static constexpr int kRingOff = (kBBytes + 127) / 128 * 128;
    static constexpr int kSkipOff = kRingOff + kRing * kRowBytes;  // kSkipRing decoder-skip rows
    static constexpr int kSkipBytes = kTcM * COUT * 2;
    static constexpr int kBarOff = kSkipOff + (kSkip ? kSkipRing * kSkipBytes : 0);  // two mbarriers, TMEM address
    // at least 64 KB, as in Tc5Layout
    static constexpr int kSmem = (kBarOff + 64) > 65536 ? (kBarOff + 64) : 65536;
    static constexpr int kAccCols = COUT < 32 ? 32 : COUT;
    static constexpr int kTmemCols = 2 * kAccCols;
    static_assert(CIN % 16 == 0 && COUT % 16 == 0 && COUT <= 256, "UMMA shape");
    static_assert(kBarOff + 64 == tc6_smem_bytes(CIN, COUT, D, kSkip), "layout size");
    static_assert(kSmem <= 227 * 1024, "shared memory");
};

template <int R>
__device__ __forceinline__ int tc6_slot(int row) { return (row + 1) % R; }  // rows >= -1

// Stage input row `row` of the 130-pixel window at x0 - 1 into its slot of
// an R-slot ring (zero-filled outside the image; nearest upsampling folded
// in). The caller commits the cp.async group.
template <int CIN, int R>
__device__ __forceinline__ void tc6_stage_row(std::uint32_t ring_s, const __nv_bfloat16* __restrict__ in, int H,
                                              int W, int Win, int up, int row, int x0)
{
    constexpr int kCh = CIN / 8;
    const std::uint32_t slot_s = ring_s + tc6_slot<R>(row) * (kCh * kChunkBytes);
    const bool row_in = row >= 0 && row < H;
    const int sy = row_in ? (up ? (row >> 1) : row) : 0;
    for (int q = threadIdx.x; q < kHaloW * kCh; q += blockDim.x)
    {
        const int kc = q % kCh, j = q / kCh;
        const int xx = x0 - 1 + j;
        const bool inside = row_in && xx >= 0 && xx < W;
        const int sx = inside ? (up ? (xx >> 1) : xx) : 0;
        const __nv_bfloat16* src = in + (static_cast<std::int64_t>(sy) * Win + sx) * CIN + kc * 8;
        const std::uint32_t dst = slot_s + kc * kChunkBytes + j * 16;
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(inside ? 16 : 0)
                     : "memory");
    }
}

// Stage the decoder-skip values of output row `row` (128 pixels at x0,
// COUT channels each, zero past the image edge) into slot row % S of an
// S-slot ring. Issued ahead of the row's epilogue, which then reads the
// values from shared memory.
template <int COUT, int S>
__device__ __forceinline__ void tc6_stage_skip(std::uint32_t skip_s, const __nv_bfloat16* __restrict__ skip, int W,
                                               int row, int x0)
{
    constexpr int kCh = COUT / 8;
    const std::uint32_t slot_s = skip_s + (row % S) * (kTcM * COUT * 2);
    for (int q = threadIdx.x; q < kTcM * kCh; q += blockDim.x)
    {
        const int c = q % kCh, m = q / kCh;
        const int x = x0 + m;
        const bool inside = x < W;
        const __nv_bfloat16* src = skip + (static_cast<std::int64_t>(row) * W + (inside ? x : 0)) * COUT + c * 8;
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(slot_s + m * (COUT * 2) + c * 16),
                     "l"(src), "r"(inside ? 16 : 0)
                     : "memory");
    }
}

// The 9 x CIN/16 UMMAs of output row y (input rows y-1..y+1 in the ring)
// into accumulator column `tmem_acc`, committed to `mbar_s` (one thread).
template <int CIN, int COUT, int D, bool kSkip>
__device__ __forceinline__ void tc6_issue(std::uint32_t tmem_acc, std::uint32_t ring_s, std::uint32_t b_s, int y,
                                          std::uint32_t mbar_s)
{
    using Lt = Tc6Layout<CIN, COUT, D, kSkip>;
    constexpr std::uint32_t idesc = tc5_idesc<COUT>();
    const std::uint64_t bd0 = tc5_desc(b_s, 128, Lt::kSboB);
    std::uint64_t rowd[3];
#pragma unroll
    for (int dy = 0; dy < 3; ++dy)
        rowd[dy] = tc5_desc(ring_s + tc6_slot<Lt::kRing>(y + dy - 1) * Lt::kRowBytes, kChunkBytes, 128);
#pragma unroll
    for (int t = 0; t < 9; ++t)
    {
        const int dy = t / 3, dx = t - dy * 3;
#pragma unroll
        for (int ks = 0; ks < CIN / 16; ++ks)
            umma_f16(tmem_acc, desc_plus(rowd[dy], 2 * ks * kChunkBytes + dx * 16),
                     desc_plus(bd0, t * Lt::kTapBytes + 2 * ks * 128), idesc, (t | ks) ? 1u : 0u);
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar_s)
                 : "memory");
}

// Per output row y of a CTA's segment [y0, y1): stage the input row tile
// y+D+1 will need and the skip row of tile y+D+1, make sure tile y+1's rows
// have landed, issue tile y+1's MMAs into the other accumulator, wait for
// tile y's MMAs and drain them. Copies run D rows ahead (D + 1 cp.async
// groups in flight). An input slot is restaged only after the MMAs that read
// it completed (tile y's MMAs read rows y-1..y+1, and row y+D+2 goes to row
// y-2's slot); a skip slot only after every thread passed the barrier that
// follows its last epilogue.
template <int CIN, int COUT, int D, bool kSkip>
__global__ void __launch_bounds__(256) k_conv_tc6(int H, int W, int up, const __nv_bfloat16* __restrict__ in,
                                                  const __nv_bfloat16* __restrict__ wpk,
                                                  const float* __restrict__ bias, int mode,
                                                  const __nv_bfloat16* __restrict__ skip,
                                                  __nv_bfloat16* __restrict__ pre, __nv_bfloat16* __restrict__ out,
                                                  unsigned* __restrict__ err)
{
    LSDTT_COUNT();
    using Lt = Tc6Layout<CIN, COUT, D, kSkip>;
    constexpr int R = Lt::kRing, S = Lt::kSkipRing;
    extern __shared__ __align__(1024) unsigned char tc6_smem[];
    const int tid = threadIdx.x, warp = tid >> 5;
    const std::uint32_t base_s = static_cast<std::uint32_t>(__cvta_generic_to_shared(tc6_smem));
    const std::uint32_t b_s = base_s;
    const std::uint32_t ring_s = base_s + Lt::kRingOff;
    const std::uint32_t mbar_s = base_s + Lt::kBarOff;  // [0], [8]: per accumulator
    const std::uint32_t tslot_s = mbar_s + 16;
    const std::uint32_t* tslot = reinterpret_cast<const std::uint32_t*>(tc6_smem + Lt::kBarOff + 16);

    for (int q = tid; q < 9 * COUT * Lt::kChunks; q += blockDim.x)
    {
        const int kc = q % Lt::kChunks;
        const int rest = q / Lt::kChunks;
        const int n = rest % COUT, t = rest / COUT;
        const uint4 v = *reinterpret_cast<const uint4*>(wpk + (static_cast<std::int64_t>(n) * 9 + t) * CIN + kc * 8);
        *reinterpret_cast<uint4*>(tc6_smem + t * Lt::kTapBytes + (n >> 3) * Lt::kSboB + kc * 128 + (n & 7) * 16) = v;
    }
    if (warp == 0)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tslot_s),
                     "r"(Lt::kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0)
    {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar_s) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar_s + 8) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const std::uint32_t tmem = *tslot;
    const int Win = up ? (W >> 1) : W;
    const int nb = (W + kTcM - 1) / kTcM;                                   // 128-pixel bands
    const int segs = max(1, static_cast<int>(gridDim.x) / nb);  // row segments per band: one item per CTA
    const int rps = (H + segs - 1) / segs;
    const int items = nb * segs;
    const std::uint32_t skip_s = base_s + Lt::kSkipOff;
    const bool has_skip = kSkip && mode == 1;
    std::uint32_t phase[2] = {0u, 0u};
    bool failed = false;
    for (int item = blockIdx.x; item < items && !failed; item += gridDim.x)
    {
        const int x0 = (item % nb) * kTcM;
        const int y0 = (item / nb) * rps, y1 = min(H, y0 + rps);
        if (y0 >= y1) continue;  // block-uniform
        // every thread is past the last item's epilogue (skip slots) before
        // this item's staging
        __syncthreads();
        // prologue: group 0 = rows y0-1 .. y0+1 and skip row y0 (tile y0);
        // group k = 1..D: row y0+k+1 and skip row y0+k (tile y0+k)
        for (int r = y0 - 1; r <= y0 + 1; ++r) tc6_stage_row<CIN, R>(ring_s, in, H, W, Win, up, r, x0);
        if (has_skip) tc6_stage_skip<COUT, S>(skip_s, skip, W, y0, x0);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
#pragma unroll
        for (int k = 1; k <= D; ++k)
        {
            if (y0 + k < y1)
            {
                tc6_stage_row<CIN, R>(ring_s, in, H, W, Win, up, y0 + k + 1, x0);
                if (has_skip) tc6_stage_skip<COUT, S>(skip_s, skip, W, y0 + k, x0);
            }
            asm volatile("cp.async.commit_group;\n" ::: "memory");
        }
        asm volatile("cp.async.wait_group %0;\n" ::"n"(D) : "memory");  // group 0
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (tid == 0) tc6_issue<CIN, COUT, D, kSkip>(tmem, ring_s, b_s, y0, mbar_s);
        for (int y = y0; y < y1; ++y)
        {
            const int cur = (y - y0) & 1, nxt = cur ^ 1;
            // input row y+D+2 goes to the slot of row y-2 (tile y-1's MMAs
            // completed), skip row y+D+1 to the slot row y-2's epilogue read
            // (every thread passed the barrier below since)
            if (y + D + 1 < y1)
            {
                tc6_stage_row<CIN, R>(ring_s, in, H, W, Win, up, y + D + 2, x0);
                if (has_skip) tc6_stage_skip<COUT, S>(skip_s, skip, W, y + D + 1, x0);
            }
            asm volatile("cp.async.commit_group;\n" ::: "memory");
            // the group holding row y+2 (tile y+1) and skip row y+1, and all
            // before it, have landed
            asm volatile("cp.async.wait_group %0;\n" ::"n"(D) : "memory");
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            // every thread's copies, and the last epilogue's reads of the
            // other accumulator, are ordered before tile y+1's MMAs
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncthreads();
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const bool more = y + 1 < y1;
            if (tid == 0 && more)
                tc6_issue<CIN, COUT, D, kSkip>(tmem + nxt * Lt::kAccCols, ring_s, b_s, y + 1, mbar_s + 8 * nxt);
            const bool ok = tc5_wait(mbar_s + 8 * cur, phase[cur]);
            if (__syncthreads_or(ok ? 0 : 1))  // block-uniform: every thread leaves together
            {
                if (tid == 0) atomicOr(err, 1u);
                if (!ok) tc5_wait(mbar_s + 8 * cur, phase[cur]);  // once more for the MMAs in flight
                if (more) tc5_wait(mbar_s + 8 * nxt, phase[nxt]);
                failed = true;
                break;
            }
            phase[cur] ^= 1u;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            tc_epilogue<COUT>(tmem + cur * Lt::kAccCols, y, x0, W, bias, mode,
                              reinterpret_cast<const __nv_bfloat16*>(tc6_smem + Lt::kSkipOff +
                                                                     (y % S) * Lt::kSkipBytes),
                              pre, out);
        }
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(Lt::kTmemCols)
                     : "memory");
}

// ---------------------------------------------------------------------------
// Warp-specialised rolling-row convolution (same UMMAs and epilogue
// arithmetic as k_conv_tc6, so the same bits). Roles of the 288 threads:
//   warps 0-3  epilogue: thread m drains TMEM lane m (pixel m of the tile),
//              all COUT columns, adds bias / ReLU / skip and stores;
//   warps 4-7  producers: stage input rows (and decoder skip rows) with
//              cp.async, two groups in flight, and signal each row when it
//              has landed;
//   warp 8     MMA: lane 0 issues a tile's UMMAs once its three rows are
//              full and its accumulator is empty, then frees the oldest row.
// The roles meet only at mbarriers (full / empty rings for input rows, skip
// rows and the two accumulators), so copies, MMAs and epilogues of
// different rows overlap instead of running in lockstep behind block-wide
// barriers. Every wait is bounded: a role that gives up raises the shared
// abort flag and the error word, the others leave at their next wait, and
// the MMA thread waits (bounded) for its last UMMAs before TMEM is freed.
// ---------------------------------------------------------------------------
constexpr int kWsThreads = 288;

// Tiles the MMA warp issues together: their UMMA chains interleave into G
// accumulators. A tile's 9 x CIN/16 UMMAs accumulate into one TMEM column
// block one after another, and with N = 16..64 each UMMA is short, so a
// single chain runs at the accumulation latency, not the tensor pipe's rate;
// independent chains fill the gaps.
constexpr int kWsGroup = 1;  // measured: pairs of tiles ran no faster (the A reads from shared memory bound first)
constexpr int kWsLagDefault = 2;

// Shared bytes of the warp-specialised kernel with producer lag L: L + 2 + G
// input row slots, L + 2 skip row slots, 2G accumulators.
__host__ __device__ constexpr int ws_smem_bytes(int cin, int cout, bool skip, int lag, int g)
{
    return (9 * cout * cin * 2 + 127) / 128 * 128 + (lag + 2 + g) * (cin / 8) * kChunkBytes +
           (skip ? (lag + 2) * kTcM * cout * 2 : 0) + 8 * (2 * (lag + 2 + g) + 2 * (lag + 2) + 4 * g + 1) + 16 +
           4 * cout;
}

// Lag 2 where it fits one CTA's shared memory, else 1 (the ring needs
// L + 2 + G input slots and L + 2 >= G + L skip slots for the roles never to
// wait on one another in a cycle).
__host__ __device__ constexpr int ws_fit_lag(int cin, int cout, bool skip)
{
    return ws_smem_bytes(cin, cout, skip, kWsLagDefault, kWsGroup) <= 227 * 1024 ? kWsLagDefault : 1;
}

template <int CIN, int COUT, bool kSkip, int L = ws_fit_lag(CIN, COUT, kSkip), int G = kWsGroup>
struct WsLayout
{
    static constexpr int kWsLag = L;          // producer cp.async groups in flight
    static constexpr int kWsRing = L + 2 + G;  // input row slots
    static constexpr int kWsSkip = L + 2;      // skip row slots
    static constexpr int kG = G;
    static constexpr int kAccs = 2 * G;        // accumulators: G being drained, G being computed
    static constexpr int kChunks = CIN / 8;
    static constexpr int kRowBytes = kChunks * kChunkBytes;
    static constexpr int kSboB = kChunks * 128;
    static constexpr int kTapBytes = (COUT / 8) * kSboB;
    static constexpr int kBBytes = 9 * kTapBytes;
    static constexpr int kRingOff = (kBBytes + 127) / 128 * 128;
    static constexpr int kSkipOff = kRingOff + kWsRing * kRowBytes;
    static constexpr int kSkipBytes = kTcM * COUT * 2;
    static constexpr int kBarOff = kSkipOff + (kSkip ? kWsSkip * kSkipBytes : 0);
    // mbarriers: full_in[R], empty_in[R], full_skip[S], empty_skip[S],
    // acc_full[2G], acc_empty[2G], done
    static constexpr int kFullIn = 0, kEmptyIn = kWsRing, kFullSkip = 2 * kWsRing, kEmptySkip = kFullSkip + kWsSkip,
                         kAccFull = kEmptySkip + kWsSkip, kAccEmpty = kAccFull + kAccs, kDone = kAccEmpty + kAccs,
                         kBars = kDone + 1;
    static constexpr int kTmemOff = kBarOff + 8 * kBars;  // TMEM base address, then the abort flag
    static constexpr int kAbortOff = kTmemOff + 4;
    static constexpr int kBiasOff = kTmemOff + 16;  // the layer's COUT biases (FP32)
    static constexpr int kSmem = kBiasOff + 4 * COUT;
    static constexpr int kAccCols = COUT < 32 ? 32 : COUT;
    static constexpr int kTmemCols = kAccs * kAccCols;
    static_assert(CIN % 16 == 0 && COUT % 16 == 0 && COUT <= 256, "UMMA shape");
    static_assert(kTmemCols == 64 || kTmemCols == 128 || kTmemCols == 256 || kTmemCols == 512, "TMEM allocation");
    static_assert(kSmem == ws_smem_bytes(CIN, COUT, kSkip, L, G), "layout size");
    static_assert(kSmem <= 227 * 1024, "shared memory");
};

__device__ __forceinline__ void mbar_init(std::uint32_t bar, std::uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(std::uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tc_commit(std::uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

// Bounded wait for the phase of `bar` with the given parity: at most 2^20
// tries of at most ~1 us each (the suspend-time hint), so about a second in
// all; gives up early once another role raised the abort flag. On failure
// raises it.
constexpr int kWsSpin = 1 << 20;
__device__ __forceinline__ bool ws_wait(std::uint32_t bar, std::uint32_t parity, volatile int* abort_flag,
                                        int tries = kWsSpin)
{
    for (int spin = 0; spin < tries; ++spin)
    {
        std::uint32_t ok;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity), "r"(1000)
            : "memory");
        if (ok) return true;
        if ((spin & 63) == 63 && *abort_flag) return false;
    }
    *abort_flag = 1;
    return false;
}

// Failure-detection self-test of the bounded mbarrier wait: one thread
// initialises an mbarrier that expects one arrival and waits on its first
// phase, which nothing completes; ws_wait gives up after `tries` polls and
// raises the abort flag, and the kernel reports it.
__global__ void ws_wait_selftest(int* __restrict__ abort_flag, int* __restrict__ released, int tries)
{
    LSDTT_COUNT();
    __shared__ __align__(8) unsigned long long mbar;
    const std::uint32_t bar = static_cast<std::uint32_t>(__cvta_generic_to_shared(&mbar));
    if (threadIdx.x == 0)
    {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) *released = ws_wait(bar, 0u, abort_flag, tries) ? 1 : 0;
}

// Input row `row` of the 130-pixel window at x0 - 1 into the slot at slot_s
// (zero outside the image, nearest upsampling folded in), by `nt` threads.
template <int CIN>
__device__ __forceinline__ void ws_stage_row(std::uint32_t slot_s, const __nv_bfloat16* __restrict__ in, int H, int W,
                                             int Win, int up, int row, int x0, int t, int nt)
{
    constexpr int kCh = CIN / 8;
    const bool row_in = row >= 0 && row < H;
    const int sy = row_in ? (up ? (row >> 1) : row) : 0;
    for (int q = t; q < kHaloW * kCh; q += nt)
    {
        const int kc = q % kCh, j = q / kCh;
        const int xx = x0 - 1 + j;
        const bool inside = row_in && xx >= 0 && xx < W;
        const int sx = inside ? (up ? (xx >> 1) : xx) : 0;
        const __nv_bfloat16* src = in + (static_cast<std::int64_t>(sy) * Win + sx) * CIN + kc * 8;
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(slot_s + kc * kChunkBytes + j * 16),
                     "l"(src), "r"(inside ? 16 : 0)
                     : "memory");
    }
}

// Skip values of output row `row` (128 pixels at x0, zero past the edge)
// into the slot at slot_s, by `nt` threads.
template <int COUT>
__device__ __forceinline__ void ws_stage_skip(std::uint32_t slot_s, const __nv_bfloat16* __restrict__ skip, int W,
                                              int row, int x0, int t, int nt)
{
    constexpr int kCh = COUT / 8;
    for (int q = t; q < kTcM * kCh; q += nt)
    {
        const int c = q % kCh, m = q / kCh;
        const int x = x0 + m;
        const bool inside = x < W;
        const __nv_bfloat16* src = skip + (static_cast<std::int64_t>(row) * W + (inside ? x : 0)) * COUT + c * 8;
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(slot_s + m * (COUT * 2) + c * 16),
                     "l"(src), "r"(inside ? 16 : 0)
                     : "memory");
    }
}

// The UMMAs of g <= G consecutive tiles, interleaved: tile i reads input
// rows row_s[i .. i+2] and accumulates into column block acc[i]; each
// tile's 9 x CIN/16 UMMAs keep their order (one thread).
template <int CIN, int COUT, int G>
__device__ __forceinline__ void ws_issue_group(std::uint32_t tmem, const std::uint32_t (&acc)[G],
                                               const std::uint32_t (&row_s)[G + 2], int g, std::uint32_t b_s)
{
    using Lt = WsLayout<CIN, COUT, false>;
    constexpr std::uint32_t idesc = tc5_idesc<COUT>();
    const std::uint64_t bd0 = tc5_desc(b_s, 128, Lt::kSboB);
    std::uint64_t rowd[G + 2];
#pragma unroll
    for (int k = 0; k < G + 2; ++k) rowd[k] = tc5_desc(row_s[k], kChunkBytes, 128);
#pragma unroll
    for (int t = 0; t < 9; ++t)
    {
        const int dy = t / 3, dx = t - dy * 3;
#pragma unroll
        for (int ks = 0; ks < CIN / 16; ++ks)
        {
            const std::uint64_t bd = desc_plus(bd0, t * Lt::kTapBytes + 2 * ks * 128);
#pragma unroll
            for (int i = 0; i < G; ++i)
                if (i < g)
                    umma_f16(tmem + acc[i], desc_plus(rowd[i + dy], 2 * ks * kChunkBytes + dx * 16), bd, idesc,
                             (t | ks) ? 1u : 0u);
        }
    }
}

// Epilogue thread of pixel m = 32 warp + lane (warps 0-3): its TMEM lane 16
// columns at a time, the accumulator handed back to the MMA warp after the
// last load, the same arithmetic as tc_epilogue. skip_row: the tile's skip
// values in shared memory (mode 1).
template <int COUT>
__device__ __forceinline__ void ws_epilogue(std::uint32_t tmem_acc, int warp, int lane, int y, int x0, int W,
                                            const float* __restrict__ bias, int mode, const __nv_bfloat16* skip_row,
                                            __nv_bfloat16* __restrict__ pre, __nv_bfloat16* __restrict__ out,
                                            std::uint32_t acc_empty, float* __restrict__ yout,
                                            const float* __restrict__ rms)
{
    const int m = warp * 32 + lane;
    const int x = x0 + m;
    const std::uint32_t lane_col = tmem_acc + (static_cast<std::uint32_t>(warp * 32) << 16);
    const std::int64_t o = (static_cast<std::int64_t>(y) * W + x) * COUT;
#pragma unroll
    for (int n0 = 0; n0 < COUT; n0 += 16)
    {
        std::uint32_t r[16];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
            "%14, %15}, [%16];\n"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
            : "r"(lane_col + static_cast<std::uint32_t>(n0)));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (n0 + 16 == COUT)
        {
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            mbar_arrive(acc_empty);
        }
        if (x >= W) continue;
        if (mode == 2)
        {
            // output layer: one channel (column 0; the padded weight rows
            // are zero), plus bias, times the input's rms, FP32
            if (n0 == 0) yout[static_cast<std::int64_t>(y) * W + x] = __fmul_rn(__fadd_rn(__uint_as_float(r[0]), bias[0]), *rms);
            continue;
        }
        alignas(16) __nv_bfloat16 ov[16];
        alignas(16) __nv_bfloat16 pv[16];
        alignas(16) __nv_bfloat16 sv[16];
        if (mode == 1)
        {
            *reinterpret_cast<uint4*>(sv) = *reinterpret_cast<const uint4*>(skip_row + m * COUT + n0);
            *reinterpret_cast<uint4*>(sv + 8) = *reinterpret_cast<const uint4*>(skip_row + m * COUT + n0 + 8);
        }
#pragma unroll
        for (int j = 0; j < 16; ++j)
        {
            const float a = __fadd_rn(__uint_as_float(r[j]), bias[n0 + j]);
            if (mode == 0)
                ov[j] = __float2bfloat16_rn(fmaxf(a, 0.f));
            else
            {
                pv[j] = __float2bfloat16_rn(a);
                ov[j] = __float2bfloat16_rn(__fadd_rn(fmaxf(a, 0.f), __bfloat162float(sv[j])));
            }
        }
        *reinterpret_cast<uint4*>(out + o + n0) = *reinterpret_cast<const uint4*>(ov);
        *reinterpret_cast<uint4*>(out + o + n0 + 8) = *reinterpret_cast<const uint4*>(ov + 8);
        if (mode == 1 && pre)
        {
            *reinterpret_cast<uint4*>(pre + o + n0) = *reinterpret_cast<const uint4*>(pv);
            *reinterpret_cast<uint4*>(pre + o + n0 + 8) = *reinterpret_cast<const uint4*>(pv + 8);
        }
    }
}

// Items: 128-pixel bands x row segments, one per CTA where the grid allows
// (as k_conv_tc6). Within an item, row k is image row y0 - 1 + k (k = 0 ..
// n + 1 for n tiles) and tile j reads rows j .. j + 2; sequence numbers run
// on across items, so slot = seq % ring and the phase parity = (seq / ring)
// & 1. kSkip: decoder layer (mode 1), skip rows staged by the producers.
template <int CIN, int COUT, bool kSkip>
__global__ void __launch_bounds__(kWsThreads, CIN == 64 ? 1 : 3) k_conv_ws(int H, int W, int up, const __nv_bfloat16* __restrict__ in,
                                                        const __nv_bfloat16* __restrict__ wpk,
                                                        const float* __restrict__ bias, int mode,
                                                        const __nv_bfloat16* __restrict__ skip,
                                                        __nv_bfloat16* __restrict__ pre,
                                                        __nv_bfloat16* __restrict__ out, unsigned* __restrict__ err,
                                                        float* __restrict__ yout, const float* __restrict__ rms)
{
    LSDTT_COUNT();
    using Lt = WsLayout<CIN, COUT, kSkip>;
    constexpr int R = Lt::kWsRing, S = Lt::kWsSkip;
    extern __shared__ __align__(1024) unsigned char ws_smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const std::uint32_t base_s = static_cast<std::uint32_t>(__cvta_generic_to_shared(ws_smem));
    const std::uint32_t b_s = base_s, ring_s = base_s + Lt::kRingOff, skip_s = base_s + Lt::kSkipOff;
    const std::uint32_t bar_s = base_s + Lt::kBarOff;
    auto bar = [&](int k) { return bar_s + 8u * static_cast<std::uint32_t>(k); };
    volatile int* abort_flag = reinterpret_cast<volatile int*>(ws_smem + Lt::kAbortOff);

    for (int q = tid; q < 9 * COUT * Lt::kChunks; q += blockDim.x)
    {
        const int kc = q % Lt::kChunks;
        const int rest = q / Lt::kChunks;
        const int n = rest % COUT, t = rest / COUT;
        const uint4 v = *reinterpret_cast<const uint4*>(wpk + (static_cast<std::int64_t>(n) * 9 + t) * CIN + kc * 8);
        *reinterpret_cast<uint4*>(ws_smem + t * Lt::kTapBytes + (n >> 3) * Lt::kSboB + kc * 128 + (n & 7) * 16) = v;
    }
    // biases into shared memory: the epilogue reads them every row (the
    // output layer, mode 2, has one)
    float* bias_s = reinterpret_cast<float*>(ws_smem + Lt::kBiasOff);
    for (int k = tid; k < COUT; k += blockDim.x) bias_s[k] = (mode == 2 && k > 0) ? 0.0f : bias[k];
    // the weights, stored by the generic proxy, are read by the UMMAs
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (tid == 0)
    {
        for (int k = 0; k < R; ++k)
        {
            mbar_init(bar(Lt::kFullIn + k), 128);
            mbar_init(bar(Lt::kEmptyIn + k), 1);
        }
        if (kSkip)
            for (int k = 0; k < S; ++k)
            {
                mbar_init(bar(Lt::kFullSkip + k), 128);
                mbar_init(bar(Lt::kEmptySkip + k), 128);
            }
        for (int k = 0; k < Lt::kAccs; ++k)
        {
            mbar_init(bar(Lt::kAccFull + k), 1);
            mbar_init(bar(Lt::kAccEmpty + k), 128);
        }
        mbar_init(bar(Lt::kDone), 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 8)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(base_s + Lt::kTmemOff),
                     "r"(Lt::kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const std::uint32_t tmem = *reinterpret_cast<const std::uint32_t*>(ws_smem + Lt::kTmemOff);
    const int Win = up ? (W >> 1) : W;
    const int nb = (W + kTcM - 1) / kTcM;
    const int segs = max(1, static_cast<int>(gridDim.x) / nb);
    const int rps = (H + segs - 1) / segs;
    const int items = nb * segs;
    bool ok = true;

    if (warp >= 4 && warp < 8)
    {
        // producers: row k of an item, and with it (k >= 2) tile k-2's skip
        // row; step k - L is signalled once its group has landed
        constexpr int L = Lt::kWsLag;
        const int pt = tid - 128;
        std::uint32_t q = 0, u = 0;
        for (int item = blockIdx.x; item < items && ok; item += gridDim.x)
        {
            const int x0 = (item % nb) * kTcM;
            const int y0 = (item / nb) * rps, y1 = min(H, y0 + rps);
            if (y0 >= y1) continue;
            const int n_rows = y1 - y0 + 2;
            const std::uint32_t qb = q;
            auto signal = [&](int k) {
                mbar_arrive(bar(Lt::kFullIn + static_cast<int>((qb + k) % R)));
                if (kSkip && k >= 2) mbar_arrive(bar(Lt::kFullSkip + static_cast<int>((u + k - 2) % S)));
            };
            for (int k = 0; k < n_rows; ++k)
            {
                const std::uint32_t qk = qb + static_cast<std::uint32_t>(k);
                const int slot = static_cast<int>(qk % R);
                if (qk >= static_cast<std::uint32_t>(R))
                    ok = ws_wait(bar(Lt::kEmptyIn + slot), ((qk / R) - 1) & 1u, abort_flag);
                if (!ok) break;
                ws_stage_row<CIN>(ring_s + slot * Lt::kRowBytes, in, H, W, Win, up, y0 - 1 + k, x0, pt, 128);
                if (kSkip && k >= 2)
                {
                    const std::uint32_t uu = u + static_cast<std::uint32_t>(k - 2);
                    const int sk = static_cast<int>(uu % S);
                    if (uu >= static_cast<std::uint32_t>(S))
                        ok = ws_wait(bar(Lt::kEmptySkip + sk), ((uu / S) - 1) & 1u, abort_flag);
                    if (ok) ws_stage_skip<COUT>(skip_s + sk * Lt::kSkipBytes, skip, W, y0 + k - 2, x0, pt, 128);
                }
                asm volatile("cp.async.commit_group;\n" ::: "memory");
                if (!ok) break;
                asm volatile("cp.async.wait_group %0;\n" ::"n"(L) : "memory");
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                if (k >= L) signal(k - L);
            }
            asm volatile("cp.async.wait_group 0;\n" ::: "memory");
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            if (ok)
                for (int k = max(0, n_rows - L); k < n_rows; ++k) signal(k);
            q = qb + static_cast<std::uint32_t>(n_rows);
            u += static_cast<std::uint32_t>(y1 - y0);
        }
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    }
    else if (warp == 8)
    {
        if (lane == 0)
        {
            // MMA: tiles j .. j+g-1 (g <= G) once rows j .. j+g+1 are full
            // and their accumulators drained; then rows j .. j+g-1 (tile
            // j+i is the last reader of row j+i) are freed. Tile u uses
            // accumulator u % 2G.
            constexpr int G = Lt::kG, NA = Lt::kAccs;
            std::uint32_t q = 0, u = 0;
            for (int item = blockIdx.x; item < items && ok; item += gridDim.x)
            {
                const int y0 = (item / nb) * rps, y1 = min(H, y0 + rps);
                if (y0 >= y1) continue;
                const int n_tiles = y1 - y0;
                const std::uint32_t qb = q;
                std::uint32_t next_row = qb;  // first row not yet waited for
                for (int j = 0; j < n_tiles && ok; j += G)
                {
                    const int g = min(G, n_tiles - j);
                    for (; next_row <= qb + static_cast<std::uint32_t>(j + g + 1) && ok; ++next_row)
                        ok = ws_wait(bar(Lt::kFullIn + static_cast<int>(next_row % R)), (next_row / R) & 1u, abort_flag);
                    std::uint32_t acc[G];
                    std::uint32_t rows[G + 2];
#pragma unroll
                    for (int i = 0; i < G; ++i)
                    {
                        const std::uint32_t ui = u + static_cast<std::uint32_t>(i);
                        acc[i] = static_cast<std::uint32_t>((ui % NA) * Lt::kAccCols);
                        if (ok && i < g && ui >= static_cast<std::uint32_t>(NA))
                            ok = ws_wait(bar(Lt::kAccEmpty + static_cast<int>(ui % NA)), ((ui / NA) - 1) & 1u,
                                         abort_flag);
                    }
#pragma unroll
                    for (int k = 0; k < G + 2; ++k)
                        rows[k] = ring_s + ((qb + static_cast<std::uint32_t>(j + k)) % R) * Lt::kRowBytes;
                    if (!ok) break;
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    ws_issue_group<CIN, COUT, G>(tmem, acc, rows, g, b_s);
                    for (int i = 0; i < g; ++i)
                        tc_commit(bar(Lt::kAccFull + static_cast<int>((u + static_cast<std::uint32_t>(i)) % NA)));
                    for (int i = 0; i < g; ++i)
                        tc_commit(bar(Lt::kEmptyIn + static_cast<int>((qb + static_cast<std::uint32_t>(j + i)) % R)));
                    u += static_cast<std::uint32_t>(g);
                }
                if (!ok) break;
                tc_commit(bar(Lt::kEmptyIn + static_cast<int>((qb + n_tiles) % R)));
                tc_commit(bar(Lt::kEmptyIn + static_cast<int>((qb + n_tiles + 1) % R)));
                q = qb + static_cast<std::uint32_t>(n_tiles + 2);
            }
            // every UMMA issued has completed before TMEM is freed
            tc_commit(bar(Lt::kDone));
            if (!tc5_wait(bar(Lt::kDone), 0)) ok = false;
        }
    }
    else
    {
        // epilogue (warps 0-3)
        std::uint32_t u = 0;
        for (int item = blockIdx.x; item < items && ok; item += gridDim.x)
        {
            const int x0 = (item % nb) * kTcM;
            const int y0 = (item / nb) * rps, y1 = min(H, y0 + rps);
            if (y0 >= y1) continue;
            for (int y = y0; y < y1; ++y, ++u)
            {
                const int a = static_cast<int>(u % Lt::kAccs);
                ok = ws_wait(bar(Lt::kAccFull + a), (u / Lt::kAccs) & 1u, abort_flag);
                const int sk = static_cast<int>(u % S);
                if (ok && kSkip) ok = ws_wait(bar(Lt::kFullSkip + sk), (u / S) & 1u, abort_flag);
                if (!ok) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                ws_epilogue<COUT>(tmem + a * Lt::kAccCols, warp, lane, y, x0, W, bias_s, mode,
                                  reinterpret_cast<const __nv_bfloat16*>(ws_smem + Lt::kSkipOff + sk * Lt::kSkipBytes),
                                  pre, out, bar(Lt::kAccEmpty + a), yout, rms);
                if (kSkip) mbar_arrive(bar(Lt::kEmptySkip + sk));
            }
        }
    }
    if (!ok)
    {
        *abort_flag = 1;
        atomicOr(err, 1u);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 8)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(Lt::kTmemCols)
                     : "memory");
}

// Output layer: 16 -> 1 channel, times rms, FP32.
__global__ void k_conv_out(int H, int W, const __nv_bfloat16* __restrict__ d0, const float* __restrict__ wg,
                           const float* __restrict__ b, const float* __restrict__ rms, float* __restrict__ y)
{
    LSDTT_COUNT();
    __shared__ float w[9 * 16];
    for (int k = threadIdx.x; k < 9 * 16; k += blockDim.x) w[k] = wg[k];
    __syncthreads();
    const std::int64_t p = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= static_cast<std::int64_t>(H) * W) return;
    const int py = static_cast<int>(p / W), px = static_cast<int>(p % W);
    float s = b[0];
    for (int t = 0; t < 9; ++t)
    {
        const int yy = py + t / 3 - 1, xx = px + t % 3 - 1;
        if (yy < 0 || yy >= H || xx < 0 || xx >= W) continue;
        const __nv_bfloat16* src = d0 + (static_cast<std::int64_t>(yy) * W + xx) * 16;
        alignas(16) __nv_bfloat16 v16[16];
        *reinterpret_cast<uint4*>(v16) = *reinterpret_cast<const uint4*>(src);
        *reinterpret_cast<uint4*>(v16 + 8) = *reinterpret_cast<const uint4*>(src + 8);
#pragma unroll
        for (int c = 0; c < 16; ++c) s = __fadd_rn(s, __fmul_rn(__bfloat162float(v16[c]), w[t * 16 + c]));
    }
    y[p] = __fmul_rn(s, *rms);
}

// ---------------------------------------------------------------------------
// loss and backward (FP32, CUDA cores)
// ---------------------------------------------------------------------------
// Per-block partials of sum (y-e)^2 (part[b]) and sum e^2 (part[kRedBlocks + b]).
__global__ void k_loss_sums(const float* __restrict__ y, const float* __restrict__ e, std::int64_t n,
                            double* __restrict__ part)
{
    LSDTT_COUNT();
    std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    double num = 0, den = 0;
    for (; i < n; i += static_cast<std::int64_t>(gridDim.x) * blockDim.x)
    {
        const double d = static_cast<double>(y[i]) - e[i];
        num += d * d;
        den += static_cast<double>(e[i]) * e[i];
    }
    num = block_sum_ordered(num);
    den = block_sum_ordered(den);
    if (threadIdx.x == 0)
    {
        part[blockIdx.x] = num;
        part[kRedBlocks + blockIdx.x] = den;
    }
}

// go = 2 (y - e) / den * rms
__global__ void k_loss_grad(const float* __restrict__ y, const float* __restrict__ e, std::int64_t n,
                            const double* __restrict__ acc, const float* __restrict__ rms, float* __restrict__ go)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double den = acc[1] > 0 ? acc[1] : 1.0;
    go[i] = static_cast<float>(2.0 * (static_cast<double>(y[i]) - e[i]) / den * (*rms));
}

// Backward of a 3x3 conv w.r.t. its input: dX[q][ci] = sum_tap sum_co
// g[q - off(tap)][co] * w[co][tap][ci]. g is [H][W][Cout] FP32 at the conv's
// output resolution. With `up`, X was the nearest upsampling of a half-
// resolution field, and the result is summed over each 2x2 block (written
// at half resolution). With `pool_from` (encoder), dX is the gradient of the
// pooled input, which is distributed /4 onto the full-resolution skip
// gradient `acc_full` ([2H][2W][Cin], accumulated with +=) instead.
__global__ void k_conv_bwd_data(int H, int W, int Cin, int Cout, int up, const float* __restrict__ g,
                                const float* __restrict__ w, float* __restrict__ dx, int pool_to_full,
                                float* __restrict__ acc_full)
{
    LSDTT_COUNT();
    const int Ho = up ? H / 2 : H, Wo = up ? W / 2 : W;  // resolution of the result
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= static_cast<std::int64_t>(Ho) * Wo * Cin) return;
    const int ci = static_cast<int>(i % Cin);
    const std::int64_t q = i / Cin;
    const int qy = static_cast<int>(q / Wo), qx = static_cast<int>(q % Wo);
    float s = 0.f;
    const int reps = up ? 4 : 1;
    for (int sub = 0; sub < reps; ++sub)
    {
        const int fy = up ? 2 * qy + (sub >> 1) : qy, fx = up ? 2 * qx + (sub & 1) : qx;
        for (int t = 0; t < 9; ++t)
        {
            const int py = fy - (t / 3 - 1), px = fx - (t % 3 - 1);  // output pixel that reads (fy,fx) via tap t
            if (py < 0 || py >= H || px < 0 || px >= W) continue;
            const float* gp = g + (static_cast<std::int64_t>(py) * W + px) * Cout;
            const float* wp = w + static_cast<std::int64_t>(t) * Cin + ci;
            for (int co = 0; co < Cout; ++co) s += gp[co] * wp[static_cast<std::int64_t>(co) * 9 * Cin];
        }
    }
    if (pool_to_full)
    {
        const int W2 = 2 * Wo;
        const float v = s * 0.25f;
        for (int sub = 0; sub < 4; ++sub)
        {
            const std::int64_t f = (static_cast<std::int64_t>(2 * qy + (sub >> 1)) * W2 + 2 * qx + (sub & 1)) * Cin + ci;
            acc_full[f] += v;
        }
    }
    else
        dx[i] = s;
}

// Weight/bias gradients of a 3x3 conv: gw[co][tap][ci] = sum_p g[p][co] *
// X[p + off(tap)][ci], gb[co] = sum_p g[p][co]. Blocks (x, co * 9 + tap)
// reduce over the x-th grid-strided share of the pixels and write their
// partial sums to part[((co * 9 + tap) * (Cin + 1) + c) * gridDim.x + x]
// (c = Cin: the bias term, tap 4 only); k_conv_bwd_w_sum adds the
// gridDim.x partials of each entry in index order, so the gradient has the
// same bits on every run. X is bf16 ([H][W][Cin], or half resolution with
// `up`).
__global__ void k_conv_bwd_w(int H, int W, int Cin, int Cout, int up, const float* __restrict__ g,
                             const __nv_bfloat16* __restrict__ X, float* __restrict__ part)
{
    LSDTT_COUNT();
    extern __shared__ float red[];  // [Cin + 1][32]
    const int co = blockIdx.y / 9, t = blockIdx.y % 9;
    const int Win = up ? W / 2 : W;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    float acc_c[64 + 1];
    for (int c = 0; c <= Cin; ++c) acc_c[c] = 0.f;
    const std::int64_t npix = static_cast<std::int64_t>(H) * W;
    for (std::int64_t p = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; p < npix;
         p += static_cast<std::int64_t>(gridDim.x) * blockDim.x)
    {
        const float gv = g[p * Cout + co];
        if (gv == 0.f) continue;
        if (t == 4) acc_c[Cin] += gv;
        const int py = static_cast<int>(p / W) + t / 3 - 1, px = static_cast<int>(p % W) + t % 3 - 1;
        if (py < 0 || py >= H || px < 0 || px >= W) continue;
        const __nv_bfloat16* xp = X + (static_cast<std::int64_t>(up ? py >> 1 : py) * Win + (up ? px >> 1 : px)) * Cin;
        for (int c = 0; c < Cin; ++c) acc_c[c] += gv * __bfloat162float(xp[c]);
    }
    for (int c = 0; c <= Cin; ++c)
    {
        float v = acc_c[c];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[c * 32 + warp] = v;
    }
    __syncthreads();
    if (threadIdx.x <= Cin)
    {
        float v = 0.f;
        for (int k = 0; k < nw; ++k) v += red[threadIdx.x * 32 + k];
        part[(static_cast<std::int64_t>(blockIdx.y) * (Cin + 1) + threadIdx.x) * gridDim.x + blockIdx.x] = v;
    }
}

// gw / gb from the partials of k_conv_bwd_w (nx per entry), in index order.
__global__ void k_conv_bwd_w_sum(int Cin, int Cout, int nx, const float* __restrict__ part, float* __restrict__ gw,
                                 float* __restrict__ gb)
{
    LSDTT_COUNT();
    const std::int64_t j = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= static_cast<std::int64_t>(Cout) * 9 * (Cin + 1)) return;
    const int y = static_cast<int>(j / (Cin + 1)), c = static_cast<int>(j % (Cin + 1));
    const float* p = part + j * nx;
    float v = 0.f;
    for (int k = 0; k < nx; ++k) v += p[k];
    if (c < Cin) gw[static_cast<std::int64_t>(y) * Cin + c] = v;
    else if (y % 9 == 4) gb[y / 9] = v;
}

// Decoder split: ga = gd * (pre > 0); gskip += gd.
__global__ void k_relu_skip_bwd(std::int64_t n, const float* __restrict__ gd, const __nv_bfloat16* __restrict__ pre,
                                float* __restrict__ ga, float* __restrict__ gskip)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float v = gd[i];
    ga[i] = __bfloat162float(pre[i]) > 0.f ? v : 0.f;
    gskip[i] += v;
}

// Encoder: g = gsum * (act > 0) (act = relu output, bf16).
__global__ void k_relu_mask(std::int64_t n, const float* __restrict__ gsum, const __nv_bfloat16* __restrict__ act,
                            float* __restrict__ g)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    g[i] = __bfloat162float(act[i]) > 0.f ? gsum[i] : 0.f;
}

__global__ void k_adam(std::int64_t n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void k_sgd(std::int64_t n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                      float lr, float mom)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float mi = mom * m[i] + g[i];
    m[i] = mi;
    w[i] -= lr * mi;
}

// The output layer's weights (1 x 9 x 16, FP32 at w_out) as a 16 x 9 x 16
// BF16 block whose rows 1..15 are zero, for the UMMA form of that layer.
__global__ void k_pack_out(const float* __restrict__ w_out, __nv_bfloat16* __restrict__ wb_out)
{
    LSDTT_COUNT();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 16 * 144) wb_out[i] = __float2bfloat16_rn(i < 144 ? w_out[i] : 0.0f);
}

__global__ void k_pack(std::int64_t n, const float* __restrict__ w, __nv_bfloat16* __restrict__ wb)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) wb[i] = __float2bfloat16_rn(w[i]);
}

// Weights as used by the forward pass: bf16 round trip of the FP32 master.
__global__ void k_bf16_round(std::int64_t n, const float* __restrict__ w, float* __restrict__ wr)
{
    LSDTT_COUNT();
    const std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) wr[i] = bfr(w[i]);
}

}  // namespace
}  // namespace lsdtt_gb300

using namespace lsdtt_gb300;

struct lsdtt_gpu_unet
{
    int maxH = 0, maxW = 0;
    std::int64_t woff[kLayers + 1] = {};  // weight offsets into the parameter vector
    std::int64_t boff[kLayers + 1] = {};  // bias offsets
    std::int64_t nparam = 0;
    std::int64_t wb_out_off = 0;  // BF16 offset of the padded output-layer block in wb (64-element aligned:
                                  // the convolution kernels read weights with 16-byte loads)
    int conv_kind = 3;          // 0: mma.sync, 1: tcgen05 tiles, 2: tcgen05 rolling rows, 3: warp-specialised
                                // rolling rows (default)
    unsigned* d_err = nullptr;  // device error word of the tcgen05 kernels
    float* w = nullptr;   // FP32 master: weights then biases
    float* wr = nullptr;  // bf16-rounded copy as FP32 (CUDA-core layers, backward)
    __nv_bfloat16* wb = nullptr;
    float *g = nullptr, *m = nullptr, *v = nullptr;
    long step = 0;
    // activations (bf16, NHWC)
    __nv_bfloat16 *x0 = nullptr, *e0 = nullptr, *p0 = nullptr, *e1 = nullptr, *p1 = nullptr, *e2 = nullptr,
                  *p2 = nullptr, *e3 = nullptr, *a2 = nullptr, *d2 = nullptr, *a1 = nullptr, *d1 = nullptr,
                  *a0 = nullptr, *d0 = nullptr;
    float *y = nullptr, *go = nullptr, *rms = nullptr;
    double* acc = nullptr;
    double* part = nullptr;  // per-block partial sums of the fixed-order reductions [3][kRedBlocks]
    double* hacc = nullptr;
    // training-only buffers (decoder pre-activations a0..a2 above, FP32
    // backward scratch), allocated by the first gradient evaluation
    float *gA = nullptr, *gB = nullptr, *ge0 = nullptr, *ge1 = nullptr, *ge2 = nullptr, *ge3 = nullptr;
    float* gwpart = nullptr;  // weight-gradient partials [Cout * 9][Cin + 1][kWgradBlocks] of the widest layer
};

namespace
{

int unet_conv_kind(const lsdtt_gpu_unet* U) { return U->conv_kind; }
unsigned* unet_err(const lsdtt_gpu_unet* U) { return U->d_err; }

std::int64_t level_px(const lsdtt_gpu_unet* U, int l)
{
    return static_cast<std::int64_t>(U->maxH >> l) * (U->maxW >> l);
}

template <class T>
cudaError_t ualloc(T** p, std::size_t count)
{
    return cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * (count ? count : 1));
}

int check_shape(const lsdtt_gpu_unet* U, int H, int W)
{
    if (H <= 0 || W <= 0 || (H & 7) || (W & 7) || H > U->maxH || W > U->maxW ||
        static_cast<std::int64_t>(H) * W > static_cast<std::int64_t>(U->maxH) * U->maxW)
        return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_unet: image must be a multiple of 8 on each side and fit the "
                                      "handle's capacity (" + std::to_string(U->maxH) + " x " +
                                          std::to_string(U->maxW) + ")");
    return LSDTT_GPU_OK;
}

// CTAs of `func` (`threads` a CTA, `smem` dynamic bytes, carveout set to all
// shared memory) that one SM holds at once, from the device limits and the
// function's registers, capped by the TMEM columns every resident CTA keeps
// for its whole life. (Computed directly: the occupancy query was seen to
// answer one CTA for these kernels where three were resident.)
static int resident_ctas(const void* func, int smem, int tmem_cols, int threads = 256)
{
    int dev = 0, smem_sm = 0, reserved = 0, regs_sm = 0, threads_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&threads_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, func) != cudaSuccess) return 1;
    const int per_warp_regs = (fa.numRegs * 32 + 255) / 256 * 256;  // allocation unit: 256 registers a warp
    int n = std::min(threads_sm / threads, regs_sm / std::max(1, per_warp_regs * ((threads + 31) / 32)));
    n = std::min(n, smem_sm / std::max(1, smem + static_cast<int>(fa.sharedSizeBytes) + reserved));
    n = std::min(n, 512 / tmem_cols);
    return std::max(1, n);
}

// Persistent grid of the tcgen05 kernel: every SM, as many CTAs as fit.
template <int CI, int CO>
unsigned tc5_grid(int tiles)
{
    static int per_sm = -1, sms = 0;
    if (per_sm < 0)
    {
        cudaFuncSetAttribute(k_conv_tc5<CI, CO>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             Tc5Layout<CI, CO>::kSmem);
        // the whole unified L1/shared array as shared memory, so that several
        // CTAs (each holding its TMEM columns) share an SM
        cudaFuncSetAttribute(k_conv_tc5<CI, CO>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        per_sm = resident_ctas(reinterpret_cast<const void*>(k_conv_tc5<CI, CO>), Tc5Layout<CI, CO>::kSmem,
                               Tc5Layout<CI, CO>::kTmemCols);
    }
    return static_cast<unsigned>(std::max(1, std::min(tiles, sms * per_sm)));
}

// Persistent grid of the rolling-row tcgen05 kernel (same rule).
template <int CI, int CO, int D, bool SK>
unsigned tc6_grid(int H, int W)
{
    using Lt = Tc6Layout<CI, CO, D, SK>;
    static int per_sm = -1, sms = 0;
    if (per_sm < 0)
    {
        cudaFuncSetAttribute(k_conv_tc6<CI, CO, D, SK>, cudaFuncAttributeMaxDynamicSharedMemorySize, Lt::kSmem);
        cudaFuncSetAttribute(k_conv_tc6<CI, CO, D, SK>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        per_sm = resident_ctas(reinterpret_cast<const void*>(k_conv_tc6<CI, CO, D, SK>), Lt::kSmem, Lt::kTmemCols);
    }
    // at most one CTA per band row-segment of three or more rows
    const int nb = (W + kTcM - 1) / kTcM;
    const int most = std::max(1, nb * std::max(1, H / 3));
    return static_cast<unsigned>(std::max(1, std::min(most, sms * per_sm)));
}

// Grid of the warp-specialised kernel (same rule as tc6_grid).
template <int CI, int CO, bool SK>
unsigned ws_grid(int H, int W)
{
    using Lt = WsLayout<CI, CO, SK>;
    static int per_sm = -1, sms = 0;
    if (per_sm < 0)
    {
        cudaFuncSetAttribute(k_conv_ws<CI, CO, SK>, cudaFuncAttributeMaxDynamicSharedMemorySize, Lt::kSmem);
        cudaFuncSetAttribute(k_conv_ws<CI, CO, SK>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        per_sm = resident_ctas(reinterpret_cast<const void*>(k_conv_ws<CI, CO, SK>), Lt::kSmem, Lt::kTmemCols,
                               kWsThreads);
    }
    const int nb = (W + kTcM - 1) / kTcM;
    const int most = std::max(1, nb * std::max(1, H / 3));
    return static_cast<unsigned>(std::max(1, std::min(most, sms * per_sm)));
}

// mode 0 (encoder), 1 (decoder, skip rows staged) or 2 (the output layer:
// FP32 y = (column 0 + bias) x rms).
template <int CI, int CO>
void launch_ws(int H, int W, int up, const __nv_bfloat16* in, const __nv_bfloat16* wpk, const float* b, int mode,
               const __nv_bfloat16* skip, __nv_bfloat16* pre, __nv_bfloat16* out, unsigned* err, double bytes,
               cudaStream_t st, float* yout = nullptr, const float* rms = nullptr)
{
    if (mode == 1)
        LSDTT_TIMED("unet_conv_ws", bytes, st,
                    (k_conv_ws<CI, CO, true><<<ws_grid<CI, CO, true>(H, W), kWsThreads,
                                               WsLayout<CI, CO, true>::kSmem, st>>>(H, W, up, in, wpk, b, mode,
                                                                                    skip, pre, out, err, yout, rms)));
    else
        LSDTT_TIMED("unet_conv_ws", bytes, st,
                    (k_conv_ws<CI, CO, false><<<ws_grid<CI, CO, false>(H, W), kWsThreads,
                                                WsLayout<CI, CO, false>::kSmem, st>>>(H, W, up, in, wpk, b, mode,
                                                                                      skip, pre, out, err, yout,
                                                                                      rms)));
}

// Rolling-row launch with prefetch depth D: the skip ring only for decoder
// layers (mode 1). (At 4096^2, D = 1 with three CTAs an SM ran the network
// faster than the deepest prefetch that fits, which costs CTAs per SM.)
template <int CI, int CO, int D>
void launch_tc6(int H, int W, int up, const __nv_bfloat16* in, const __nv_bfloat16* wpk, const float* b, int mode,
                const __nv_bfloat16* skip, __nv_bfloat16* pre, __nv_bfloat16* out, unsigned* err, double bytes,
                cudaStream_t st)
{
    constexpr int DS = D, DN = D;
    if (mode == 1)
        LSDTT_TIMED("unet_conv_tc6", bytes, st,
                    (k_conv_tc6<CI, CO, DS, true><<<tc6_grid<CI, CO, DS, true>(H, W), 256,
                                                    Tc6Layout<CI, CO, DS, true>::kSmem, st>>>(
                        H, W, up, in, wpk, b, mode, skip, pre, out, err)));
    else
        LSDTT_TIMED("unet_conv_tc6", bytes, st,
                    (k_conv_tc6<CI, CO, DN, false><<<tc6_grid<CI, CO, DN, false>(H, W), 256,
                                                     Tc6Layout<CI, CO, DN, false>::kSmem, st>>>(
                        H, W, up, in, wpk, b, mode, skip, pre, out, err)));
}

static void launch_conv_kind(const lsdtt_gpu_unet* U, int l, int H, int W, int up, const __nv_bfloat16* in,
                             const __nv_bfloat16* wpk, const float* b, int mode, const __nv_bfloat16* skip,
                             __nv_bfloat16* pre, __nv_bfloat16* out, cudaStream_t st)
{
    const int warps = H * ((W + 15) / 16);
    const unsigned blocks = static_cast<unsigned>((warps + 3) / 4);
    const double bytes = 2.0 * static_cast<double>(H) * W * (layer_cin(l) / (up ? 4.0 : 1.0) + layer_cout(l));
    const int tiles = H * ((W + kTcM - 1) / kTcM);
#define LSDTT_CONV_CASE(CI, CO)                                                                                     \
    if (layer_cin(l) == CI && layer_cout(l) == CO)                                                                  \
    {                                                                                                               \
        if (unet_conv_kind(U) == 3)                                                                                 \
            launch_ws<CI, CO>(H, W, up, in, wpk, b, mode, skip, pre, out, unet_err(U), bytes, st);                 \
        else if (unet_conv_kind(U) == 2)                                                                            \
            launch_tc6<CI, CO, 1>(H, W, up, in, wpk, b, mode, skip, pre, out, unet_err(U), bytes, st);             \
        else if (unet_conv_kind(U) == 1)                                                                            \
            LSDTT_TIMED("unet_conv_tc5", bytes, st,                                                                 \
                        (k_conv_tc5<CI, CO><<<tc5_grid<CI, CO>(tiles), 256, Tc5Layout<CI, CO>::kSmem, st>>>(       \
                            H, W, up, in, wpk, b, mode, skip, pre, out, unet_err(U))));                            \
        else                                                                                                        \
            LSDTT_TIMED("unet_conv_tc", bytes, st,                                                                  \
                        (k_conv_tc<CI, CO><<<blocks, 128, 0, st>>>(H, W, up, in, wpk, b, mode, skip, pre, out)));   \
        return;                                                                                                     \
    }
    LSDTT_CONV_CASE(16, 32)
    LSDTT_CONV_CASE(32, 64)
    LSDTT_CONV_CASE(64, 64)
    LSDTT_CONV_CASE(64, 32)
    LSDTT_CONV_CASE(32, 16)
#undef LSDTT_CONV_CASE
}

// Tensor-core layer l, timed under its own name as well when profiling is
// on (algorithmic bytes: input read once, output written once).
void launch_conv_tc(const lsdtt_gpu_unet* U, int l, int H, int W, int up, const __nv_bfloat16* in,
                    const __nv_bfloat16* wpk, const float* b, int mode, const __nv_bfloat16* skip,
                    __nv_bfloat16* pre, __nv_bfloat16* out, cudaStream_t st)
{
    static const char* const kName[7] = {"", "unet_layer1", "unet_layer2", "unet_layer3",
                                         "unet_layer4", "unet_layer5", "unet_layer6"};
    const double bytes = 2.0 * static_cast<double>(H) * W * (layer_cin(l) / (up ? 4.0 : 1.0) + layer_cout(l));
    LSDTT_TIMED(kName[l], bytes, st, launch_conv_kind(U, l, H, W, up, in, wpk, b, mode, skip, pre, out, st));
}

// Forward pass on an H x W residual (device, FP32) -> U->y. Without
// `for_training` the decoder pre-activations (needed only by the backward
// pass) are not stored.
cudaError_t unet_forward(lsdtt_gpu_unet* U, const float* r, int H, int W, cudaStream_t st, bool for_training)
{
    const std::int64_t n = static_cast<std::int64_t>(H) * W;
    // Algorithmic bytes: r 4 in (twice), x0 2 out per pixel.
    LSDTT_TIMED("unet_prep", 10.0 * static_cast<double>(n), st, ({
                    k_sumsq<<<kRedBlocks, 256, 0, st>>>(r, n, U->part);
                    k_rms<<<1, 256, 0, st>>>(n, U->part, U->rms);
                    k_prep<<<grid_blocks(n, 256), 256, 0, st>>>(r, n, U->rms, U->x0);
                }));
    const float* wr = U->wr;
    // Algorithmic bytes: x0 2 in, e0 32 out per pixel.
    // Algorithmic bytes: x0 2 in, e0 32 out, p0 8 out per pixel.
    int h = H / 2, w = W / 2;
    LSDTT_TIMED("unet_conv_in", 42.0 * static_cast<double>(n), st,
                (k_conv_in_pool<<<grid_blocks(static_cast<std::int64_t>(h) * w, 128), 128, 0, st>>>(
                    H, W, U->x0, wr + U->woff[0], U->w + U->boff[0], U->e0, U->p0)));
    launch_conv_tc(U, 1, h, w, 0, U->p0, U->wb + U->woff[1], U->w + U->boff[1], 0, nullptr, nullptr, U->e1, st);
    h /= 2; w /= 2;
    LSDTT_TIMED("unet_pool", 80.0 * static_cast<double>(h) * w * 4, st,
                (k_pool<<<grid_blocks(static_cast<std::int64_t>(h) * w * 4, 256), 256, 0, st>>>(h, w, 32, U->e1,
                                                                                                  U->p1)));
    launch_conv_tc(U, 2, h, w, 0, U->p1, U->wb + U->woff[2], U->w + U->boff[2], 0, nullptr, nullptr, U->e2, st);
    h /= 2; w /= 2;
    LSDTT_TIMED("unet_pool", 160.0 * static_cast<double>(h) * w * 4, st,
                (k_pool<<<grid_blocks(static_cast<std::int64_t>(h) * w * 8, 256), 256, 0, st>>>(h, w, 64, U->e2,
                                                                                                  U->p2)));
    launch_conv_tc(U, 3, h, w, 0, U->p2, U->wb + U->woff[3], U->w + U->boff[3], 0, nullptr, nullptr, U->e3, st);
    launch_conv_tc(U, 4, H / 4, W / 4, 1, U->e3, U->wb + U->woff[4], U->w + U->boff[4], 1, U->e2,
                   for_training ? U->a2 : nullptr, U->d2, st);
    launch_conv_tc(U, 5, H / 2, W / 2, 1, U->d2, U->wb + U->woff[5], U->w + U->boff[5], 1, U->e1,
                   for_training ? U->a1 : nullptr, U->d1, st);
    launch_conv_tc(U, 6, H, W, 1, U->d1, U->wb + U->woff[6], U->w + U->boff[6], 1, U->e0,
                   for_training ? U->a0 : nullptr, U->d0, st);
    // Algorithmic bytes: d0 32 in, y 4 out per pixel. The tcgen05 kinds run
    // the 16 -> 1 layer as a 16 -> 16 UMMA convolution with zero weight
    // rows 1..15 (wb_out), reading column 0.
    if (unet_conv_kind(U) >= 1)
        LSDTT_TIMED("unet_conv_out", 36.0 * static_cast<double>(n), st,
                    (launch_ws<16, 16>(H, W, 0, U->d0, U->wb + U->wb_out_off, U->w + U->boff[7], 2, nullptr, nullptr,
                                       nullptr, unet_err(U), 36.0 * static_cast<double>(n), st, U->y, U->rms)));
    else
        LSDTT_TIMED("unet_conv_out", 36.0 * static_cast<double>(n), st,
                    (k_conv_out<<<grid_blocks(n, 128), 128, 0, st>>>(H, W, U->d0, wr + U->woff[7], U->w + U->boff[7],
                                                                      U->rms, U->y)));
    return cudaGetLastError();
}

// Backward pass: gradients of loss = sum (y-e)^2/sum e^2 into U->g.
cudaError_t unet_backward(lsdtt_gpu_unet* U, const float* e, int H, int W, cudaStream_t st)
{
    const std::int64_t n = static_cast<std::int64_t>(H) * W;
    // every weight and bias entry is assigned by k_conv_bwd_w_sum below
    k_loss_sums<<<kRedBlocks, 256, 0, st>>>(U->y, e, n, U->part + kRedBlocks);
    red_partials<<<2, 256, 0, st>>>(U->part + kRedBlocks, kRedBlocks, U->acc + 1);
    k_loss_grad<<<grid_blocks(n, 256), 256, 0, st>>>(U->y, e, n, U->acc + 1, U->rms, U->go);
    const float* wr = U->wr;
    auto bw = [&](int l, int h, int w, int up, const float* g, const __nv_bfloat16* X) {
        const int ci = layer_cin(l), co = layer_cout(l);
        const dim3 grid(kWgradBlocks, co * 9);
        k_conv_bwd_w<<<grid, 256, sizeof(float) * (ci + 1) * 32, st>>>(h, w, ci, co, up, g, X, U->gwpart);
        const std::int64_t entries = static_cast<std::int64_t>(co) * 9 * (ci + 1);
        k_conv_bwd_w_sum<<<grid_blocks(entries, 256), 256, 0, st>>>(ci, co, kWgradBlocks, U->gwpart,
                                                                     U->g + U->woff[l], U->g + U->boff[l]);
    };
    // out layer (16 -> 1): input d0 at H x W
    bw(7, H, W, 0, U->go, U->d0);
    k_conv_bwd_data<<<grid_blocks(n * 16, 256), 256, 0, st>>>(H, W, 16, 1, 0, U->go, wr + U->woff[7], U->gA, 0,
                                                              nullptr);
    // ge0 starts as the skip gradient from d0; dec0: d0 = relu(a0) + e0
    cudaMemsetAsync(U->ge0, 0, sizeof(float) * n * 16, st);
    k_relu_skip_bwd<<<grid_blocks(n * 16, 256), 256, 0, st>>>(n * 16, U->gA, U->a0, U->gB, U->ge0);
    bw(6, H, W, 1, U->gB, U->d1);  // input of dec0 is up(d1)
    const std::int64_t n1 = n / 4, n2 = n / 16, n3 = n / 64;
    k_conv_bwd_data<<<grid_blocks(n1 * 32, 256), 256, 0, st>>>(H, W, 32, 16, 1, U->gB, wr + U->woff[6], U->gA, 0,
                                                               nullptr);  // gd1 (half res) in gA
    cudaMemsetAsync(U->ge1, 0, sizeof(float) * n1 * 32, st);
    k_relu_skip_bwd<<<grid_blocks(n1 * 32, 256), 256, 0, st>>>(n1 * 32, U->gA, U->a1, U->gB, U->ge1);
    bw(5, H / 2, W / 2, 1, U->gB, U->d2);
    k_conv_bwd_data<<<grid_blocks(n2 * 64, 256), 256, 0, st>>>(H / 2, W / 2, 64, 32, 1, U->gB, wr + U->woff[5], U->gA,
                                                               0, nullptr);  // gd2
    cudaMemsetAsync(U->ge2, 0, sizeof(float) * n2 * 64, st);
    k_relu_skip_bwd<<<grid_blocks(n2 * 64, 256), 256, 0, st>>>(n2 * 64, U->gA, U->a2, U->gB, U->ge2);
    bw(4, H / 4, W / 4, 1, U->gB, U->e3);
    k_conv_bwd_data<<<grid_blocks(n3 * 64, 256), 256, 0, st>>>(H / 4, W / 4, 64, 64, 1, U->gB, wr + U->woff[4],
                                                               U->ge3, 0, nullptr);  // ge3 (1/8 res)
    // encoder 3: e3 = relu(conv(p2)); p2 = pool(e2)
    k_relu_mask<<<grid_blocks(n3 * 64, 256), 256, 0, st>>>(n3 * 64, U->ge3, U->e3, U->gB);
    bw(3, H / 8, W / 8, 0, U->gB, U->p2);
    k_conv_bwd_data<<<grid_blocks(n3 * 64, 256), 256, 0, st>>>(H / 8, W / 8, 64, 64, 0, U->gB, wr + U->woff[3],
                                                               nullptr, 1, U->ge2);
    k_relu_mask<<<grid_blocks(n2 * 64, 256), 256, 0, st>>>(n2 * 64, U->ge2, U->e2, U->gB);
    bw(2, H / 4, W / 4, 0, U->gB, U->p1);
    k_conv_bwd_data<<<grid_blocks(n2 * 32, 256), 256, 0, st>>>(H / 4, W / 4, 32, 64, 0, U->gB, wr + U->woff[2],
                                                               nullptr, 1, U->ge1);
    k_relu_mask<<<grid_blocks(n1 * 32, 256), 256, 0, st>>>(n1 * 32, U->ge1, U->e1, U->gB);
    bw(1, H / 2, W / 2, 0, U->gB, U->p0);
    k_conv_bwd_data<<<grid_blocks(n1 * 16, 256), 256, 0, st>>>(H / 2, W / 2, 16, 32, 0, U->gB, wr + U->woff[1],
                                                               nullptr, 1, U->ge0);
    k_relu_mask<<<grid_blocks(n * 16, 256), 256, 0, st>>>(n * 16, U->ge0, U->e0, U->gB);
    bw(0, H, W, 0, U->gB, U->x0);
    return cudaGetLastError();
}

}  // namespace

namespace lsdtt_gb300
{
int unet_check_shape(const lsdtt_gpu_unet* U, int H, int W) { return check_shape(U, H, W); }

cudaError_t unet_forward_dev(lsdtt_gpu_unet* U, const float* r_dev, int H, int W, cudaStream_t st,
                             const float** y_dev)
{
    *y_dev = U->y;
    return unet_forward(U, r_dev, H, W, st, false);
}
}  // namespace lsdtt_gb300

extern "C" {

int lsdtt_gpu_unet_create(int32_t max_rows, int32_t max_cols, uint64_t seed, lsdtt_gpu_unet** out)
{
    if (!out) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_unet_create: out is null");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(LSDTT_GPU_ENODEV, "lsdtt_gpu_unet_create: no CUDA device");
    if (max_rows <= 0 || max_cols <= 0 || (max_rows & 7) || (max_cols & 7))
        return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_unet_create: capacity must be positive multiples of 8");
    auto* U = new lsdtt_gpu_unet();
    U->maxH = max_rows;
    U->maxW = max_cols;
    std::int64_t off = 0;
    for (int l = 0; l < kLayers; ++l)
    {
        U->woff[l] = off;
        off += static_cast<std::int64_t>(layer_cout(l)) * 9 * layer_cin(l);
    }
    U->woff[kLayers] = off;
    for (int l = 0; l < kLayers; ++l)
    {
        U->boff[l] = off;
        off += layer_cout(l);
    }
    U->boff[kLayers] = off;
    U->nparam = off;
    // He initialisation from a splitmix-seeded Box-Muller stream, on the host.
    std::vector<float> h(static_cast<std::size_t>(off), 0.0f);
    std::uint64_t s = seed ? seed : 0x1234567ULL;
    auto next = [&]() {
        s += 0x9E3779B97F4A7C15ULL;
        std::uint64_t x = s;
        x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
        x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
        x ^= x >> 31;
        return (static_cast<double>(x >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    };
    for (int l = 0; l < kLayers; ++l)
    {
        const double std_dev = (l == kLayers - 1) ? 0.1 * std::sqrt(1.0 / (9.0 * layer_cin(l)))
                                                  : std::sqrt(2.0 / (9.0 * layer_cin(l)));
        for (std::int64_t i = U->woff[l]; i < U->woff[l + 1]; ++i)
        {
            const double u1 = next(), u2 = next();
            h[static_cast<std::size_t>(i)] =
                static_cast<float>(std_dev * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
        }
    }
    const std::int64_t px0 = level_px(U, 0);
    cudaError_t e = ualloc(&U->w, off);
    if (e == cudaSuccess) e = ualloc(&U->wr, off);
    U->wb_out_off = (off + 63) / 64 * 64;
    // the convolution kernels stage weights with 16-byte loads: every
    // layer's BF16 block must start on a 16-byte boundary
    for (int l = 1; l < kLayers; ++l)
        if ((U->woff[l] * 2) % 16 != 0)
        {
            lsdtt_gpu_unet_destroy(U);
            return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_unet_create: unaligned weight block");
        }
    if (e == cudaSuccess) e = ualloc(&U->wb, U->wb_out_off + 16 * 144);  // then the padded output-layer block
    if (e == cudaSuccess) e = ualloc(&U->g, off);
    if (e == cudaSuccess) e = ualloc(&U->m, off);
    if (e == cudaSuccess) e = ualloc(&U->v, off);
    if (e == cudaSuccess) e = ualloc(&U->x0, px0);
    if (e == cudaSuccess) e = ualloc(&U->e0, px0 * 16);
    if (e == cudaSuccess) e = ualloc(&U->d0, px0 * 16);
    if (e == cudaSuccess) e = ualloc(&U->p0, level_px(U, 1) * 16);
    if (e == cudaSuccess) e = ualloc(&U->e1, level_px(U, 1) * 32);
    if (e == cudaSuccess) e = ualloc(&U->d1, level_px(U, 1) * 32);
    if (e == cudaSuccess) e = ualloc(&U->p1, level_px(U, 2) * 32);
    if (e == cudaSuccess) e = ualloc(&U->e2, level_px(U, 2) * 64);
    if (e == cudaSuccess) e = ualloc(&U->d2, level_px(U, 2) * 64);
    if (e == cudaSuccess) e = ualloc(&U->p2, level_px(U, 3) * 64);
    if (e == cudaSuccess) e = ualloc(&U->e3, level_px(U, 3) * 64);
    if (e == cudaSuccess) e = ualloc(&U->y, px0);
    if (e == cudaSuccess) e = ualloc(&U->go, px0);
    if (e == cudaSuccess) e = ualloc(&U->rms, 1);
    if (e == cudaSuccess) e = ualloc(&U->acc, 4);
    if (e == cudaSuccess) e = ualloc(&U->part, 3 * kRedBlocks);
    if (e == cudaSuccess) e = ualloc(&U->d_err, 1);
    if (e == cudaSuccess) e = cudaMemset(U->d_err, 0, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&U->hacc), sizeof(double) * 4);
    if (e == cudaSuccess) e = cudaMemcpy(U->w, h.data(), sizeof(float) * off, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(U->m, 0, sizeof(float) * off);
    if (e == cudaSuccess) e = cudaMemset(U->v, 0, sizeof(float) * off);
    if (e != cudaSuccess)
    {
        lsdtt_gpu_unet_destroy(U);
        return cuda_fail(e, "lsdtt_gpu_unet_create");
    }
    k_pack<<<grid_blocks(off, 256), 256>>>(off, U->w, U->wb);
    k_pack_out<<<9, 256>>>(U->w + U->woff[7], U->wb + U->wb_out_off);
    k_bf16_round<<<grid_blocks(off, 256), 256>>>(off, U->w, U->wr);
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess)
    {
        lsdtt_gpu_unet_destroy(U);
        return cuda_fail(e, "lsdtt_gpu_unet_create");
    }
    *out = U;
    return LSDTT_GPU_OK;
}

int lsdtt_gpu_unet_destroy(lsdtt_gpu_unet* U)
{
    if (!U) return LSDTT_GPU_OK;
    void* ptrs[] = {U->w, U->wr, U->wb, U->g, U->m, U->v, U->x0, U->e0, U->a0, U->d0, U->p0, U->e1, U->a1, U->d1, U->p1,
                    U->e2, U->a2, U->d2, U->p2, U->e3, U->y, U->go, U->rms, U->acc, U->part, U->gA, U->gB, U->ge0,
                    U->ge1, U->ge2, U->ge3, U->gwpart, U->d_err};
    for (void* p : ptrs) cudaFree(p);
    cudaFreeHost(U->hacc);
    delete U;
    return LSDTT_GPU_OK;
}

int64_t lsdtt_gpu_unet_num_params(const lsdtt_gpu_unet* U) { return U ? U->nparam : 0; }

int lsdtt_gpu_unet_set_conv_kernel(lsdtt_gpu_unet* U, int32_t kind)
{
    if (!U || kind < 0 || kind > 3) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_unet_set_conv_kernel: bad argument");
    U->conv_kind = kind;
    return LSDTT_GPU_OK;
}

int lsdtt_gpu_unet_status(const lsdtt_gpu_unet* U)
{
    if (!U) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_unet_status: null");
    unsigned h = 0;
    if (cudaMemcpy(&h, U->d_err, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess)
        return fail(LSDTT_GPU_ECUDA, "lsdtt_gpu_unet_status: copy failed");
    if (h) return fail(LSDTT_GPU_ETIMEOUT, "lsdtt_gpu_unet: a tensor-core convolution hit its barrier wait limit");
    return LSDTT_GPU_OK;
}

int lsdtt_gpu_unet_get_params(const lsdtt_gpu_unet* U, float* host, int64_t count)
{
    if (!U || !host || count != U->nparam) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_unet_get_params: bad argument");
    return cudaMemcpy(host, U->w, sizeof(float) * count, cudaMemcpyDeviceToHost) == cudaSuccess
               ? LSDTT_GPU_OK
               : fail(LSDTT_GPU_ECUDA, "lsdtt_gpu_unet_get_params: copy failed");
}

int lsdtt_gpu_unet_set_params(lsdtt_gpu_unet* U, const float* host, int64_t count)
{
    if (!U || !host || count != U->nparam) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_unet_set_params: bad argument");
    if (cudaMemcpy(U->w, host, sizeof(float) * count, cudaMemcpyHostToDevice) != cudaSuccess)
        return fail(LSDTT_GPU_ECUDA, "lsdtt_gpu_unet_set_params: copy failed");
    k_pack<<<grid_blocks(count, 256), 256>>>(count, U->w, U->wb);
    k_pack_out<<<9, 256>>>(U->w + U->woff[7], U->wb + U->wb_out_off);
    k_bf16_round<<<grid_blocks(count, 256), 256>>>(count, U->w, U->wr);
    return cudaDeviceSynchronize() == cudaSuccess ? LSDTT_GPU_OK : fail(LSDTT_GPU_ECUDA, "lsdtt_gpu_unet_set_params");
}

// y = U(r) for an H x W residual (device, FP32), written to y_dev.
int lsdtt_gpu_unet_apply(lsdtt_gpu_unet* U, const float* r_dev, int32_t H, int32_t W, float* y_dev, void* stream)
{
    if (!U || !r_dev || !y_dev) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_unet_apply: null argument");
    if (int s = check_shape(U, H, W)) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = unet_forward(U, r_dev, H, W, st, false);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(y_dev, U->y, sizeof(float) * static_cast<std::size_t>(H) * W, cudaMemcpyDeviceToDevice, st);
    return e == cudaSuccess ? LSDTT_GPU_OK : cuda_fail(e, "lsdtt_gpu_unet_apply");
}

// Loss and parameter gradients (FP32, [nparam] into grad_host when given)
// without updating the weights; for gradient checks.
int lsdtt_gpu_unet_loss_grad(lsdtt_gpu_unet* U, const float* r_dev, const float* e_dev, int32_t H, int32_t W,
                             double* loss, float* grad_host, void* stream)
{
    if (!U || !r_dev || !e_dev) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_unet_loss_grad: null argument");
    if (int s = check_shape(U, H, W)) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaSuccess;
    if (!U->gA)
    {
        // Backward scratch (FP32, 4x the bf16 activations): only when training.
        const std::int64_t px0 = level_px(U, 0);
        // decoder pre-activations (ReLU masks of the backward pass)
        e = ualloc(&U->a0, px0 * 16);
        if (e == cudaSuccess) e = ualloc(&U->a1, level_px(U, 1) * 32);
        if (e == cudaSuccess) e = ualloc(&U->a2, level_px(U, 2) * 64);
        if (e == cudaSuccess) e = ualloc(&U->gA, px0 * 16);
        if (e == cudaSuccess) e = ualloc(&U->gB, px0 * 16);
        if (e == cudaSuccess) e = ualloc(&U->ge0, px0 * 16);
        if (e == cudaSuccess) e = ualloc(&U->ge1, level_px(U, 1) * 32);
        if (e == cudaSuccess) e = ualloc(&U->ge2, level_px(U, 2) * 64);
        if (e == cudaSuccess) e = ualloc(&U->ge3, level_px(U, 3) * 64);
        // widest weight-gradient reduction: Cout 64 x 9 taps x (Cin 64 + bias)
        if (e == cudaSuccess) e = ualloc(&U->gwpart, static_cast<std::size_t>(64) * 9 * 65 * kWgradBlocks);
        if (e != cudaSuccess)
        {
            void* bufs[] = {U->a0, U->a1, U->a2, U->gA, U->gB, U->ge0, U->ge1, U->ge2, U->ge3, U->gwpart};
            for (void* b : bufs) cudaFree(b);
            U->a0 = U->a1 = U->a2 = nullptr;
            U->gA = U->gB = U->ge0 = U->ge1 = U->ge2 = U->ge3 = nullptr;
            U->gwpart = nullptr;
            return cuda_fail(e, "lsdtt_gpu_unet_loss_grad");
        }
    }
    e = unet_forward(U, r_dev, H, W, st, true);
    if (e == cudaSuccess) e = unet_backward(U, e_dev, H, W, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(U->hacc, U->acc + 1, sizeof(double) * 2, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && grad_host)
        e = cudaMemcpyAsync(grad_host, U->g, sizeof(float) * U->nparam, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_unet_loss_grad");
    if (loss) *loss = U->hacc[0] / (U->hacc[1] > 0 ? U->hacc[1] : 1.0);
    return LSDTT_GPU_OK;
}

// One optimiser step on the pair (r, e); returns the loss before the step.
int lsdtt_gpu_unet_train_step(lsdtt_gpu_unet* U, const float* r_dev, const float* e_dev, int32_t H, int32_t W,
                              int32_t optimizer, float lr, double* loss, void* stream)
{
    if (optimizer != 0 && optimizer != 1)
        return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_unet_train_step: optimizer must be 0 (SGD) or 1 (Adam)");
    int s = lsdtt_gpu_unet_loss_grad(U, r_dev, e_dev, H, W, loss, nullptr, stream);
    if (s != LSDTT_GPU_OK) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    ++U->step;
    const unsigned nb = grid_blocks(U->nparam, 256);
    if (optimizer == 1)
    {
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.0f - std::pow(b1, static_cast<float>(U->step));
        const float c2 = 1.0f - std::pow(b2, static_cast<float>(U->step));
        k_adam<<<nb, 256, 0, st>>>(U->nparam, U->w, U->g, U->m, U->v, lr, b1, b2, 1e-8f, c1, c2);
    }
    else
        k_sgd<<<nb, 256, 0, st>>>(U->nparam, U->w, U->g, U->m, lr, 0.9f);
    k_pack<<<nb, 256, 0, st>>>(U->nparam, U->w, U->wb);
    k_pack_out<<<9, 256, 0, st>>>(U->w + U->woff[7], U->wb + U->wb_out_off);
    k_bf16_round<<<nb, 256, 0, st>>>(U->nparam, U->w, U->wr);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? LSDTT_GPU_OK : cuda_fail(e, "lsdtt_gpu_unet_train_step");
}

// lsdtt_gpu_selftest_mbarrier_wait (no reference counterpart): runs the
// tensor-core convolutions' bounded mbarrier wait against a phase that never
// completes. LSDTT_GPU_ETIMEOUT when the wait gave up as designed (the
// expected outcome), LSDTT_GPU_OK if it was released (a fault of the wait),
// another status on a CUDA error. The context stays usable.
int lsdtt_gpu_selftest_mbarrier_wait(int32_t tries)
{
    if (tries <= 0) return fail(LSDTT_GPU_EINVAL, "lsdtt_gpu_selftest_mbarrier_wait: tries must be positive");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(LSDTT_GPU_ENODEV, "lsdtt_gpu_selftest_mbarrier_wait: no CUDA device");
    int* buf = nullptr;  // abort flag, released
    cudaError_t e = cudaMalloc(&buf, 2 * sizeof(int));
    if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_selftest_mbarrier_wait");
    int host[2] = {0, -1};
    e = cudaMemset(buf, 0, 2 * sizeof(int));
    if (e == cudaSuccess)
    {
        ws_wait_selftest<<<1, 32>>>(buf, buf + 1, tries);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(host, buf, sizeof(host), cudaMemcpyDeviceToHost);
    cudaFree(buf);
    if (e != cudaSuccess) return cuda_fail(e, "lsdtt_gpu_selftest_mbarrier_wait");
    if (host[1] == 0 && host[0] == 1)
        return fail(LSDTT_GPU_ETIMEOUT, "lsdtt_gpu_selftest_mbarrier_wait: the bounded mbarrier wait gave up after " +
                                            std::to_string(tries) + " polls and raised the abort flag");
    return LSDTT_GPU_OK;
}

}  // extern "C"

namespace lsdtt_gb300
{
LSDTT_DEFINE_LAUNCH_READER(unet)
}  // namespace lsdtt_gb300
