// sp_node.cuh -- the per-node implicit stream-power update, shared by the
// single-grid sweep (stream_power.cu) and the packed ensemble (ensemble.cu).
#pragma once

#include <cmath>

#include "common.cuh"

namespace lsdtt_gb300
{
namespace
{

struct SpParams
{
    float K, m, n, dt, threshold, slope_clamp, dx, dx_diag;
    int divide_by_dx;
    int n_is_one;
};

// slope^e for the Newton iteration. The stream-power exponents the
// configurations use (n = 1, 1.5, 2, hence e in {0.5, 1, 1.5, 2}) take
// exact identities with one or two correct roundings (x*x, x, sqrt(x),
// x*sqrt(x)), which are at least as accurate as the general double pow
// and avoid its FP64 cost inside the level-ordered sweep; any other
// exponent takes pow.
__device__ __forceinline__ double sp_pow(double x, double e)
{
    if (e == 2.0) return __dmul_rn(x, x);
    if (e == 1.0) return x;
    if (e == 0.5) return __dsqrt_rn(x);
    if (e == 1.5) return __dmul_rn(x, __dsqrt_rn(x));
    return pow(x, e);
}

// K * A^m of one node in the reference's double arithmetic
// (stream_power_cpu.cpp:236-262), or -1 when the node is below the
// incision threshold (not eroded). area_d is the accumulate() total.
__device__ __forceinline__ double sp_kam(const SpParams& P, double area_d, float Ki)
{
    double area = area_d;
    if (P.divide_by_dx) area = __ddiv_rn(area, static_cast<double>(P.dx));
    if (P.threshold > 0.0f && area < static_cast<double>(P.threshold)) return -1.0;
    return __dmul_rn(static_cast<double>(Ki), pow(area, static_cast<double>(P.m)));
}

// The implicit update of one node (stream_power_cpu.cpp:263-318): its new
// elevation from its own old elevation zo, its receiver's final elevation
// zr, kam = sp_kam(...) and the step length to the receiver. Returns zo when
// the node is not eroded.
// tol_dx: the length the elevation tolerance slope_clamp * tol_dx is taken
// over (the step length to the receiver for D8; the cardinal cell size for
// D-infinity, stream_power_cpu.cpp:437).
__device__ __forceinline__ float sp_solve_tol(const SpParams& P, bool diagonal, double kam, float zo, float zr,
                                              float tol_dx)
{
    if (zr >= zo) return zo;
    const float dx_eff = diagonal ? P.dx_diag : P.dx;
    const double tol = __dmul_rn(static_cast<double>(P.slope_clamp), static_cast<double>(tol_dx));
    float zn = zo;
    if (P.n_is_one)
    {
        const double spf = __dmul_rn(kam, static_cast<double>(__fdiv_rn(P.dt, dx_eff)));
        const double num = __dadd_rn(static_cast<double>(zo), __dmul_rn(static_cast<double>(zr), spf));
        zn = static_cast<float>(__ddiv_rn(num, __dadd_rn(1.0, spf)));
        if (__fsub_rn(zn, zo) > static_cast<float>(tol) || isnan(zn)) zn = zo;
    }
    else
    {
        double eps = tol + 1.0;
        int it = 0;
        const double nd = static_cast<double>(P.n);
        const double kdt = __dmul_rn(kam, static_cast<double>(P.dt));
        const double ndx = static_cast<double>(__fdiv_rn(P.n, dx_eff));
        do
        {
            const double slope = static_cast<double>(__fdiv_rn(__fsub_rn(zn, zr), dx_eff));
            if (slope <= 0.0) eps = 0.0;
            else
            {
                const double fz = __dadd_rn(static_cast<double>(__fsub_rn(zn, zo)), __dmul_rn(kdt, sp_pow(slope, nd)));
                const double fdz =
                    __dadd_rn(1.0, __dmul_rn(__dmul_rn(kdt, ndx), sp_pow(slope, __dsub_rn(nd, 1.0))));
                eps = __ddiv_rn(fz, fdz);
            }
            zn = __fsub_rn(zn, static_cast<float>(eps));
            ++it;
            if (it > 100) eps = tol / 2.0;
        } while (fabs(eps) > tol);
        if (__fsub_rn(zn, zo) > static_cast<float>(tol) || isnan(zn)) zn = zo;
        if (zn < zr) zn = __fadd_rn(zr, __fmul_rn(P.slope_clamp, dx_eff));
    }
    return zn;
}

__device__ __forceinline__ float sp_solve(const SpParams& P, bool diagonal, double kam, float zo, float zr)
{
    return sp_solve_tol(P, diagonal, kam, zo, zr, diagonal ? P.dx_diag : P.dx);
}

// sp_solve for node `flat` with its own loads and store. Any receiver-
// before-donor order gives the reference's bits: a node reads only
// z_old[self] and z[receiver]. Indices are those of the arrays passed
// (n = their length). kCoherent reads the receiver's elevation from L2
// (bypassing L1), for sweeps whose levels are written by other SMs of the
// same launch.
template <bool kCoherent = false>
__device__ __forceinline__ void sp_node_kam(const SpParams& P, std::int64_t n, std::int64_t flat,
                                            const std::int64_t* __restrict__ receiver,
                                            const std::uint8_t* __restrict__ dir, double kam,
                                            const float* __restrict__ z_old, float* __restrict__ z)
{
    const std::int64_t recv = receiver[flat];
    if (recv < 0 || recv >= n || kam < 0.0) return;  // outlets, nodata, below threshold
    const float zo = z_old[flat];
    const float zr = kCoherent ? __ldcg(z + recv) : z[recv];
    const float zn = sp_solve(P, (dir[flat] & 1u) != 0, kam, zo, zr);
    z[flat] = zn;  // zo when not eroded: z[flat] already holds it
}

// Both parts for one node.
__device__ __forceinline__ void sp_node(const SpParams& P, std::int64_t n, std::int64_t flat,
                                        const std::int64_t* __restrict__ receiver, const std::uint8_t* __restrict__ dir,
                                        const double* __restrict__ area_d, const float* __restrict__ z_old,
                                        const float* __restrict__ kfield, float* __restrict__ z)
{
    const std::int64_t recv = receiver[flat];
    if (recv < 0 || recv >= n) return;
    const float Ki = kfield ? kfield[flat] : P.K;
    sp_node_kam(P, n, flat, receiver, dir, sp_kam(P, area_d[flat], Ki), z_old, z);
}

}  // namespace
}  // namespace lsdtt_gb300
