// xrdt_device.cuh -- device helpers shared by the kernels.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "xrdt_internal.h"

namespace xrdt {

// IEEE double operations the compiler may not fuse into FMA.  The integer
// decisions of the line integral (which ROI edge a ray enters, how many
// samples it takes) must round exactly as the FP64 oracle does: for
// axis-aligned rays Lr/DQ is an exact integer, and a fused multiply-add in
// the entry point moves Lr by an ulp and drops the last sample.
__host__ __device__ __forceinline__ double dmul(double a, double b)
{
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
__host__ __device__ __forceinline__ double dadd(double a, double b)
{
#ifdef __CUDA_ARCH__
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
__host__ __device__ __forceinline__ double dsub(double a, double b)
{
#ifdef __CUDA_ARCH__
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}

// Detector pixel position (integrate_diffraction.cu:104-109), rounded as the
// oracle rounds it.
__host__ __device__ inline void det_position(const DevProblem &P, double sphi, double cphi, int det,
                                             double *x, double *y, double *z)
{
    const int col = det % P.n_col, row = det / P.n_col;
    const double rdet = dmul(dadd(dsub((double)col, (double)P.n_col / 2.0), 0.5), P.col_pitch);
    *x = dadd(dsub(P.cx, dmul(P.r_det, sphi)), dmul(rdet, cphi));
    *y = dadd(dadd(P.cy, dmul(P.r_det, cphi)), dmul(rdet, sphi));
    *z = dadd(P.z0, dmul((double)row, P.row_pitch));
}

// __float2int_rd semantics on a double: NaN -> 0, saturating.
__host__ __device__ inline int floor_to_int(double x)
{
    if (x != x) return 0;
    double f = floor(x);
    if (f >= 2147483647.0) return 2147483647;
    if (f <= -2147483648.0) return (-2147483647 - 1);
    return (int)f;
}

// Source-energy window of detector bin nrg: find_src_nrg_range.cu:8-25, with
// the centre bin generalised to separate source and detector grids (the
// centre is nrg itself when the grids coincide).
__host__ __device__ inline void src_nrg_range(const DevProblem &P, int same_grid, int nrg,
                                              int *lo, int *hi)
{
    int c;
    if (same_grid) {
        c = nrg;
    } else {
        double ec = P.e_det_min + ((double)nrg + 0.5) * P.dEd;
        c = floor_to_int((ec - P.e_src_min) / P.dEs);
    }
    int mn = c - P.dnrg;
    if (mn < 0) mn = 0;
    int mx = mn + 2 * P.dnrg;
    if (mx >= P.nrg_src) {
        mx = P.nrg_src - 1;
        mn = mx - 2 * P.dnrg;
    }
    *lo = mn;
    *hi = mx;
}

// GetIntersection.cu:9-57 in double: first ROI edge crossed by the segment.
__host__ __device__ inline bool get_intersection(double x1, double y1, double x2, double y2,
                                                 int nx, int ny, double *rx, double *ry, int *edge = nullptr)
{
    const double NX = (double)nx, NY = (double)ny;
    const double eps = (double)0.00001f;
    const double x2_x1 = x2 - x1, y2_y1 = y2 - y1;
    for (int i = 0; i < 4; i++) {
        const double x3 = (i == 1 || i == 2) ? NX : 0.0;
        const double x4 = (i == 0 || i == 1) ? NX : 0.0;
        const double y3 = (i >= 2) ? NY : 0.0;
        const double y4 = (i == 1 || i == 2) ? NY : 0.0;
        const double x4_x3 = x4 - x3, y3_y1 = y3 - y1, y4_y3 = y4 - y3, x3_x1 = x3 - x1;
        const double den = dsub(dmul(x4_x3, y2_y1), dmul(x2_x1, y4_y3));
        if (den > eps || den < -eps) {
            const double u_a = dsub(dmul(x4_x3, y3_y1), dmul(x3_x1, y4_y3)) / den;
            if (u_a > -eps && u_a < 1.0 + eps) {
                const double u_b = dsub(dmul(x2_x1, y3_y1), dmul(x3_x1, y2_y1)) / den;
                if (u_b > -eps && u_b < 1.0 + eps) {
                    *rx = dadd(x1, dmul(x2_x1, u_a));
                    *ry = dadd(y1, dmul(y2_y1, u_a));
                    if (edge) *edge = i;
                    return true;
                }
            }
        }
    }
    *rx = NAN;
    *ry = NAN;
    if (edge) *edge = -1;
    return false;
}

// tex2D of Forward_XRD.cu:229-233 evaluated exactly in double from the
// float maps: texel (i,j) centred at (i+0.5, j+0.5), zero outside.
__device__ inline void bilinear_f64(const float *__restrict__ a1, const float *__restrict__ a2,
                                    int nx, int ny, double x, double y, double *v1, double *v2)
{
    const double xb = x - 0.5, yb = y - 0.5;
    const double fi = floor(xb), fj = floor(yb);
    const double fx = xb - fi, fy = yb - fj;
    const int i0 = (int)fi, j0 = (int)fj;
    double s1 = 0.0, s2 = 0.0;
#pragma unroll
    for (int dj = 0; dj < 2; dj++) {
        const int j = j0 + dj;
        if (j < 0 || j >= ny) continue;
        const double wy = dj ? fy : 1.0 - fy;
#pragma unroll
        for (int di = 0; di < 2; di++) {
            const int i = i0 + di;
            if (i < 0 || i >= nx) continue;
            const double w = wy * (di ? fx : 1.0 - fx);
            const int64_t idx = (int64_t)i + (int64_t)j * nx;
            s1 += w * (double)__ldg(a1 + idx);
            s2 += w * (double)__ldg(a2 + idx);
        }
    }
    *v1 = s1;
    *v2 = s2;
}

// floor(x) without a conversion instruction.  On this GPU the int<->float
// conversions and float rounding instructions share the FP64 pipe, which runs
// at 1/64 of the FP32 rate, so the hot loops avoid them: adding 1.5*2^23
// rounds x to the nearest integer inside the float's mantissa, from which the
// integer is read by reinterpreting the bits.  Valid for |x| < 2^22; the
// argument is clamped to that range (NaN becomes -2^22).
__device__ __forceinline__ int floor_nc(float x, float *fl)
{
    x = fminf(fmaxf(x, -4194304.f), 4194304.f);
    const float t = x + 12582912.f;
    const float r = t - 12582912.f;          // round(x), exact
    const int i = __float_as_int(t) - 0x4B400000;
    const bool up = r > x;
    *fl = up ? r - 1.f : r;
    return up ? i - 1 : i;
}

__device__ __forceinline__ int floor_nc(float x)
{
    float fl;
    return floor_nc(x, &fl);
}

// ceil(x) = -floor(-x), same range
__device__ __forceinline__ int ceil_nc(float x) { return -floor_nc(-x); }

// floor_nc without the clamp, for arguments bounded well inside |x| < 2^22
// by construction.  Outside that range (infinite or NaN arguments included)
// the result is an arbitrary int: every caller clamps it into a table or
// tests for an empty range before using it as an index.
__device__ __forceinline__ int floor_bounded(float x, float *fl)
{
    const float t = x + 12582912.f;
    const float r = t - 12582912.f;
    const int i = __float_as_int(t) - 0x4B400000;
    const bool up = r > x;
    *fl = up ? r - 1.f : r;
    return up ? i - 1 : i;
}

__device__ __forceinline__ int floor_bounded(float x)
{
    float fl;
    return floor_bounded(x, &fl);
}

__device__ __forceinline__ int ceil_bounded(float x) { return -floor_bounded(-x); }

__device__ inline double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ inline float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

} // namespace xrdt
