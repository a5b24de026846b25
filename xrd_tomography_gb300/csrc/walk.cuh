// walk.cuh -- the attenuation line integral (attenuator.cu:9-109) as a
// warp-cooperative walk over the bilinear cell map.
//
// The integer decisions (which ROI edge is entered, how many samples the ray
// takes) are made in FP64 exactly as the reference defines them; the
// samples themselves are summed in FP32 by the 32 lanes of a warp, lane l
// taking samples l, l+32, ... (consecutive samples of one ray are 0.25 voxel
// apart, so one warp instruction touches a few neighbouring cells).
#pragma once

#include "xrdt_device.cuh"

namespace xrdt {

struct WalkSetup {
    float rx, ry;   // ROI entry point (GetIntersection)
    float Lx, Ly;   // unit direction entry -> voxel
    int n;          // number of samples: k = 0 .. n-1
};

// GetIntersection + the sample count of attenuator.cu:19-52: every k in
// [0, kmax) with DQ*k <= Lr.  A segment that misses the ROI gives n = 0
// (the reference compares against a NaN length and takes no sample).
__device__ inline void walk_setup(const DevProblem &P, double ex, double ey, double vx, double vy,
                                  WalkSetup *w)
{
    double rx, ry;
    get_intersection(ex, ey, vx, vy, P.nx, P.ny, &rx, &ry);
    double Lx = vx - rx, Ly = vy - ry;
    const double L2 = dadd(dmul(Lx, Lx), dmul(Ly, Ly));
    const double Lr = sqrt(L2);
    const double rL = 1.0 / sqrt(L2);
    Lx *= rL;
    Ly *= rL;
    long long n = 0;
    if (Lr >= 0.0) {
        long long k = (long long)floor(Lr / P.DQ);
        while (dmul(P.DQ, (double)(k + 1)) <= Lr) k++;
        while (k >= 0 && !(dmul(P.DQ, (double)k) <= Lr)) k--;
        n = k + 1;
        if (n > P.kmax) n = P.kmax;
    }
    w->rx = (float)rx;
    w->ry = (float)ry;
    w->Lx = (float)Lx;
    w->Ly = (float)Ly;
    w->n = (int)n;
}

// One bilinear sample of the cell map at (x, y) in voxel units (the
// texture's unnormalised coordinates).  Returns (a1, a2).
__device__ __forceinline__ float2 cell_sample(const float4 *__restrict__ cells, int nx, int ny, float x,
                                              float y)
{
    const float xb = x - 0.5f, yb = y - 0.5f;
    const float fx = floorf(xb), fy = floorf(yb);
    const float ux = xb - fx, uy = yb - fy;
    int ci = (int)fx + 1, cj = (int)fy + 1;
    ci = min(max(ci, 0), nx);
    cj = min(max(cj, 0), ny);
    const float4 *c = cells + 2 * ((int64_t)ci + (int64_t)cj * (nx + 1));
    const float4 c0 = __ldg(c), c1 = __ldg(c + 1);
    const float b0 = fmaf(ux, c0.z - c0.x, c0.x), b1 = fmaf(ux, c1.z - c1.x, c1.x);
    const float d0 = fmaf(ux, c0.w - c0.y, c0.y), d1 = fmaf(ux, c1.w - c1.y, c1.y);
    return make_float2(fmaf(uy, b1 - b0, b0), fmaf(uy, d1 - d0, d0));
}

// Sum of the n samples times DQ; every lane returns the total.
__device__ __forceinline__ float2 walk_coop(const float4 *__restrict__ cells, int nx, int ny,
                                            const WalkSetup &w, float DQ, int lane)
{
    float s1 = 0.f, s2 = 0.f;
    for (int k = lane; k < w.n; k += 32) {
        const float qr = DQ * (float)k;
        const float2 v = cell_sample(cells, nx, ny, fmaf(w.Lx, qr, w.rx), fmaf(w.Ly, qr, w.ry));
        s1 += v.x;
        s2 += v.y;
    }
    s1 = warp_sum(s1);
    s2 = warp_sum(s2);
    return make_float2(s1 * DQ, s2 * DQ);
}

} // namespace xrdt
