// scatter.cuh -- per-(source, pixel) and per-voxel scattering geometry of
// integrate_diffraction.cu:81-255 in the form the FP32 kernels consume, and
// the SFU helpers they share (k_fwd.cu: materials; k_vox.cu: per-voxel
// coefficients).
//
// The wavevector transfer is carried as a float pair (about 48 significant
// bits) because the Gaussian q resolution at 3 sigma amplifies its relative
// error by several hundred; 1 - cos(theta) comes from the cross product, so
// small angles lose nothing to cancellation.  The rest is FP32.
#pragma once

#include "xrdt_device.cuh"
#include "ff.cuh"
#include "walk.cuh"

namespace xrdt {

// Per-(source, pixel) constants of the scattering geometry.
struct PairGeom {
    ff Rsx, Rsy, Rdx, Rdy, Rdz;   // source and detector positions
    ff k1;                        // tan(geomphi/2) / |nsrc_xy|
    ff nsx2, nsy2;                // in-plane source orientation as pairs
    float nsx, nsy, nsz, ndx, ndy, sphi, cphi;
    float k2;                     // tan(geomphi) / |nsrc_xy|
    float tan_full, adet12, vox2, focal2_12;
};

// Per-voxel results of the scattering geometry.
struct VoxGeom {
    ff s;        // sin(theta/2)
    ff omc;      // 1 - cos(theta)
    float sg;    // (sS2 + vV2 + dD2) / (|a|^2 |b|^2)
    float gp;    // geom_src2vox * geom_vox2det
    float Wg;    // gp * Rayleigh factor
    float cos2;  // cos^2(theta)
};

// A pair's constants with its detector position in double, tabulated once
// per operator (k_vox.cu).
struct PairRec {
    PairGeom G;
    double Rdx, Rdy;
};

namespace {

constexpr float kSig = 7.5f;            // Gaussian window, in sigma (tail below 7e-13)
constexpr float kLog2e = 1.4426950408889634f;

__device__ __forceinline__ void kahan_add(float &s, float &c, float x)
{
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
}

// SFU approximations with denormals flushed (no denormal fix-up code; the
// arguments here are far from the denormal range)
__device__ __forceinline__ float ex2_approx(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_approx(float x)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float lg2_approx(float x)
{
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rsqrt_approx(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// FP64 walk set-up out of line: the rare fallback of walk_setup_f32 stays a
// real branch instead of being predicated into the caller's loop.
__device__ __noinline__ void walk_setup_f64(const DevProblem &P, double ex, double ey, double vx, double vy,
                                            WalkSetup *w)
{
    walk_setup(P, ex, ey, vx, vy, w);
}

// integrate_diffraction.cu:93-128 for source g and pixel det: the pair's
// constants and the detector position in double.
__device__ __forceinline__ void pair_geom(const DevProblem &P, const SrcGeom &g, int det, PairGeom *G,
                                          double *Rdet_x, double *Rdet_y)
{
    double Rdz;
    det_position(P, g.sphi, g.cphi, det, Rdet_x, Rdet_y, &Rdz);
    G->Rsx = ff_from_double(g.Rsrc_x);
    G->Rsy = ff_from_double(g.Rsrc_y);
    G->Rdx = ff_from_double(*Rdet_x);
    G->Rdy = ff_from_double(*Rdet_y);
    G->Rdz = ff_from_double(Rdz);
    const double nsx = -g.sphi * P.sta, nsy = g.cphi * P.sta, nsz = -P.cta;
    const double nsxy = sqrt(nsx * nsx + nsy * nsy);
    G->nsx = (float)nsx;
    G->nsy = (float)nsy;
    G->nsx2 = ff_from_double(nsx);
    G->nsy2 = ff_from_double(nsy);
    G->nsz = (float)nsz;
    G->k1 = ff_from_double(P.tan_half / nsxy);
    G->k2 = (float)(P.tan_full / nsxy);
    G->ndx = (float)g.sphi;
    G->ndy = (float)(-g.cphi);
    G->sphi = (float)g.sphi;
    G->cphi = (float)g.cphi;
    G->tan_full = (float)P.tan_full;
    G->adet12 = (float)(P.geomAdet / 12.0);
    G->vox2 = (float)(P.vox * P.vox);
    G->focal2_12 = (float)(P.focal * P.focal / 12.0);
}

// integrate_diffraction.cu:196-255 for one voxel.  a = voxel - source and
// b = detector - voxel as float pairs; 1 - cos(theta) from the cross product
// |a x b|^2 / (|a||b| (|a||b| + a.b)), which has no cancellation at small
// angles; the blur vectors S = ((a x b) x a)/|a|^2 = b - (a.b/|a|^2) a and
// D = ((a x b) x b)/|b|^2 = -a + (a.b/|b|^2) b in FP32.
__device__ __forceinline__ VoxGeom vox_geom(const PairGeom &G, float vx, float vy)
{
    const ff ax = ff_fsub(vx, G.Rsx), ay = ff_fsub(vy, G.Rsy);
    const ff proj = ff_add(ff_mul(ax, G.nsx2), ff_mul(ay, G.nsy2));
    const ff az = ff_neg(ff_mul(proj, G.k1));          // Rvox_z; Rsrc_z = 0
    const float Hvox = proj.hi * G.k2;
    const ff bx = ff_add(G.Rdx, ff{-vx, 0.f}), by = ff_add(G.Rdy, ff{-vy, 0.f});
    const ff bz = ff_sub(G.Rdz, az);
    const ff ab = ff_add(ff_add(ff_mul(ax, bx), ff_mul(ay, by)), ff_mul(az, bz));
    const ff an = ff_add(ff_add(ff_sqr(ax), ff_sqr(ay)), ff_sqr(az));
    const ff bn = ff_add(ff_add(ff_sqr(bx), ff_sqr(by)), ff_sqr(bz));
    const ff cx = ff_sub(ff_mul(ay, bz), ff_mul(az, by));
    const ff cy = ff_sub(ff_mul(az, bx), ff_mul(ax, bz));
    const ff cz = ff_sub(ff_mul(ax, by), ff_mul(ay, bx));
    const ff cn = ff_add(ff_add(ff_sqr(cx), ff_sqr(cy)), ff_sqr(cz));
    const ff nab = ff_sqrt(ff_mul(an, bn));
    VoxGeom r;
    if (ab.hi > 0.f) r.omc = ff_div(cn, ff_mul(nab, ff_add(nab, ab)));
    else r.omc = ff_fsub(1.f, ff_div(ab, nab));
    r.s = ff_sqrt(ff_mulf(r.omc, 0.5f));
    const float costh = 1.f - r.omc.hi;
    r.cos2 = costh * costh;
    // FP32 remainder of the geometry
    const float Ax = ax.hi, Ay = ay.hi, Az = az.hi, Bx = bx.hi, By = by.hi, Bz = bz.hi;
    const float Cx = cx.hi, Cy = cy.hi, Cz = cz.hi, An = an.hi, Bn = bn.hi;
    const float ia = __fdividef(1.f, An), ib = __fdividef(1.f, Bn);
    const float Sx = (Cy * Az - Cz * Ay) * ia, Sy = (Cz * Ax - Cx * Az) * ia, Sz = (Cx * Ay - Cy * Ax) * ia;
    const float Dx = (Cy * Bz - Cz * By) * ib, Dy = (Cz * Bx - Cx * Bz) * ib, Dz = (Cx * By - Cy * Bx) * ib;
    const float Vx = -(Sx + Dx), Vy = -(Sy + Dy), Vz = -(Sz + Dz);
    const float Dndet = Dx * G.ndx + Dy * G.ndy;
    const float Snsrc = Sx * G.nsx + Sy * G.nsy + Sz * G.nsz;
    const float dD2 = (Dx * Dx + Dy * Dy + Dz * Dz - Dndet * Dndet) * G.adet12;
    const float vV2 = (G.vox2 * (Vx * Vx + Vy * Vy) + Hvox * Hvox * Vz * Vz) * (1.f / 12.f);
    const float sS2 = (Sx * Sx + Sy * Sy + Sz * Sz - Snsrc * Snsrc) * G.focal2_12;
    const float Rdotn = -G.sphi * Ax + G.cphi * Ay;
    const float cospsi = Rdotn * rsqrtf(Ax * Ax + Ay * Ay);
    const float gsv = cospsi * rsqrtf(An) * G.tan_full;
    const float gvd = -(G.ndx * Bx + G.ndy * By) * rsqrtf(Bn * Bn * Bn);
    r.gp = gsv * gvd;
    r.Wg = r.gp * ((1.f + r.cos2) * 0.5f);
    r.sg = (sS2 + vV2 + dD2) * ia * ib;
    return r;
}

// Coarse q bins that can lie within `half` of w: invert the bin edges
// edge(n) = q_lo + b n + a n^2 of wvt_value.cu:8-22 at w - half and w + half,
// widened by one bin on each side against rounding.  Returns the full range
// when the parabola has no real inverse there.
__device__ __forceinline__ void coarse_window(float w, float half, float q_lo, float qa, float qb, int nwt,
                                              int *klo, int *khi)
{
    int lo = 0, hi = nwt - 1;
    const float ua = w - half - q_lo, ub = w + half - q_lo;
    const float da = fmaf(4.f * qa, ua, qb * qb), db = fmaf(4.f * qa, ub, qb * qb);
    if (da >= 0.f && db >= 0.f) {
        const float na_ = 2.f * ua / (qb + sqrtf(da));
        const float nb_ = 2.f * ub / (qb + sqrtf(db));
        lo = max(lo, floor_nc(na_) - 1);
        hi = min(hi, floor_nc(nb_) + 1);
    }
    *klo = lo;
    *khi = hi;
}

} // namespace

} // namespace xrdt
