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
    ff k2f;                       // the same as a pair
    float tan_full, adet12, vox2, focal2_12;
};

// Per-voxel results of the scattering geometry.
struct VoxGeom {
    ff s;        // sin(theta/2)
    ff omc;      // 1 - cos(theta)
    ff sg;       // (sS2 + vV2 + dD2) / (|a|^2 |b|^2)
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
// The adjoint's window: every term that FP32 can represent.  2^(c d^2) flushes
// to zero below 2^-126, i.e. beyond sqrt(2 * 126 / log2(e)) = 13.2 sigma, so
// summing out to 13.25 sigma gives exactly the dense sum.  A sensitivity
// made of far-tail terms only can still be comparable to the 1e-7 that MLEM
// adds to it (main.m:162), so the adjoint cannot drop them.
constexpr float kSigAdj = 13.25f;
constexpr float kLog2e = 1.4426950408889634f;
constexpr float kLog2e_lo = (float)(1.4426950408889634074 - (double)kLog2e);

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
__device__ __forceinline__ float sqrt_approx(float x)
{
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rsqrt_approx(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

constexpr float kLn2 = 0.6931471805599453f;
constexpr float kTwelfth_hi = (float)(1.0 / 12.0);
constexpr float kTwelfth_lo = (float)(1.0 / 12.0 - (double)kTwelfth_hi);
// 0.5 log2(e) as a float pair: the Gaussian exp(-d^2 / (2 sigma^2)) is
// evaluated as 2^(c d^2) with c = -0.5 log2(e) / sigma^2
constexpr double kHalfLog2e = 0.72134752044448170368;
constexpr float kHalfLog2e_hi = (float)kHalfLog2e;
constexpr float kHalfLog2e_lo = (float)(kHalfLog2e - (double)kHalfLog2e_hi);

// c = -0.5 log2(e) / sigma^2 as a float pair, from sigma^2 as a pair.  The
// residual of the correctly rounded quotient is exact through the FMA.
__device__ __forceinline__ ff gauss_scale(ff sig2)
{
    const float rcp = rcp_approx(sig2.hi);
    const float ch = -kHalfLog2e_hi * rcp;
    // the quotient's residual, exact through the FMA to a bit or two
    float r = fmaf(-ch, sig2.hi, -kHalfLog2e_hi);
    r = fmaf(-ch, sig2.lo, r) - kHalfLog2e_lo;
    return {ch, r * rcp};
}

// 2^(c (w - q)^2) with the argument in FP32 but c as a pair: the scale c
// carries the systematic part of the error (sigma), the difference and its
// square round independently per term.
__device__ __forceinline__ float gauss_f32(float wh, float wl, float qh, float ql, float ch, float cl)
{
    const float d = (wh - qh) + (wl - ql);
    const float d2 = d * d;
    return ex2_approx(fmaf(ch, d2, cl * d2));
}

// 2^(c (w - q)^2) with w, q and c as float pairs.  The argument is formed
// as a pair (exact difference, exact square through the FMA), so its error
// is a few units of 2^-44 relative instead of a few FP32 ulps: deep in the
// Gaussian's tail, where the argument is tens, an FP32 argument would move
// the term by about 1e-6 relative.  The low part enters as 2^lo = 1 + lo ln2.
__device__ __forceinline__ float gauss_ff(float wh, float wl, float qh, float ql, float ch, float cl)
{
    const float t = wh - qh;   // exact while w and q are within a factor of two
    const float u = wl - ql;
    const float dh = t + u;
    const float dl = u - (dh - t);
    const float d2h = dh * dh;
    float d2l = fmaf(dh, dh, -d2h);
    d2l = fmaf(dh + dh, dl, d2l);
    const float ah = ch * d2h;
    float al = fmaf(ch, d2h, -ah);
    al = fmaf(ch, d2l, al);
    al = fmaf(cl, d2h, al);
    const float e = ex2_approx(ah);
    return fmaf(e, al * kLn2, e);
}

// Compton table bin of integrate_diffraction.cu:331-337 decided in FP64, as
// the oracle decides it; used only when the FP32 value lies within 2e-4 of a
// bin edge.  Kept out of line so that the rare FP64 path is a real branch
// and not predicated into every iteration of the energy loop.
__device__ __noinline__ int compton_bin_f64(const DevProblem &P, double ein, float omc_hi, float omc_lo)
{
    const double omcd = (double)omc_hi + (double)omc_lo;
    const double sd = sqrt(fabs(omcd) / 2.0);
    const double erd = 1.0 + ein * omcd;
    const double wd = ein * sd;
    const double l2d = log2(wd * sqrt(erd + wd * wd) / erd);
    return floor_to_int((l2d - P.q_min) / P.dq_tab);
}

// Compton table bin nq = floor((log2(w sqrt(eratio + w^2) / eratio) - q_min) / dq)
// with w = ein sin(theta/2), clamped to [0, NQ) (integrate_diffraction.cu:331-337).
// Decided in FP32 from the voxel's 1 - cos(theta) (pair (oh, ol)) and
// sin(theta/2) (hi part sh); within 2e-4 of a bin edge it is decided again in
// FP64.  eratio = 1 + ein oh and inv_er = 1/eratio as the caller formed them.
__device__ __forceinline__ int compton_bin(const DevProblem &P, float ein, float eratio, float inv_er, float sh,
                                           float oh, float ol, double ein_d, float qmin_t, float inv_dqt)
{
    const float wC = ein * sh;
    const float arg = eratio + wC * wC;
    const float l2 = lg2_approx(wC * arg * rsqrt_approx(arg) * inv_er);
    const float tq = (l2 - qmin_t) * inv_dqt;
    float ftq;
    int nq = floor_bounded(tq, &ftq);   // clamped to the table below
    const float fr = tq - ftq;
    if (!(fr > 2e-4f && fr < 1.f - 2e-4f))  // near a table edge
        nq = compton_bin_f64(P, ein_d, oh, ol);
    return nq < 0 ? 0 : (nq >= P.nq ? P.nq - 1 : nq);
}

// The cross-section table path (code the reference keeps commented out,
// integrate_diffraction.cu:701-719): the coherent table's wavevector bin
// nq = floor((log2(w) - q_min) / dq) with w = ein sin(theta/2), clamped to
// [0, NQ), decided in FP32 from the hi part of sin(theta/2); within 2e-4 of a
// bin edge again in FP64 from 1 - cos(theta) (pair (oh, ol)).
__device__ __noinline__ int coherent_bin_f64(const DevProblem &P, double ein, float omc_hi, float omc_lo)
{
    const double omcd = (double)omc_hi + (double)omc_lo;
    const double sd = sqrt(fabs(omcd) / 2.0);
    return floor_to_int((log2(ein * sd) - P.q_min) / P.dq_tab);
}

__device__ __forceinline__ int coherent_bin(const DevProblem &P, float ein, float sh, float oh, float ol,
                                            double ein_d, float qmin_t, float inv_dqt)
{
    const float tq = (lg2_approx(ein * sh) - qmin_t) * inv_dqt;
    float ftq;
    int nq = floor_bounded(tq, &ftq);   // clamped to the table below
    const float fr = tq - ftq;
    if (!(fr > 2e-4f && fr < 1.f - 2e-4f)) nq = coherent_bin_f64(P, ein_d, oh, ol);
    return nq < 0 ? 0 : (nq >= P.nq ? P.nq - 1 : nq);
}

// Bilinear value of a table [nq, na] (index q + a*nq, values as floats) at
// grid coordinates (tq, ta): the grid points are the table's entries,
// q_min + i (q_max - q_min)/(NQ - 1) (XSection_builder.m:121-125); clamped to
// the table (a NaN coordinate reads the first row or column).
__device__ __forceinline__ float table_bilinear(const float *S, int nq, int na, float tq, float ta)
{
    tq = fminf(fmaxf(tq, 0.f), (float)(nq - 1));
    ta = fminf(fmaxf(ta, 0.f), (float)(na - 1));
    const int i = min((int)tq, nq - 2), j = min((int)ta, na - 2);
    const float f = tq - (float)i, g = ta - (float)j;
    const float *r0 = S + i + j * nq, *r1 = r0 + nq;
    const float lo = fmaf(f, r0[1] - r0[0], r0[0]);
    const float hi = fmaf(f, r1[1] - r1[0], r1[0]);
    return fmaf(g, hi - lo, lo);
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
    G->k2f = ff_from_double(P.tan_full / nsxy);
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
// SIGMA_PAIR: sigma's blur terms as float pairs (the per-voxel operator,
// whose adjoint sums deep Gaussian tails); otherwise in FP32 (the material
// forward projector, whose counts are dominated by the Gaussians' cores).
template <bool SIGMA_PAIR>
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
    const float ia = __fdividef(1.f, An);
    const float Sx = (Cy * Az - Cz * Ay) * ia, Sy = (Cz * Ax - Cx * Az) * ia, Sz = (Cx * Ay - Cy * Ax) * ia;
    const float Snsrc = Sx * G.nsx + Sy * G.nsy + Sz * G.nsz;
    const float sS2 = (Sx * Sx + Sy * Sy + Sz * Sz - Snsrc * Snsrc) * G.focal2_12;
    if (!SIGMA_PAIR) {
        const float ib = __fdividef(1.f, Bn);
        const float Dx = (Cy * Bz - Cz * By) * ib, Dy = (Cz * Bx - Cx * Bz) * ib, Dz = (Cx * By - Cy * Bx) * ib;
        const float Vx = -(Sx + Dx), Vy = -(Sy + Dy), Vz = -(Sz + Dz);
        const float Dndet = Dx * G.ndx + Dy * G.ndy;
        const float dD2 = (Dx * Dx + Dy * Dy + Dz * Dz - Dndet * Dndet) * G.adet12;
        const float vV2 = (G.vox2 * (Vx * Vx + Vy * Vy) + Hvox * Hvox * Vz * Vz) * (1.f / 12.f);
        r.sg = ff{(sS2 + vV2 + dD2) * ia * ib, 0.f};
    } else {
        // The blur terms that make up most of sigma^2 as pairs: the Gaussian's
        // tail amplifies their relative error by (q distance / sigma)^2 / 2, and
        // FP32 leaves them about two ulps off.  V = -(S + D) = u x C with
        // u = a/|a|^2 + b/|b|^2 (S = C x a/|a|^2, D = C x b/|b|^2, C = a x b), and
        // |D|^2 - (D.n_det)^2 = Dz^2 + (Dx n_y - Dy n_x)^2 for the in-plane unit
        // normal n_det.
        const ff iaf = ff_div(ff{1.f, 0.f}, an), ibf = ff_div(ff{1.f, 0.f}, bn);
        const ff ux = ff_add(ff_mul(ax, iaf), ff_mul(bx, ibf));
        const ff uy = ff_add(ff_mul(ay, iaf), ff_mul(by, ibf));
        const ff uz = ff_add(ff_mul(az, iaf), ff_mul(bz, ibf));
        const ff Vx = ff_sub(ff_mul(uy, cz), ff_mul(uz, cy));
        const ff Vy = ff_sub(ff_mul(uz, cx), ff_mul(ux, cz));
        const ff Vz = ff_sub(ff_mul(ux, cy), ff_mul(uy, cx));
        const ff Hv = ff_mul(proj, G.k2f);
        const ff vV = ff_add(ff_mulf(ff_add(ff_sqr(Vx), ff_sqr(Vy)), G.vox2), ff_mul(ff_sqr(Hv), ff_sqr(Vz)));
        const ff Dx = ff_mul(ff_sub(ff_mul(cy, bz), ff_mul(cz, by)), ibf);
        const ff Dy = ff_mul(ff_sub(ff_mul(cz, bx), ff_mul(cx, bz)), ibf);
        const ff Dz = ff_mul(ff_sub(ff_mul(cx, by), ff_mul(cy, bx)), ibf);
        const ff Dt = ff_sub(ff_mulf(Dx, G.ndy), ff_mulf(Dy, G.ndx));
        const ff dD = ff_mulf(ff_add(ff_sqr(Dz), ff_sqr(Dt)), G.adet12);
        const ff blur = ff_add(ff_add(ff_mul(vV, ff{kTwelfth_hi, kTwelfth_lo}), dD), ff{sS2, 0.f});
        r.sg = ff_mul(ff_mul(blur, iaf), ibf);
    }
    const float Rdotn = -G.sphi * Ax + G.cphi * Ay;
    if (!SIGMA_PAIR) {
        const float cospsi = Rdotn * rsqrtf(Ax * Ax + Ay * Ay);
        const float gsv = cospsi * rsqrtf(An) * G.tan_full;
        const float gvd = -(G.ndx * Bx + G.ndy * By) * rsqrtf(Bn * Bn * Bn);
        r.gp = gsv * gvd;
    } else {
        // correctly rounded roots and quotients: the adjoint's column sums
        // inherit any bias of these factors, and MLEM amplifies it tenfold
        const float axy = __fsqrt_rn(fmaf(Ax, Ax, Ay * Ay));
        const float gsv = __fdiv_rn(__fdiv_rn(Rdotn, axy), __fsqrt_rn(An)) * G.tan_full;
        const float nb = __fsqrt_rn(Bn);
        const float gvd = __fdiv_rn(-(G.ndx * Bx + G.ndy * By), Bn * nb);
        r.gp = gsv * gvd;
    }
    r.Wg = r.gp * ((1.f + r.cos2) * 0.5f);
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
        // approximate root and quotient: the bin window is widened by one bin
        // on each side anyway
        const float na_ = __fdividef(2.f * ua, qb + sqrt_approx(da));
        const float nb_ = __fdividef(2.f * ub, qb + sqrt_approx(db));
        lo = max(lo, floor_nc(na_) - 1);
        hi = min(hi, floor_nc(nb_) + 1);
    }
    *klo = lo;
    *khi = hi;
}

} // namespace

} // namespace xrdt
