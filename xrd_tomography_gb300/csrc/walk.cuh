// walk.cuh -- the attenuation line integral (attenuator.cu:9-109) over the
// bilinear cell map.
//
// The integer decisions (which ROI edge is entered, how many samples the ray
// takes) are those of the reference, made in FP32 with guard bands
// (walk_setup_f32) or in FP64 (walk_setup).  Two ways to sum the samples:
// walk_cells, one lane per ray, cell by cell with closed-form sums over the
// samples inside each cell, anchored at the voxel with float-pair offsets
// (the projector's and the operators' walks); and walk_coop, the 32 lanes of
// a warp on one ray, lane l taking samples l, l+32, ... (the CT sinogram).
#pragma once

#include "xrdt_device.cuh"
#include "ff.cuh"

namespace xrdt {

struct WalkSetup {
    float rx, ry;   // ROI entry point (GetIntersection) minus one voxel in x and y
    float Lx, Ly;   // DQ times the unit direction entry -> voxel
    int n;          // number of samples: k = 0 .. n-1
    int edge;       // ROI edge entered (GetIntersection's order: bottom, right,
                    // top, left), -1 when the segment misses the ROI
    // The same samples anchored at the voxel v, for walk_cells: sample k sits
    // at v + (dlt + (n-1-k) DQ) u with u the unit vector from the voxel back
    // to the entry point and dlt = Lr - (n-1) DQ the distance of the last
    // sample from the voxel, both as float pairs.
    ff dlt, ux, uy;
};

// GetIntersection + the sample count of attenuator.cu:19-52: every k in
// [0, kmax) with DQ*k <= Lr.  A segment that misses the ROI gives n = 0
// (the reference compares against a NaN length and takes no sample).
__device__ inline void walk_setup(const DevProblem &P, double ex, double ey, double vx, double vy,
                                  WalkSetup *w)
{
    double rx, ry;
    get_intersection(ex, ey, vx, vy, P.nx, P.ny, &rx, &ry, &w->edge);
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
    w->rx = (float)(rx - 1.0);
    w->ry = (float)(ry - 1.0);
    w->Lx = (float)(Lx * P.DQ);
    w->Ly = (float)(Ly * P.DQ);
    w->n = (int)n;
    if (n > 0) {
        w->dlt = ff_from_double(Lr - P.DQ * (double)(n - 1));
        w->ux = ff_from_double(-Lx);
        w->uy = ff_from_double(-Ly);
    } else {
        w->dlt = w->ux = w->uy = ff{0.f, 0.f};
    }
}

// The voxel-anchored form of a set-up whose edge and sample count are
// decided (walk_setup_f32), from the endpoint (ex, ey) as float pairs: with
// D = v - e, the entry point on edge x = X0 lies at Lr = |D| (vx - X0)/Dx
// from the voxel (y = Y0: |D| (vy - Y0)/Dy), and u = -D/|D|.
__device__ __forceinline__ void walk_anchor_ff(const F32Consts &C, ff ex, ff ey, float vx, float vy, WalkSetup *w)
{
    if (w->n <= 0) {
        w->dlt = w->ux = w->uy = ff{0.f, 0.f};
        return;
    }
    const ff Dx = ff_fsub(vx, ex), Dy = ff_fsub(vy, ey);
    const ff D = ff_sqrt(ff_add(ff_sqr(Dx), ff_sqr(Dy)));
    ff ratio;
    switch (w->edge) {
    case 0: ratio = ff_div(ff{vy, 0.f}, Dy); break;              // y = 0
    case 1: ratio = ff_div(ff{vx - C.nxf, 0.f}, Dx); break;      // x = NX
    case 2: ratio = ff_div(ff{vy - C.nyf, 0.f}, Dy); break;      // y = NY
    default: ratio = ff_div(ff{vx, 0.f}, Dx); break;             // x = 0
    }
    const ff Lr = ff_mul(D, ratio);
    w->dlt = ff_sub(Lr, ff_mulf(ff{(float)(w->n - 1), 0.f}, C.DQ));
    w->ux = ff_neg(ff_div(Dx, D));
    w->uy = ff_neg(ff_div(Dy, D));
}

// FP32 version of walk_setup for the endpoint (ex, ey) rounded to float.
// Returns false when a decision is too close to its threshold for FP32 to be
// trusted -- a nearly edge-parallel ray, a ray through an ROI corner, or a
// length within a few FP32 errors of a multiple of DQ (axis-aligned rays hit
// the latter exactly) -- and the caller then decides in FP64 with
// walk_setup.  Endpoint rounding (|e| ~ 300 voxels -> 1.5e-5) dominates the
// FP32 error; the guards are several times that.
__device__ __forceinline__ bool walk_setup_f32(const DevProblem &P, const F32Consts &C, float ex, float ey,
                                               float vx, float vy, WalkSetup *w)
{
    const float NX = C.nxf, NY = C.nyf, DQ = C.DQ, inv_DQ = C.inv_DQ;
    const float eps = 0.00001f;
    const float G = 2e-4f;
    const float dx = vx - ex, dy = vy - ey;
    float rx = 0.f, ry = 0.f;
    bool found = false;
    int edge = -1;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const float x3 = (i == 1 || i == 2) ? NX : 0.f;
        const float x4 = (i == 0 || i == 1) ? NX : 0.f;
        const float y3 = (i >= 2) ? NY : 0.f;
        const float y4 = (i == 1 || i == 2) ? NY : 0.f;
        const float x4_x3 = x4 - x3, y3_y1 = y3 - ey, y4_y3 = y4 - y3, x3_x1 = x3 - ex;
        const float den = x4_x3 * dy - dx * y4_y3;
        if (fabsf(den) < 1e-2f) return false;     // edge-parallel within FP32 error
        const float inv = __fdividef(1.f, den);
        const float ua = (x4_x3 * y3_y1 - x3_x1 * y4_y3) * inv;
        if (fabsf(ua + eps) < G || fabsf(ua - (1.f + eps)) < G) return false;
        if (ua > -eps && ua < 1.f + eps) {
            const float ub = (dx * y3_y1 - x3_x1 * dy) * inv;
            if (fabsf(ub + eps) < G || fabsf(ub - (1.f + eps)) < G) return false;
            if (ub > -eps && ub < 1.f + eps) {
                rx = fmaf(dx, ua, ex);
                ry = fmaf(dy, ua, ey);
                found = true;
                edge = i;
                break;
            }
        }
    }
    if (!found) return false;
    float Lx = vx - rx, Ly = vy - ry;
    const float L2 = fmaf(Lx, Lx, Ly * Ly);
    const float rL = rsqrtf(L2);
    const float t = sqrtf(L2) * inv_DQ;
    float ft;
    const int it = floor_nc(t, &ft);
    const float fr = t - ft;
    const float gt = fmaf(4e-7f, t, 1e-3f);
    if (fr < gt || fr > 1.f - gt) return false;
    long long n = (long long)it + 1;
    if (n > P.kmax) n = P.kmax;
    w->rx = rx - 1.f;
    w->ry = ry - 1.f;
    w->Lx = Lx * rL * DQ;
    w->Ly = Ly * rL * DQ;
    w->n = (int)n;
    w->edge = edge;
    return true;
}

// One bilinear sample of the cell map at texture coordinates (X+1, Y+1),
// P = (X, Y).  Cell (ci, cj) holds the coefficients of the texels
// (ci-1..ci, cj-1..cj) of the zero-bordered map in the frame of the cell
// centre: f = d00 + d10 u + d01 v + d11 u v with u = X - round(X) and
// v = Y - round(Y) in [-0.5, 0.5] (k_prep.cu).  The interpolant is
// continuous, so any base cell whose square holds the point gives the same
// value, and rounding through the float mantissa (adding 1.5 * 2^23) needs
// no conversion instruction.  Valid for |X| < 2^22; the cell index is
// clamped for memory safety.  Both components are evaluated with packed
// FP32 instructions (two lanes of one register pair: a1 and a2).
__device__ __forceinline__ float2 cell_sample(const float4 *__restrict__ cells, int nx, unsigned ncell_m1, float2 P)
{
    const float2 t = __fadd2_rn(P, make_float2(12582912.f, 12582912.f));
    const int ix = __float_as_int(t.x) - 0x4B400000, iy = __float_as_int(t.y) - 0x4B400000;
    const float2 r = __fadd2_rn(t, make_float2(-12582912.f, -12582912.f));   // round(P), exact
    const float2 d = __ffma2_rn(r, make_float2(-1.f, -1.f), P);               // P - round(P), exact
    const unsigned c = min((unsigned)(ix + 1 + (iy + 1) * (nx + 1)), ncell_m1);
    const float4 c0 = __ldg(cells + 2 * c), c1 = __ldg(cells + 2 * c + 1);
    const float2 lo = __ffma2_rn(make_float2(d.y, d.y), make_float2(c1.x, c1.y), make_float2(c0.x, c0.y));
    const float2 hi = __ffma2_rn(make_float2(d.y, d.y), make_float2(c1.z, c1.w), make_float2(c0.z, c0.w));
    return __ffma2_rn(make_float2(d.x, d.x), hi, lo);
}

// Sum of the n samples times DQ; every lane returns the total.  Lane l takes
// samples l, l+32, l+64, ... two per iteration; the sample index is carried
// as a float (no int-to-float conversion per sample) and the sample point
// r + k L is formed for x and y in one packed FMA.
__device__ __forceinline__ float2 walk_coop(const float4 *__restrict__ cells, int nx, int ny,
                                            const WalkSetup &w, float DQ, int lane)
{
    const unsigned ncell_m1 = (unsigned)((nx + 1) * (ny + 1) - 1);
    const float2 L2 = make_float2(w.Lx, w.Ly), R2 = make_float2(w.rx, w.ry);
    float2 sa = make_float2(0.f, 0.f), sb = make_float2(0.f, 0.f);
    float kf = __int_as_float(0x4B000000 | lane) - 8388608.f;   // (float)lane
    int k = lane;
    for (; k + 32 < w.n; k += 64, kf += 64.f) {
        const float2 a = cell_sample(cells, nx, ncell_m1, __ffma2_rn(L2, make_float2(kf, kf), R2));
        const float kg = kf + 32.f;
        const float2 b = cell_sample(cells, nx, ncell_m1, __ffma2_rn(L2, make_float2(kg, kg), R2));
        sa = __fadd2_rn(sa, a);
        sb = __fadd2_rn(sb, b);
    }
    if (k < w.n) sa = __fadd2_rn(sa, cell_sample(cells, nx, ncell_m1, __ffma2_rn(L2, make_float2(kf, kf), R2)));
    const float s1 = warp_sum(sa.x + sb.x);
    const float s2 = warp_sum(sa.y + sb.y);
    return make_float2(s1 * DQ, s2 * DQ);
}

// The same sum walked cell by cell by one lane.  The bilinear patch of a
// cell is a polynomial in the sample index, so the samples j = 0 .. m-1 of
// a run inside one cell add up in closed form: with (u0, v0) the first
// sample's offset from the cell centre, S1 = m(m-1)/2 and
// S2 = (m-1)m(2m-1)/6,
//     sum u = m u0 + Lx S1,   sum v = m v0 + Ly S1,
//     sum uv = m u0 v0 + (u0 Ly + v0 Lx) S1 + Lx Ly S2,
//     sum f = m c00 + c10 sum u + c01 sum v + c11 sum uv.
// Each step takes the cell of its first sample (as cell_sample does) and
// the run up to the first sample beyond the cell's exit edge, at least one
// sample.  A sample within rounding of an edge may fall on either side; the
// interpolant is continuous there, so the sum changes only by rounding.  The
// runs are added with Kahan compensation.  One cell load serves the 3-4
// samples of a run (DQ = 1/4 voxel), where the cooperative walk loads a cell
// per sample.  The samples are taken from the last (next to the voxel) to
// the first: rays that end on one voxel then start together and part slowly,
// so the lanes of a warp walking such rays read neighbouring cells.
// Cell (ci, cj) is cells[2 (ci sx + cj sy)]: sx = 1, sy = NX+1 for the
// row-major map, sx = NY+1, sy = 1 for the column-major copy.  Each step
// reads its 32-byte cell with one 256-bit load (sm_100 and later; cells are
// 32-byte aligned in a device allocation): the L1 cost of a warp-wide load
// follows the cache lines its lanes touch, so one load per cell instead of
// two halves it.  Measured on the 256x256 workload: 1085 ms against 1140 ms
// for two 16-byte loads.
__device__ __forceinline__ void ld_cell256(const float4 *p, float4 &c0, float4 &c1)
{
    asm("ld.global.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(c0.x), "=f"(c0.y), "=f"(c0.z), "=f"(c0.w), "=f"(c1.x), "=f"(c1.y), "=f"(c1.z), "=f"(c1.w)
        : "l"(p));
}

__device__ __forceinline__ float2 walk_cells(const float4 *__restrict__ cells, int sx, int sy, unsigned ncell_m1,
                                             const WalkSetup &w, float vx, float vy, float DQ)
{
    const float magic = 12582912.f;
    const float nf = (float)w.n;
    // samples from the voxel outwards: sample j at v + (dlt + j DQ) u
    const float2 L = make_float2(w.ux.hi * DQ, w.uy.hi * DQ);
    // minus the inverse steps, clamped so that a run is never overestimated
    const float ilx = fabsf(L.x) > 1e-4f ? -1.f / L.x : (L.x < 0.f ? 1e4f : -1e4f);
    const float ily = fabsf(L.y) > 1e-4f ? -1.f / L.y : (L.y < 0.f ? 1e4f : -1e4f);
    const float2 ninv = make_float2(ilx, ily);
    // exit edge offset h = +-0.5 (towards the step) times the inverse step
    const float2 hinv = make_float2(L.x < 0.f ? 0.5f * ilx : -0.5f * ilx, L.y < 0.f ? 0.5f * ily : -0.5f * ily);
    const float lxly = L.x * L.y;
    const float2 uhi = make_float2(w.ux.hi, w.uy.hi), ulo = make_float2(w.ux.lo, w.uy.lo), v2 = make_float2(vx, vy);
    // the distance of the voxel's nearest sample is below one step unless the
    // sample count was capped: then a two-sum that needs no ordering
    const bool small_dlt = w.dlt.hi <= DQ;
    float2 acc = make_float2(0.f, 0.f), comp = make_float2(0.f, 0.f);
    for (float k0 = 0.f; k0 < nf;) {
        // distance s = dlt + k0 DQ and displacement t = s u as float pairs
        // (exact products through the FMA): the sample's offset from its cell
        // centre is then good to about 1e-7 voxel, where a position formed
        // at a magnitude of hundreds of voxels in FP32 would be off by 1e-5
        // and shift the interpolant by as much at material edges
        // (explicitly rounded operations, x and y packed in one instruction:
        // a contracted multiply-add would count a product's error twice)
        const float kq = __fmul_rn(k0, DQ);
        const float kqe = fmaf(k0, DQ, -kq);
        const float sh = __fadd_rn(w.dlt.hi, kq);
        float sl;
        if (small_dlt) {
            sl = __fadd_rn(__fsub_rn(w.dlt.hi, __fsub_rn(sh, kq)), __fadd_rn(kqe, w.dlt.lo));   // |kq| >= dlt
        } else {
            const float bb = __fsub_rn(sh, w.dlt.hi);
            sl = __fadd_rn(__fadd_rn(__fsub_rn(w.dlt.hi, __fsub_rn(sh, bb)), __fsub_rn(kq, bb)),
                           __fadd_rn(kqe, w.dlt.lo));
        }
        const float2 s2 = make_float2(sh, sh);
        const float2 p = __fmul2_rn(s2, uhi);
        const float2 e = __fadd2_rn(__ffma2_rn(s2, uhi, make_float2(-p.x, -p.y)),
                                    __ffma2_rn(s2, ulo, __fmul2_rn(make_float2(sl, sl), uhi)));
        // the cell whose centre is nearest (any cell holding the point gives
        // the same value: the interpolant is continuous), then the offset
        const float2 t = __fadd2_rn(__fadd2_rn(v2, p), make_float2(magic, magic));
        const int ix = __float_as_int(t.x) - 0x4B400000, iy = __float_as_int(t.y) - 0x4B400000;
        const unsigned c = min((unsigned)(ix * sx + iy * sy), ncell_m1);
        float4 c0, c1;
        ld_cell256(cells + 2 * c, c0, c1);
        // the cell centre (exact) minus the anchor is exact, and it cancels
        // p but for the offset (Sterbenz), so only e rounds
        const float2 r = __fadd2_rn(t, make_float2(-magic, -magic));
        const float2 d = __fadd2_rn(__fadd2_rn(__fadd2_rn(v2, make_float2(-r.x, -r.y)), p), e);
        const float2 s = __ffma2_rn(d, ninv, hinv);                                // steps to each exit edge
        // ceil(s) as round(s + 1/2) through the float mantissa (either way at a tie)
        float m = __fadd_rn(__fadd_rn(__fadd_rn(fminf(s.x, s.y), 0.5f), magic), -magic);
        m = fminf(fmaxf(m, 1.f), nf - k0);
        const float S1 = 0.5f * __fmaf_rn(m, m, -m);
        const float S2 = S1 * __fmaf_rn(m, 2.f / 3.f, -1.f / 3.f);
        const float2 su = __ffma2_rn(d, make_float2(m, m), __fmul2_rn(L, make_float2(S1, S1)));
        float suv = __fmul_rn(__fmul_rn(d.x, d.y), m);
        suv = __fmaf_rn(__fmaf_rn(d.x, L.y, __fmul_rn(d.y, L.x)), S1, suv);
        suv = __fmaf_rn(lxly, S2, suv);
        float2 part = __fmul2_rn(make_float2(suv, suv), make_float2(c1.z, c1.w));
        part = __ffma2_rn(make_float2(su.y, su.y), make_float2(c1.x, c1.y), part);
        part = __ffma2_rn(make_float2(su.x, su.x), make_float2(c0.z, c0.w), part);
        part = __ffma2_rn(make_float2(m, m), make_float2(c0.x, c0.y), part);
        const float2 y = __fadd2_rn(part, make_float2(-comp.x, -comp.y));
        const float2 tt = __fadd2_rn(acc, y);
        comp = __fadd2_rn(__fadd2_rn(tt, make_float2(-acc.x, -acc.y)), make_float2(-y.x, -y.y));
        acc = tt;
        k0 += m;
    }
    return make_float2((acc.x - comp.x) * DQ, (acc.y - comp.y) * DQ);
}

} // namespace xrdt
