// k_fwd.cu -- factored forward projector (Nphotons, Cphotons, Amatrix).
//
// Same model as integrate_diffraction.cu:9-409, reorganised for the GPU:
//
//  * One block per (source, detector pixel) instead of one per
//    (source, pixel, detector energy bin).  Everything except the spectrum
//    weight RF = spectrum[e, nrg] and the Compton channel overlap depends on
//    the source energy e only (:266-356), so the block accumulates
//    T[e] = sum_v W(v,e) ... once per source bin and applies the banded
//    response afterwards: Nphotons[nrg] = sum_{e in window(nrg)} RF[e,nrg] T[e].
//    The reference evaluates each (voxel, e) pair once per detector bin whose
//    window holds e (11 times).
//  * Gaussian q-resolution sums (:299-315) run over the bins within 7.5 sigma
//    of the wavevector transfer only (each dropped term is below 7e-13 of the
//    peak); the reference sums every fine bin.
//  * The detector-side line integrals of the block's pair come from the table
//    that k_det_walk (k_walk.cu) writes for the current tile of pairs, one
//    float2 per voxel; the source-side ones from a per-(source, voxel) table
//    (k_prep.cu), since they do not depend on the detector pixel.
//  * Scattering geometry, ROI entry points and sample counts are FP64; the
//    wavevector transfer is carried as a float pair (about 48 significant
//    bits) because the Gaussian at 3 sigma amplifies its relative error by
//    several hundred; the rest is FP32 with Kahan-compensated sums over
//    voxels.
//
// Work split inside a block (8 warps): warp w takes voxel chunks w, w+8, ...
// of 32 voxels.  For a chunk, lane = voxel computes the scattering geometry
// and reads the voxel's line integrals; then for each voxel of the chunk
// lane = source energy evaluates the (voxel, energy) term and adds it to the
// warp's compensated per-energy sums.  A window of more than 32 energies that
// is not a multiple of 32 takes the chunk's (voxel, energy) items 32 at a
// time instead, so that no step runs with a few lanes.
#include "scatter.cuh"

namespace xrdt {

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;

struct Layout {
    size_t en, rf, offse, winlo, wn, ifine, fq, cq, s2, s1, tn, tns, cs, ck, ta, total;
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

// Shared-memory layout; identical on host and device.
__host__ __device__ inline Layout fwd_layout(const DevProblem &P, int E, int SL, int e_pass, bool with_n,
                                             bool with_a, int tab)
{
    Layout L;
    const int W = 2 * P.dnrg + 1;
    size_t o = 0;
    L.tn = o; o = align16(o + sizeof(double) * E);
    L.tns = o; o = align16(o + sizeof(float2) * kWarps * E);
    L.ck = o; o = align16(o + sizeof(float2) * kWarps * P.nrg_det);
    L.en = o; o = align16(o + sizeof(float) * 11 * E);
    L.rf = o; o = align16(o + sizeof(float) * P.nrg_det * W);
    L.offse = o; o = align16(o + sizeof(float) * E * SL);
    L.winlo = o; o = align16(o + sizeof(int) * P.nrg_det);
    L.wn = o; o = align16(o + sizeof(int) * 2 * E);
    L.cs = o; o = align16(o + sizeof(float) * kWarps * E * SL);
    L.ifine = o; if (with_n && !tab) o = align16(o + sizeof(float) * P.n_mat * (P.nqf + 3));
    L.fq = o; if (with_n && !tab) o = align16(o + sizeof(float2) * P.nqf);
    L.cq = o; if (with_a) o = align16(o + sizeof(float4) * P.nwt);
    L.s2 = o; o = align16(o + sizeof(float) * (size_t)P.nq * P.na);
    L.s1 = o; if (tab) o = align16(o + sizeof(float) * (size_t)P.nq * P.na);
    L.ta = o; if (with_a) o = align16(o + sizeof(float) * (size_t)e_pass * P.n_mat * P.nwt);
    L.total = o;
    return L;
}

struct FwdArgs {
    DevProblem P;
    const SrcGeom *sg;
    FwdTables T;
    const int *vox_xy, *vox_mat, *vox_na;
    const float *vox_a2;
    const float4 *cells;
    const float2 *atten_src;
    const unsigned char *s2u8;
    const unsigned char *s1u8;   // the table path: the coherent table
    const float *vox_ta;         // the table path, bilinear: the Compton column as a grid coordinate
    const float *Ifine;
    float *N, *C, *A;
    const int2 *pairs;         // a list of pairs, or NULL: the linear pairs src + det*SRC
    long long p0;              // block b takes pair p0 + b (of the list or of the linear index)
    int n_pairs;               // blocks of this launch
    long long n_cols;          // output columns: the list's length, or SRC*DET
    const float2 *walk;        // [block][nv] detector-side line integrals (k_walk.cu)
    int nv, E, e_pass, sl;
    F32Consts c;
};

// TAB: 0 the coherent term from the materials' fine-q patterns
// (integrate_diffraction.cu:299-308); 1 from the coherent table S1 by nearest
// bin, 2 with both tables read bilinearly (the cross-section table path).
template <bool WITH_N, bool WITH_A, int TAB>
__global__ void __launch_bounds__(kThreads, 3)
k_fwd(const FwdArgs args)
{
    extern __shared__ __align__(16) unsigned char sm[];
    __shared__ PairRec pair;   // the block's (source, pixel) constants
    const DevProblem &P = args.P;
    const F32Consts &c = args.c;
    const int E = args.E;
    const int W = 2 * P.dnrg + 1;
    const int SL = args.sl;
    const Layout L = fwd_layout(P, E, SL, args.e_pass, WITH_N, WITH_A, TAB);
    double *TN = (double *)(sm + L.tn);
    float2 *TNs = (float2 *)(sm + L.tns);
    float2 *Ck = (float2 *)(sm + L.ck);
    float *en = (float *)(sm + L.en);   // SoA: 9 rows of E
    float *en_if1 = en, *en_if2 = en + E, *en_wh = en + 2 * E, *en_wl = en + 3 * E;
    float *en_c1 = en + 4 * E, *en_c2 = en + 5 * E, *en_ein = en + 6 * E, *en_e1 = en + 7 * E;
    float *en_wn0f = en + 8 * E;   // first detector bin of wn as a float
    float *en_if1l = en + 9 * E, *en_if2l = en + 10 * E;   // low parts of 1/f1, 1/f2
    float *rf = (float *)(sm + L.rf);
    float *offse = (float *)(sm + L.offse);   // [E][SL] Esrc1(e) - Edet1(wn_lo(e) + s)
    int *winlo = (int *)(sm + L.winlo);
    int *wn = (int *)(sm + L.wn);
    float *CS = (float *)(sm + L.cs);         // [warp][E][SL] Compton sums of the current chunk
    float *Is = (float *)(sm + L.ifine);
    float2 *fq = (float2 *)(sm + L.fq);
    float4 *cq = (float4 *)(sm + L.cq);
    float *S2 = (float *)(sm + L.s2);   // quantised table as floats (no u8 conversion in the loop)
    float *S1 = (float *)(sm + L.s1);   // the table path's coherent table, the same way
    float *TA = (float *)(sm + L.ta);

    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    int det, src;
    int64_t colidx, ncols;   // output column of this block and the number of columns
    if (args.pairs) {
        colidx = args.p0 + blockIdx.x;
        const int2 pr = args.pairs[colidx];
        src = pr.x;
        det = pr.y;
        ncols = args.n_cols;
    } else {
        colidx = args.p0 + blockIdx.x;
        src = (int)(colidx % P.n_src);
        det = (int)(colidx / P.n_src);
        ncols = (int64_t)P.n_src * P.n_det;
    }
    const float2 *walk = args.walk + (int64_t)blockIdx.x * args.nv;

    // ---- stage the tables ----
    for (int i = tid; i < E; i += kThreads) {
        const EnergyRow r = args.T.energy[P.e_lo + i];
        en_if1[i] = r.inv_f1;
        en_if2[i] = r.inv_f2;
        en_if1l[i] = r.inv_f1_lo;
        en_if2l[i] = r.inv_f2_lo;
        en_wh[i] = r.wfac_hi;
        en_wl[i] = r.wfac_lo;
        en_c1[i] = r.sig_c1;
        en_c2[i] = r.sig_c2;
        en_ein[i] = r.einf;
        en_e1[i] = r.Esrc1f;
        TN[i] = 0.0;
        for (int w = 0; w < kWarps; w++) TNs[w * E + i] = make_float2(0.f, 0.f);
        wn[2 * i] = args.T.win_n[2 * (P.e_lo + i)];
        en_wn0f[i] = (float)wn[2 * i];
        wn[2 * i + 1] = args.T.win_n[2 * (P.e_lo + i) + 1];
    }
    for (int i = tid; i < P.nrg_det * W; i += kThreads) rf[i] = args.T.rf_win[i];
    for (int i = tid; i < E * SL; i += kThreads) offse[i] = args.T.offs_e[P.e_lo * SL + i];
    for (int i = tid; i < kWarps * E * SL; i += kThreads) CS[i] = 0.f;
    for (int i = tid; i < P.nrg_det; i += kThreads) winlo[i] = args.T.win_lo[i];
    for (int i = tid; i < kWarps * P.nrg_det; i += kThreads) Ck[i] = make_float2(0.f, 0.f);
    if (WITH_N && !TAB) {
        // rows of nqf + 3: each material's pattern and three zero pads
        for (int i = tid; i < P.n_mat * (P.nqf + 3); i += kThreads) {
            const int mm = i / (P.nqf + 3), j = i - mm * (P.nqf + 3);
            Is[i] = j < P.nqf ? __ldg(args.Ifine + mm * P.nqf + j) : 0.f;
        }
        for (int i = tid; i < P.nqf; i += kThreads) fq[i] = args.T.fine_q[i];
    }
    if (WITH_A)
        for (int i = tid; i < P.nwt; i += kThreads) cq[i] = args.T.coarse_q[i];
    for (int i = tid; i < P.nq * P.na; i += kThreads) S2[i] = (float)args.s2u8[i];
    if (TAB)
        for (int i = tid; i < P.nq * P.na; i += kThreads) S1[i] = (float)args.s1u8[i];

    // ---- per-(source, pixel) geometry, integrate_diffraction.cu:81-128 ----
    if (tid == 0) pair_geom(P, args.sg[src], det, &pair.G, &pair.Rdx, &pair.Rdy);
    const PairGeom &G = pair.G;
    const float rsqrt2pi = c.rsqrt2pi;
    const float dqf_hi = c.dqf_hi, dqf_lo = c.dqf_lo;
    const float inv_dqf = c.inv_dqf, qlo_f = c.q_lo;
    const float kn0 = c.kn0, kn1 = c.kn1, kn2 = c.kn2;
    const float edmin = c.edmin, inv_dEd = c.inv_dEd, dEdf = c.dEd;
    const float dEsf = c.dEs, inv_dEs = c.inv_dEs;
    const float qmin_t = c.qmin_t, inv_dqt = c.inv_dqt;
    const int lo_e = P.e_lo;
    __syncthreads();

    unsigned int nexp = 0;   // exp2 evaluations of this lane (profiling only)
    float2 *TNw = TNs + wid * E;   // this warp's Kahan sums per source energy

    const int nv = args.nv;
    const int nchunks = (nv + 31) >> 5;
    for (int pe0 = 0; pe0 < E; pe0 += args.e_pass) {
        const int pe1 = min(E, pe0 + args.e_pass);
        if (WITH_A) {
            for (int i = tid; i < (pe1 - pe0) * P.n_mat * P.nwt; i += kThreads) TA[i] = 0.f;
            __syncthreads();
        }
        for (int chunk = wid; chunk < nchunks; chunk += kWarps) {
            // ---- lane = voxel: scattering geometry (integrate_diffraction.cu:192-255) ----
            const int v = min(chunk * 32 + lane, nv - 1);
            const int xy = args.vox_xy[v];
            const float vx = ((float)(xy & 0xffff) + 0.5f) * c.vox;
            const float vy = ((float)(xy >> 16) + 0.5f) * c.vox;
            const VoxGeom vg = vox_geom<false>(G, vx, vy);
            const int mv = args.vox_mat[v];
            const int nav = args.vox_na[v];
            const float a2v = args.vox_a2[v];
            const float2 Asv = args.atten_src[(int64_t)src * nv + v];
            const float2 Adv = walk[v];
            const float tav = TAB == 2 ? args.vox_ta[v] : 0.f;
            // per-voxel factors, formed once here instead of once per term:
            // the Compton weight gp a2 / 2 (the 1/2 of Cf, :347), the
            // Rayleigh weight with 1/sqrt(2 pi), and sigma_geom / s^2
            const float gpav = vg.gp * a2v * 0.5f;
            const float wrv = vg.Wg * rsqrt2pi;
            const float sgs2v = __fdividef(vg.sg.hi, vg.s.hi * vg.s.hi);

            const int nin = min(32, nv - chunk * 32);
            // the (voxel, source energy) term, :266-356, of voxel i of the chunk
            // (its constants as arguments) for energy el.  Labels as at
            // integrate_diffraction.cu:259-260: the detector-side integral Ad
            // feeds Pin, the source-side one (Asx, Asy) Pout.
            auto term = [&](int el, float2 Ad, float sh, float sl, float oh, float ol, float gpa, float Wr,
                            float Wg, float cos2, int m, int na, float a2now, float Asx, float Asy, float ta,
                            float s2f, float sg_s2) {
                // ---- (voxel, source energy) term, :266-356 ----
                // attenuation exponents with 1/f1, 1/f2 as pairs: X reaches
                // tens at the lowest energies, where FP32 constants alone
                // would move exp(-X) by a few 1e-6
                const float if1 = en_if1[el], if2 = en_if2[el];
                const float if1l = en_if1l[el], if2l = en_if2l[el];
                const float Xin = fmaf(Ad.x, if1, fmaf(Ad.y, if2, fmaf(Ad.x, if1l, Ad.y * if2l)));
                const float Xout = fmaf(Asx, if1, fmaf(Asy, if2, fmaf(Asx, if1l, Asy * if2l)));
                const float wh0 = en_wh[el], wl0 = en_wl[el];
                float w_hi = wh0 * sh;
                float w_lo = fmaf(wh0, sh, -w_hi) + fmaf(wh0, sl, wl0 * sh);
                {
                    const float t = w_hi + w_lo;
                    w_lo = w_lo - (t - w_hi);
                    w_hi = t;
                }
                const float sig2 = fmaf(en_c1[el], s2f, en_c2[el] * sg_s2);
                const float rs = rsqrtf(sig2);
                const float cexp = -0.5f * kLog2e * rs * rs;
                const float Xio = Xin + Xout;
                const float PP = ex2_approx(-fmaf(Xio, kLog2e, Xio * kLog2e_lo));
                nexp += 1;
                const float pref = PP * Wr * rs;
                const float half = kSig * sig2 * rs;
                if (WITH_N && TAB) {
                    // the coherent term from the table S1 (the reference's
                    // commented-out kernel, integrate_diffraction.cu:701-719):
                    // Pin Pout geom Rayleigh a2 S1[wvt bin, a-ratio bin] with
                    // wvt = ein sin(theta/2) on the tables' log2 axis
                    const float ein = en_ein[el];
                    float s1v;
                    if (TAB == 1) {
                        s1v = S1[coherent_bin(P, ein, sh, oh, ol, args.T.energy[lo_e + el].ein, qmin_t, inv_dqt) +
                                 na * P.nq];
                    } else {
                        s1v = table_bilinear(S1, P.nq, P.na, (lg2_approx(ein * sh) - qmin_t) * c.inv_dqg, ta);
                    }
                    float2 k = TNw[el];
                    kahan_add(k.x, k.y, PP * Wg * a2now * s1v);
                    TNw[el] = k;
                }
                if (WITH_N && !TAB) {
                    const float jc = (w_hi - qlo_f) * inv_dqf - 0.5f;
                    // bounded floors: the indices are clamped to the grid and an
                    // empty window is skipped
                    const int jlo = max(ceil_bounded(jc - half * inv_dqf), 0);
                    int jhi = min(floor_bounded(jc + half * inv_dqf), P.nqf - 1);
                    float acc = 0.f;
                    // pref == 0: the attenuation factor underflowed, every term is 0
                    if (jlo <= jhi && pref != 0.f) {
                        // a multiple of four bins, so the loop has no tail: the
                        // extra bins are exact terms of the full sum or the zero
                        // pads after the last bin.  (A tail would make the
                        // compiler rebuild the float counter from the trip count
                        // through an int-to-float conversion, which this GPU
                        // issues on its FP64 pipe.)
                        jhi += (4 - ((jhi - jlo + 1) & 3)) & 3;
                        nexp += (unsigned)(jhi - jlo + 1);
                        // The exponent c (w - q_j)^2 as a quadratic in u = j - jc
                        // about the bin jc nearest the centre: with
                        // delta = w - q_jc (|delta| <= dq/2),
                        //   c (delta - u dq)^2 = A + B u + C u^2,
                        // A = c delta^2, B = -2 c delta dq, C = c dq^2 (dq^2
                        // with the grid step's low part).  Near the
                        // peak the sum is A alone; far out C u^2 dominates, so
                        // the exponent keeps the relative accuracy of the direct
                        // form in two FMAs per bin.
                        const float2 q0 = fq[jlo];
                        const float d0 = (w_hi - q0.x) + (w_lo - q0.y);
                        const float tc = rintf(d0 * inv_dqf);
                        const float delta = fmaf(-tc, dqf_lo, fmaf(-tc, dqf_hi, d0));
                        const float cd = cexp * delta;
                        const float Aq = cd * delta;
                        const float Bq = -2.f * cd * dqf_hi;
                        const float Cq = cexp * fmaf(dqf_hi, dqf_hi, 2.f * dqf_hi * dqf_lo);
                        const float *Ir = Is + m * (P.nqf + 3) + jlo;
                        const float *Iend = Ir + (jhi - jlo + 1);
                        float acc2 = 0.f;
                        float u = -tc;   // bin offset from jc as a float: no conversion in the loop
                        for (; Ir < Iend; Ir += 4, u += 4.f) {
                            const float u1 = u + 1.f, u2 = u + 2.f, u3 = u + 3.f;
                            acc = fmaf(ex2_approx(fmaf(fmaf(Cq, u, Bq), u, Aq)), Ir[0], acc);
                            acc2 = fmaf(ex2_approx(fmaf(fmaf(Cq, u1, Bq), u1, Aq)), Ir[1], acc2);
                            acc = fmaf(ex2_approx(fmaf(fmaf(Cq, u2, Bq), u2, Aq)), Ir[2], acc);
                            acc2 = fmaf(ex2_approx(fmaf(fmaf(Cq, u3, Bq), u3, Aq)), Ir[3], acc2);
                        }
                        acc += acc2;
                    }
                    float2 k = TNw[el];
                    kahan_add(k.x, k.y, pref * dqf_hi * acc);
                    TNw[el] = k;
                }
                if (WITH_A) {
                    int klo, khi;
                    coarse_window(w_hi, half, qlo_f, c.qpar_a, c.qpar_b, P.nwt, &klo, &khi);
                    float *tar = TA + ((size_t)(el - pe0) * P.n_mat + m) * P.nwt;
                    nexp += (unsigned)max(0, khi - klo + 1);
                    for (int k = klo; k <= khi; k++) {
                        const float4 c = cq[k];
                        const float d = (w_hi - c.x) + (w_lo - c.y);
                        atomicAdd(tar + k, pref * c.z * ex2_approx(cexp * d * d));
                    }
                }
                // ---- Compton, :318-356 ----
                {
                    const float ein = en_ein[el];
                    // no contraction: the Compton bin check forms eratio the same way
                    const float x = __fmul_rn(ein, oh);       // eratio - 1
                    const float eratio = __fadd_rn(1.f, x);
                    const float inv_er = rcp_approx(eratio);
                    const int eg = lo_e + el;
                    // detector bins whose window holds e and whose channel the
                    // outgoing range [E1, E2]/eratio can overlap
                    const float Eo_lo = en_e1[el];
                    // channels overlapped by [E1, E2]/eratio (an FP32 misjudgement at a
                    // channel edge drops an overlap below 1e-6 of the bin width)
                    float fn0;
                    // bounded floors: n0 is raised to the window, n1 lowered to it,
                    // and an empty range is skipped
                    int n0 = floor_bounded((Eo_lo * inv_er - edmin) * inv_dEd, &fn0);
                    if (n0 < wn[2 * el]) {
                        n0 = wn[2 * el];
                        fn0 = en_wn0f[el];
                    }
                    const int n1 = min(wn[2 * el + 1], floor_bounded(((Eo_lo + dEsf) * inv_er - edmin) * inv_dEd));
                    if (n0 <= n1) {
                        // the table's value: nearest bin, or bilinear in the table path
                        float s2v;
                        if (TAB == 2) {
                            const float wC = ein * sh;
                            const float arg = eratio + wC * wC;
                            const float l2 = lg2_approx(wC * arg * rsqrt_approx(arg) * inv_er);
                            s2v = table_bilinear(S2, P.nq, P.na, (l2 - qmin_t) * c.inv_dqg, ta);
                        } else {
                            s2v = S2[compton_bin(P, ein, eratio, inv_er, sh, oh, ol, args.T.energy[eg].ein, qmin_t,
                                                 inv_dqt) +
                                     na * P.nq];
                        }
                        // Pc = exp(-(Xin + Xc)) with Xc the source-side exponent at
                        // the outgoing energy eout = ein / eratio, formed as the
                        // Rayleigh one plus the small Compton change, so that Pc
                        // keeps the accuracy of PP:
                        //   Asx (1/eout^3 - 1/ein^3) = Asx/ein^3 ((1 + x)^3 - 1)
                        //   Asy (1/KN(eout) - 1/KN(ein))
                        //     = Asy (ein - eout)(kn1 + kn2 (ein + eout)) / (KN(ein) KN(eout))
                        const float eout = ein * inv_er;
                        const float f2o = fmaf(kn2 * eout, eout, fmaf(kn1, eout, kn0));
                        const float cube = x * fmaf(x, x + 3.f, 3.f);            // (1 + x)^3 - 1
                        const float dX = fmaf(Asx * if1, cube,
                                              Asy * (x * eout) * fmaf(kn2, ein + eout, kn1) * if2 * rcp_approx(f2o));
                        const float Pc = PP * ex2_approx(-dX * kLog2e);
                        nexp += 1;
                        // an underflowed Pc adds exact zeros below: no branch
                        // twice Cf of :347 (gpa holds the 1/2)
                        const float Cf2 = eratio * eratio * (eratio + inv_er - 1.f + cos2);
                        const float base = Pc * gpa * Cf2 * s2v;
                        const float span = dEsf * inv_er;   // Eout2 - Eout1
                        const float inv_span = eratio * inv_dEs;
                        // this lane's (warp, energy) row of chunk sums, indexed by n;
                        // the spectrum weight RF[e, n] is applied when the chunk is
                        // flushed, so no two lanes ever write the same word
                        const int wlo = wn[2 * el];
                        float *cs = CS + ((size_t)wid * E + el) * SL - wlo;
                        const float *oe = offse + (size_t)el * SL - wlo;
                        const float bs = base * inv_span;
                        float Ed1 = fmaf(fn0, dEdf, edmin);
                        // outgoing range relative to the channel's left edge:
                        // u1 = Eout1 - Edet1 = ((Esrc1 - Edet1) - Edet1*x)/eratio.
                        // The range is one source bin wide over eratio >= 1, so
                        // with dEs <= dEd it meets at most two channels: those
                        // two straight-line, any further ones in a loop.
                        {
                            const float u1 = fmaf(-Ed1, x, oe[n0]) * inv_er;
                            const float ov = fminf(u1 + span, dEdf) - fmaxf(u1, 0.f);
                            if (ov > 0.f) cs[n0] += ov * bs;
                        }
                        if (n0 < n1) {
                            const float Ed2 = Ed1 + dEdf;
                            const float u1 = fmaf(-Ed2, x, oe[n0 + 1]) * inv_er;
                            const float ov = fminf(u1 + span, dEdf) - fmaxf(u1, 0.f);
                            if (ov > 0.f) cs[n0 + 1] += ov * bs;
                            Ed1 = Ed2 + dEdf;
                            for (int n = n0 + 2; n <= n1; n++, Ed1 += dEdf) {
                                const float u1n = fmaf(-Ed1, x, oe[n]) * inv_er;
                                const float ovn = fminf(u1n + span, dEdf) - fmaxf(u1n, 0.f);
                                if (ovn > 0.f) cs[n] += ovn * bs;
                            }
                        }
                    }
                }
            };
            const int ne = pe1 - pe0;
            if (ne > 32 && (ne & 31)) {
                // a pass that is not a multiple of 32 energies (40 on the 64x64
                // and 128x128 workloads): the chunk's (voxel, energy) items 32
                // at a time, so that no step runs with a few lanes.  The items
                // of a step have distinct energies (32 < ne): distinct sums
                // TNw[el] and Compton cells, each still adding its voxels in
                // order, so the counts are the same to the bit.
                int i = 0, eo = lane;
                for (int t0 = 0; t0 < nin * ne; t0 += 32) {
                    const float2 Ad = make_float2(__shfl_sync(0xffffffffu, Adv.x, i), __shfl_sync(0xffffffffu, Adv.y, i));
                    const float sh = __shfl_sync(0xffffffffu, vg.s.hi, i);
                    const float sl = __shfl_sync(0xffffffffu, vg.s.lo, i);
                    const float oh = __shfl_sync(0xffffffffu, vg.omc.hi, i);
                    const float ol = __shfl_sync(0xffffffffu, vg.omc.lo, i);
                    const float gpa = __shfl_sync(0xffffffffu, gpav, i);
                    const float Wr = __shfl_sync(0xffffffffu, wrv, i);
                    const float Wg = TAB ? __shfl_sync(0xffffffffu, vg.Wg, i) : 0.f;
                    const float cos2 = __shfl_sync(0xffffffffu, vg.cos2, i);
                    const int m = __shfl_sync(0xffffffffu, mv, i);
                    const int na = __shfl_sync(0xffffffffu, nav, i);
                    const float a2now = TAB ? __shfl_sync(0xffffffffu, a2v, i) : 0.f;
                    const float Asx = __shfl_sync(0xffffffffu, Asv.x, i);
                    const float Asy = __shfl_sync(0xffffffffu, Asv.y, i);
                    const float ta = TAB == 2 ? __shfl_sync(0xffffffffu, tav, i) : 0.f;
                    const float s2f = sh * sh;
                    const float sg_s2 = __shfl_sync(0xffffffffu, sgs2v, i);
                    if (i < nin) term(pe0 + eo, Ad, sh, sl, oh, ol, gpa, Wr, Wg, cos2, m, na, a2now, Asx, Asy, ta, s2f, sg_s2);
                    eo += 32;
                    if (eo >= ne) {
                        eo -= ne;
                        i++;
                    }
                }
            } else {
                for (int i = 0; i < nin; i++) {
                    const float2 Ad = make_float2(__shfl_sync(0xffffffffu, Adv.x, i), __shfl_sync(0xffffffffu, Adv.y, i));
                    const float sh = __shfl_sync(0xffffffffu, vg.s.hi, i);
                    const float sl = __shfl_sync(0xffffffffu, vg.s.lo, i);
                    const float oh = __shfl_sync(0xffffffffu, vg.omc.hi, i);
                    const float ol = __shfl_sync(0xffffffffu, vg.omc.lo, i);
                    const float gpa = __shfl_sync(0xffffffffu, gpav, i);
                    const float Wr = __shfl_sync(0xffffffffu, wrv, i);
                    const float Wg = TAB ? __shfl_sync(0xffffffffu, vg.Wg, i) : 0.f;
                    const float cos2 = __shfl_sync(0xffffffffu, vg.cos2, i);
                    const int m = __shfl_sync(0xffffffffu, mv, i);
                    const int na = __shfl_sync(0xffffffffu, nav, i);
                    const float a2now = TAB ? __shfl_sync(0xffffffffu, a2v, i) : 0.f;
                    const float Asx = __shfl_sync(0xffffffffu, Asv.x, i);
                    const float Asy = __shfl_sync(0xffffffffu, Asv.y, i);
                    const float ta = TAB == 2 ? __shfl_sync(0xffffffffu, tav, i) : 0.f;
                    const float s2f = sh * sh;
                    const float sg_s2 = __shfl_sync(0xffffffffu, sgs2v, i);
#pragma unroll 1
                    for (int el = pe0 + lane; el < pe1; el += 32)
                        term(el, Ad, sh, sl, oh, ol, gpa, Wr, Wg, cos2, m, na, a2now, Asx, Asy, ta, s2f, sg_s2);
                }
            }
            // flush the chunk's Compton sums: lane = detector bin n gathers the
            // (energy, slot) cells that map to n, weights them with RF[e, n]
            // and adds the result to its compensated total
            __syncwarp();
            for (int n = lane; n < P.nrg_det; n += 32) {
                float s = 0.f;
                for (int j = 0; j < W; j++) {
                    const int el = winlo[n] + j - lo_e;
                    if (el < pe0 || el >= pe1) continue;
                    float *c = CS + ((size_t)wid * E + el) * SL + (n - wn[2 * el]);
                    s = fmaf(*c, rf[n * W + j], s);
                    *c = 0.f;
                }
                float2 k = Ck[wid * P.nrg_det + n];
                kahan_add(k.x, k.y, s);
                Ck[wid * P.nrg_det + n] = k;
            }
            __syncwarp();
        }
        __syncthreads();
        if (WITH_A) {
            // Amatrix[k, m, src, det, nrg] = sum_{e in window(nrg)} RF[e,nrg] T_A[e,m,k]
            const int MW = P.n_mat * P.nwt;
            const int64_t colbase = colidx * MW;
            const int64_t nstride = (int64_t)MW * ncols;
            for (int idx = tid; idx < P.nrg_det * MW; idx += kThreads) {
                const int n = idx / MW, mk = idx - n * MW;
                float acc = 0.f;
                for (int j = 0; j < W; j++) {
                    const int el = winlo[n] + j - lo_e;
                    if (el >= pe0 && el < pe1) acc = fmaf(rf[n * W + j], TA[(size_t)(el - pe0) * MW + mk], acc);
                }
                float *dst = args.A + colbase + (int64_t)n * nstride + mk;
                if (pe0 == 0) *dst = acc;
                else *dst += acc;
            }
            __syncthreads();
        }
    }

    if (args.T.work) {
        unsigned long long w = nexp;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
        if (lane == 0) atomicAdd(args.T.work, w);
    }

    // ---- outputs: ray index src + det*SRC + nrg*SRC*DET (:404) ----
    __syncthreads();
    for (int el = tid; el < E; el += kThreads) {
        double s = 0.0;
        for (int w = 0; w < kWarps; w++) s += (double)TNs[w * E + el].x - (double)TNs[w * E + el].y;
        TN[el] = s;
    }
    __syncthreads();
    for (int n = tid; n < P.nrg_det; n += kThreads) {
        const int64_t ray = colidx + (int64_t)n * ncols;
        if (WITH_N) {
            double acc = 0.0;
            for (int j = 0; j < W; j++) acc += (double)rf[n * W + j] * TN[winlo[n] + j - lo_e];
            args.N[ray] = (float)acc;
        }
        double c = 0.0;
        for (int w = 0; w < kWarps; w++) {
            const float2 k = Ck[w * P.nrg_det + n];
            c += (double)k.x - (double)k.y;
        }
        args.C[ray] = (float)c;
    }
}

template <bool WN, bool WA, int TAB>
cudaError_t launch_variant(const FwdArgs &a, size_t smem, cudaStream_t s)
{
    cudaError_t e = cudaFuncSetAttribute(k_fwd<WN, WA, TAB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_fwd<WN, WA, TAB><<<(unsigned)a.n_pairs, kThreads, smem, s>>>(a);
    return cudaGetLastError();
}

__global__ void k_gather_rays(const int64_t *__restrict__ idx, int64_t n, const float *__restrict__ Nc,
                              const float *__restrict__ Cc, const float *__restrict__ Ac, int mw,
                              float *__restrict__ N, float *__restrict__ C, float *__restrict__ A)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
        N[i] = Nc[idx[i]];
        C[i] = Cc[idx[i]];
    }
    if (A)
        for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * mw; t += stride)
            A[t] = Ac[idx[t / mw] * mw + t % mw];
}

} // namespace

cudaError_t launch_gather_rays(const int64_t *idx, int64_t n, const float *Nc, const float *Cc,
                               const float *Ac, int mw, float *N, float *C, float *A, cudaStream_t s,
                               int64_t *launches)
{
    if (n == 0) return cudaSuccess;
    k_gather_rays<<<1024, 256, 0, s>>>(idx, n, Nc, Cc, Ac, mw, N, C, A);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

size_t fast_forward_smem(const DevProblem &P, int sl, int e_pass, bool with_n, bool with_a, int tab)
{
    const int E = P.e_hi - P.e_lo + 1;
    return fwd_layout(P, E, sl, e_pass, with_n, with_a, tab).total;
}

cudaError_t launch_fast_forward(const DevProblem &P, const SrcGeom *d_src, const FwdTables &T,
                                const PrepBuffers &B, int nv, const float *Ifine, const int2 *pairs,
                                long long n_list, long long p0, int n_pairs, const float2 *walk, float *N,
                                float *C, float *A, cudaStream_t s, int64_t *launches, int tab)
{
    // the table path computes Nphotons and Cphotons only
    if (tab && (A || !N || tab > 2 || !B.s1u8 || (tab == 2 && !B.vox_ta))) return cudaErrorInvalidValue;
    FwdArgs a;
    a.pairs = pairs;
    a.p0 = p0;
    a.n_pairs = n_pairs;
    a.n_cols = pairs ? n_list : (long long)P.n_src * P.n_det;
    a.walk = walk;
    a.P = P;
    a.sg = d_src;
    a.T = T;
    a.vox_xy = B.vox_xy;
    a.vox_mat = B.vox_mat;
    a.vox_na = B.vox_na;
    a.vox_a2 = B.vox_a2;
    a.cells = B.cells;
    a.atten_src = B.atten_src;
    a.s2u8 = B.s2u8;
    a.s1u8 = B.s1u8;
    a.vox_ta = B.vox_ta;
    a.Ifine = Ifine;
    a.N = N;
    a.C = C;
    a.A = A;
    a.nv = nv;
    a.E = P.e_hi - P.e_lo + 1;
    a.sl = T.sl;
    a.c = make_f32_consts(P);
    const bool with_n = (N != nullptr);
    const bool with_a = (A != nullptr);
    // energies per pass: all of them unless the model-matrix accumulator
    // would push the block past ~110 KB of shared memory
    int e_pass = a.E;
    if (with_a) {
        while (e_pass > 1 && fwd_layout(P, a.E, a.sl, e_pass, with_n, true, 0).total > 110 * 1024) e_pass = (e_pass + 1) / 2;
    }
    a.e_pass = e_pass;
    const size_t smem = fwd_layout(P, a.E, a.sl, e_pass, with_n, with_a, tab).total;
    if (smem + sizeof(PairRec) > 227 * 1024) return cudaErrorInvalidConfiguration;   // dynamic + static
    if (launches) (*launches)++;
    if (nv == 0) {
        // empty phantom: the reference writes zeros (integrate_diffraction.cu:364-409)
        cudaError_t e = cudaSuccess;
        return e;
    }
    if (tab == 1) return launch_variant<true, false, 1>(a, smem, s);
    if (tab == 2) return launch_variant<true, false, 2>(a, smem, s);
    if (with_n && with_a) return launch_variant<true, true, 0>(a, smem, s);
    if (with_n) return launch_variant<true, false, 0>(a, smem, s);
    if (with_a) return launch_variant<false, true, 0>(a, smem, s);
    return launch_variant<false, false, 0>(a, smem, s);
}

} // namespace xrdt
