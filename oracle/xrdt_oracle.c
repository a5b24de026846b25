/*
 * xrdt_oracle.c -- FP64 CPU restatement of the reference forward projector.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  See xrdt_oracle.h.
 *
 * Each function cites the reference lines it restates.  One ray of the
 * oracle is one CUDA block of integrate_diffraction (src, det, nrg); the 256
 * threads of that block (one per coarse q bin nwt) become explicit loops and
 * the shuffle reductions become serial sums.
 */
#include "xrdt_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <limits.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* __float2int_rd with CUDA semantics: NaN -> 0, saturating at the int range. */
static int cuda_floor_int(double x)
{
    if (isnan(x)) return 0;
    double f = floor(x);
    if (f >= 2147483647.0) return INT_MAX;
    if (f <= -2147483648.0) return INT_MIN;
    return (int)f;
}

/* wvt_value.cu:8-22: parabolic coarse q grid,
 * qedge(n) = qmin + n*dq0 + (qmax - qmin - dq0*NWT) * n^2 / NWT^2. */
void xrdt_oracle_wvt_value(const xrdt_problem *p, int32_t nwt, double *qnow, double *dqnow)
{
    const double NWT = (double)p->nwt;
    double qedge1 = p->q_lo + (double)nwt * p->dq0 +
                    (p->q_hi - p->q_lo - p->dq0 * NWT) *
                        (double)((int64_t)nwt * nwt) / (double)((int64_t)p->nwt * p->nwt);
    double qedge2 = p->q_lo + (double)(nwt + 1) * p->dq0 +
                    (p->q_hi - p->q_lo - p->dq0 * NWT) *
                        (double)((int64_t)(nwt + 1) * (nwt + 1)) / (double)((int64_t)p->nwt * p->nwt);
    *qnow = 0.5 * (qedge1 + qedge2);
    *dqnow = qedge2 - qedge1;
}

/* Centre source bin of detector bin nrg.  With identical grids this is nrg
 * itself, which is what find_src_nrg_range.cu:10 uses; otherwise the source
 * bin that contains the detector bin's centre energy. */
static int src_centre_bin(const xrdt_problem *p, int nrg)
{
    if (p->nrg_src == p->nrg_det && p->e_src_min == p->e_det_min && p->e_src_max == p->e_det_max)
        return nrg;
    double dEs = (p->e_src_max - p->e_src_min) / (double)p->nrg_src;
    double dEd = (p->e_det_max - p->e_det_min) / (double)p->nrg_det;
    double ec = p->e_det_min + ((double)nrg + 0.5) * dEd;
    return cuda_floor_int((ec - p->e_src_min) / dEs);
}

/* find_src_nrg_range.cu:8-25: an always 2*DNRG+1 wide window, shifted down at
 * the top end. */
void xrdt_oracle_src_nrg_range(const xrdt_problem *p, int32_t nrg, int32_t *lo, int32_t *hi)
{
    int c = src_centre_bin(p, nrg);
    int nrg_min = c - p->dnrg;
    if (nrg_min < 0) nrg_min = 0;
    int nrg_max = nrg_min + 2 * p->dnrg;
    if (nrg_max >= p->nrg_src) {
        nrg_max = p->nrg_src - 1;
        nrg_min = nrg_max - 2 * p->dnrg;
    }
    *lo = nrg_min;
    *hi = nrg_max;
}

/* GetIntersection.cu:9-57: first of the four ROI edges (bottom, right, top,
 * left) that the segment (x1,y1)->(x2,y2) crosses, with the 1e-5 tolerances
 * of :20,:39,:43,:47; NaN if none. */
static int get_intersection_edge(double x1, double y1, double x2, double y2, int32_t nx, int32_t ny,
                                 double *rx, double *ry);

int32_t xrdt_oracle_get_intersection(double x1, double y1, double x2, double y2,
                                     int32_t nx, int32_t ny, double *rx, double *ry)
{
    return get_intersection_edge(x1, y1, x2, y2, nx, ny, rx, ry) >= 0;
}

/* The same, returning the index of the edge entered (0..3 in the order
 * above) or -1. */
static int get_intersection_edge(double x1, double y1, double x2, double y2, int32_t nx, int32_t ny,
                                 double *rx, double *ry)
{
    const double NX = (double)nx, NY = (double)ny;
    const double x3[4] = {0.0, NX, NX, 0.0};
    const double x4[4] = {NX, NX, 0.0, 0.0};
    const double y3[4] = {0.0, 0.0, NY, NY};
    const double y4[4] = {0.0, NY, NY, 0.0};
    const double eps = (double)0.00001f;
    double x2_x1 = x2 - x1, y2_y1 = y2 - y1;
    *rx = NAN;
    *ry = NAN;
    for (int i = 0; i < 4; i++) {
        double x4_x3 = x4[i] - x3[i];
        double y3_y1 = y3[i] - y1;
        double y4_y3 = y4[i] - y3[i];
        double x3_x1 = x3[i] - x1;
        double den = x4_x3 * y2_y1 - x2_x1 * y4_y3;
        if (den > eps || den < -eps) {
            double u_a = (x4_x3 * y3_y1 - x3_x1 * y4_y3) / den;
            if (u_a > -eps && u_a < 1.0 + eps) {
                double u_b = (x2_x1 * y3_y1 - x3_x1 * y2_y1) / den;
                if (u_b > -eps && u_b < 1.0 + eps) {
                    *rx = x1 + x2_x1 * u_a;
                    *ry = y1 + y2_y1 * u_a;
                    return i;
                }
            }
        }
    }
    return -1;
}

/* tex2D of Forward_XRD.cu:229-233: linear filtering, unnormalised
 * coordinates, border address mode (zero outside), texel (i,j) centred at
 * (i+0.5, j+0.5); evaluated exactly in double. */
static void tex_bilinear(const float *a1, const float *a2, int nx, int ny,
                         double x, double y, double *v1, double *v2)
{
    double xb = x - 0.5, yb = y - 0.5;
    double fi = floor(xb), fj = floor(yb);
    double fx = xb - fi, fy = yb - fj;
    long i0 = (long)fi, j0 = (long)fj;
    double s1 = 0.0, s2 = 0.0;
    for (int dj = 0; dj < 2; dj++) {
        long j = j0 + dj;
        if (j < 0 || j >= ny) continue;
        double wy = dj ? fy : 1.0 - fy;
        for (int di = 0; di < 2; di++) {
            long i = i0 + di;
            if (i < 0 || i >= nx) continue;
            double w = wy * (di ? fx : 1.0 - fx);
            s1 += w * (double)a1[i + j * (long)nx];
            s2 += w * (double)a2[i + j * (long)nx];
        }
    }
    *v1 = s1;
    *v2 = s2;
}

/* attenuator.cu:9-109.  Samples at r_int + Lhat*(DQ*k) for every k with
 * DQ*k <= Lr (:44-69), k below maxBatch*threads (:44, integrate_diffraction.cu:160-161),
 * summed then multiplied by DQ (:104-105). */
static int64_t attenuator_edge(const xrdt_problem *p, const float *a1, const float *a2,
                               double ex, double ey, double vx, double vy,
                               double *A1, double *A2, int *edge);

int64_t xrdt_oracle_attenuator(const xrdt_problem *p, const float *a1, const float *a2,
                               double ex, double ey, double vx, double vy,
                               double *A1, double *A2)
{
    return attenuator_edge(p, a1, a2, ex, ey, vx, vy, A1, A2, NULL);
}

/* The same, also reporting the ROI edge the ray enters through. */
static int64_t attenuator_edge(const xrdt_problem *p, const float *a1, const float *a2,
                               double ex, double ey, double vx, double vy,
                               double *A1, double *A2, int *edge)
{
    const int NX = p->nx, NY = p->ny;
    const double DQ = p->dq_step;
    double rx, ry;
    const int e = get_intersection_edge(ex, ey, vx, vy, NX, NY, &rx, &ry);
    if (edge) *edge = e;
    double Lx = vx - rx, Ly = vy - ry;
    double Lr = sqrt(Lx * Lx + Ly * Ly);
    double rL = 1.0 / sqrt(Lx * Lx + Ly * Ly);
    Lx *= rL;
    Ly *= rL;
    long maxBatch = (long)ceil(sqrt((double)((int64_t)NX * NX + (int64_t)NY * NY)) /
                               (DQ * (double)p->nwt));
    long kmax = maxBatch * (long)p->nwt;
    double s1 = 0.0, s2 = 0.0;
    int64_t n = 0;
    for (long k = 0; k < kmax; k++) {
        double qr = DQ * (double)k;
        if (!(qr <= Lr)) break; /* also ends on NaN, as the reference does */
        double v1, v2;
        tex_bilinear(a1, a2, NX, NY, rx + Lx * qr, ry + Ly * qr, &v1, &v2);
        s1 += v1;
        s2 += v2;
        n++;
    }
    *A1 = s1 * DQ;
    *A2 = s2 * DQ;
    return n;
}

typedef struct {
    double qnow, dqnow;
} coarse_bin;

/* The cross-section table path (xrdt_oracle_forward_tables): the coherent
 * term from the u8 table S1 instead of the fine-q pattern sum, and the
 * lookups of both tables by nearest bin or bilinear. */
typedef struct {
    const unsigned char *S1u8;
    int bilinear;
} oracle_tables;

/* Bilinear value of a u8 table [nq, na] (index q + a*nq) at grid coordinates
 * (tq, ta), the grid points being the table's entries
 * (XSection_builder.m:121-125: q_min + i (q_max - q_min)/(NQ - 1)); clamped
 * to the table. */
static double table_bilinear(const unsigned char *S, int nq, int na, double tq, double ta)
{
    if (!(tq > 0.0)) tq = 0.0;
    if (tq > (double)(nq - 1)) tq = (double)(nq - 1);
    if (!(ta > 0.0)) ta = 0.0;
    if (ta > (double)(na - 1)) ta = (double)(na - 1);
    int i = (int)floor(tq), j = (int)floor(ta);
    if (i > nq - 2) i = nq - 2;
    if (j > na - 2) j = na - 2;
    if (i < 0) i = 0;
    if (j < 0) j = 0;
    const double f = tq - (double)i, g = ta - (double)j;
    const double s00 = S[i + j * nq], s10 = S[(i + 1) + j * nq];
    const double s01 = S[i + (j + 1) * nq], s11 = S[(i + 1) + (j + 1) * nq];
    return (1.0 - g) * ((1.0 - f) * s00 + f * s10) + g * ((1.0 - f) * s01 + f * s11);
}

/* One block of integrate_diffraction.cu:9-409 in FP64. */
static void forward_one_ray(const xrdt_problem *p, const float *spectrum, const float *Ifine,
                            const int32_t *seg, const float *a1, const float *a2,
                            const unsigned char *S2u8, const coarse_bin *cb,
                            double q_min, double q_max, double a_min, double a_max,
                            int64_t ray, double *N_out, double *C_out, double *A_row,
                            double *Av_row, const double *xv, double *yv, double *gv, double wgt,
                            int32_t *dec_walk, int32_t *dec_nq, int32_t *dec_na, const oracle_tables *tab)
{
    /* dec_*: where set, the integer decisions of every non-empty voxel in loop
     * order: walk[v] = (detector-side samples, its edge, source-side samples,
     * its edge), nq[v][j] for source bin nrg_src_min + j, na[v]. */
    int64_t dec_v = 0;
    /* Per-voxel mode (xv or gv set): only the coarse-q model row matters. */
    const int want_nc = !(xv || gv);
    const int NX = p->nx, NY = p->ny;
    const int SRC = p->n_src, COL = p->n_col, DET = p->n_col * p->n_row;
    const int NWT = p->nwt, NQF = p->nqf, MAT = p->n_mat, NQ = p->nq, NA = p->na;
    const int src = (int)(ray % SRC);
    const int det = (int)((ray / SRC) % DET);
    const int nrg = (int)(ray / ((int64_t)SRC * DET));
    const int col = det % COL;             /* integrate_diffraction.cu:39-40 */
    const int row = (det - col) / COL;

    int nrg_src_min, nrg_src_max;          /* :56-57 */
    xrdt_oracle_src_nrg_range(p, nrg, &nrg_src_min, &nrg_src_max);

    /* Scanner geometry, :81-128. */
    double phi = ((double)src / (double)SRC) * p->src_arc + p->src_phi0;
    double sphi = sin(phi), cphi = cos(phi);
    double Rsrc_x = p->cx + p->r_src * sphi;
    double Rsrc_y = p->cy - p->r_src * cphi;
    double Rsrc_z = 0.0;
    double rdet = ((double)col - (double)COL / 2.0 + 0.5) * p->col_pitch;
    double Rdet_x = p->cx - p->r_det * sphi + rdet * cphi;
    double Rdet_y = p->cy + p->r_det * cphi + rdet * sphi;
    double Rdet_z = p->z0 + (double)row * p->row_pitch;
    double ndet_x = sphi, ndet_y = -cphi, ndet_z = 0.0;
    double sta = sin(p->target_angle), cta = cos(p->target_angle);
    double nsrc_x = -sphi * sta, nsrc_y = cphi * sta, nsrc_z = -cta;
    double geomphi = p->wedge_angle;
    double geomAdet = p->col_pitch * p->row_pitch;
    double geomdvox = p->vox_side;
    double tan_half = tan(geomphi / 2.0), tan_full = tan(geomphi);
    double nsrc_xy = sqrt(nsrc_x * nsrc_x + nsrc_y * nsrc_y);

    /* Energy grids, :138-142. */
    double dEs = (p->e_src_max - p->e_src_min) / (double)p->nrg_src;
    double dEd = (p->e_det_max - p->e_det_min) / (double)p->nrg_det;
    double Edet1 = p->e_det_min + (double)nrg * dEd;
    double Edet2 = p->e_det_min + (double)(nrg + 1) * dEd;

    double da = (a_max - a_min) / (double)NA; /* :167-168 */
    double dq = (q_max - q_min) / (double)NQ;
    double dq_grid = (q_max - q_min) / (double)(NQ - 1);  /* the tables' grid points */
    double da_grid = (a_max - a_min) / (double)(NA - 1);
    double dq_fine = (p->q_hi - p->q_lo) / (double)NQF; /* Forward_XRD.cu:42 */
    const int quirk_stale = (p->quirks & XRDT_QUIRK_STALE_VOXEL_A) != 0;

    double Nnow = 0.0, Cnow = 0.0;
    double Rvox_x = 0.0, Rvox_y = 0.0; /* stale coordinates start at (0,0) */

    for (int nx = 0; nx < NX; nx++) {          /* :173-174 */
        for (int ny = 0; ny < NY; ny++) {
            int matID = seg[nx + ny * NX] - 1;  /* :177 */
            if (matID < 0) continue;
            double cur_x = ((double)nx + 0.5) * geomdvox; /* :192-193 */
            double cur_y = ((double)ny + 0.5) * geomdvox;

            /* (a1,a2) at the voxel for the Compton table, :181-189. */
            double a1now, a2now;
            if (quirk_stale)
                tex_bilinear(a1, a2, NX, NY, Rvox_x, Rvox_y, &a1now, &a2now);
            else
                tex_bilinear(a1, a2, NX, NY, cur_x, cur_y, &a1now, &a2now);
            double log2aratio = log2(fabs(a1now / a2now));
            int na = cuda_floor_int((log2aratio - a_min) / da);
            if (na < 0) na = 0;
            else if (na >= NA) na = NA - 1;
            const double ta = (log2aratio - a_min) / da_grid;   /* bilinear lookups */

            Rvox_x = cur_x;
            Rvox_y = cur_y;

            /* Scattering geometry, :196-255. */
            double ax = Rvox_x - Rsrc_x;
            double ay = Rvox_y - Rsrc_y;
            double Rvox_z = -(ax * nsrc_x + ay * nsrc_y) / nsrc_xy * tan_half;
            double Hvox = (ax * nsrc_x + ay * nsrc_y) / nsrc_xy * tan_full;
            double az = Rvox_z - Rsrc_z;
            double bx = Rdet_x - Rvox_x;
            double by = Rdet_y - Rvox_y;
            double bz = Rdet_z - Rvox_z;
            double ab = ax * bx + ay * by + az * bz;
            double anorm2 = ax * ax + ay * ay + az * az;
            double bnorm2 = bx * bx + by * by + bz * bz;
            double costheta = ab * (1.0 / sqrt(anorm2)) * (1.0 / sqrt(bnorm2));
            double sinthetahalf = sqrt(fabs(1.0 - costheta) / 2.0);
            double Sx = bx - ab * ax / anorm2, Sy = by - ab * ay / anorm2, Sz = bz - ab * az / anorm2;
            double Dx = -ax + ab * bx / bnorm2, Dy = -ay + ab * by / bnorm2, Dz = -az + ab * bz / bnorm2;
            double Vx = -(Sx + Dx), Vy = -(Sy + Dy), Vz = -(Sz + Dz);
            double Dndet = Dx * ndet_x + Dy * ndet_y + Dz * ndet_z;
            double Snsrc = Sx * nsrc_x + Sy * nsrc_y + Sz * nsrc_z;
            double dD2 = (Dx * Dx + Dy * Dy + Dz * Dz - Dndet * Dndet) * geomAdet / 12.0;
            double vV2 = (geomdvox * geomdvox * (Vx * Vx + Vy * Vy) + Hvox * Hvox * Vz * Vz) / 12.0;
            double sS2 = (Sx * Sx + Sy * Sy + Sz * Sz - Snsrc * Snsrc) * p->focal_spot * p->focal_spot / 12.0;
            double Rdotn = -sphi * ax + cphi * ay;
            double cospsi = Rdotn * (1.0 / sqrt(ax * ax + ay * ay));
            double geom_src2vox = cospsi * (1.0 / sqrt(anorm2)) * tan_full;
            double geom_vox2det = -(ndet_x * bx + ndet_y * by) * (1.0 / sqrt(bnorm2 * bnorm2 * bnorm2));
            double Rayleigh_factor = (1.0 + costheta * costheta) / 2.0;
            double geomproduct = geom_src2vox * geom_vox2det;

            /* :259-260 -- the detector-side integral is named A_src2vox and
             * the source-side one A_vox2det; kept as written. */
            double As2v_x, As2v_y, Av2d_x, Av2d_y;
            int edge_d, edge_s;
            int64_t n_d = attenuator_edge(p, a1, a2, Rdet_x, Rdet_y, Rvox_x, Rvox_y, &As2v_x, &As2v_y, &edge_d);
            int64_t n_s = attenuator_edge(p, a1, a2, Rsrc_x, Rsrc_y, Rvox_x, Rvox_y, &Av2d_x, &Av2d_y, &edge_s);
            if (dec_walk) {
                int32_t *w4 = dec_walk + 4 * dec_v;
                w4[0] = (int32_t)n_d;
                w4[1] = edge_d;
                w4[2] = (int32_t)n_s;
                w4[3] = edge_s;
            }
            if (dec_na) dec_na[dec_v] = na;

            for (int nrg_src = nrg_src_min; nrg_src <= nrg_src_max; nrg_src++) { /* :266 */
                double Esrc1 = p->e_src_min + (double)nrg_src * dEs;
                double Esrc2 = p->e_src_min + (double)(nrg_src + 1) * dEs;
                double Esrc = 0.5 * (Esrc1 + Esrc2);
                double ein = Esrc / p->mec2;
                double RF = (double)spectrum[nrg_src + (int64_t)nrg * p->nrg_src]; /* :61,:281 */
                double wvt = 2.0 * Esrc / p->hbarc * sinthetahalf;                   /* :284 */
                double sigma_wvt2 =                                                   /* :287-288 */
                    (2.0 * sinthetahalf / p->hbarc) * (2.0 * sinthetahalf / p->hbarc) * dEs * dEs / 12.0 +
                    (Esrc / p->hbarc) * (Esrc / p->hbarc) * (sS2 + vV2 + dD2) /
                        (2.0 * sinthetahalf) / (2.0 * sinthetahalf) / anorm2 / bnorm2;
                double f1 = ein * ein * ein;
                double f2 = p->kn0 + p->kn1 * ein + p->kn2 * ein * ein;
                double Pin = exp(-(As2v_x / f1 + As2v_y / f2));  /* :295-296 */
                double Pout = exp(-(Av2d_x / f1 + Av2d_y / f2));

                /* Coherent term from the S1 table instead (the reference's
                 * commented-out kernel, integrate_diffraction.cu:716-719 with
                 * the bin of :701-707): wvt = ein sin(theta/2) on the log2
                 * axis of the tables (XSection_builder.m:106). */
                if (want_nc && tab) {
                    double wc = ein * sinthetahalf;
                    double s1;
                    if (tab->bilinear) {
                        s1 = table_bilinear(tab->S1u8, NQ, NA, (log2(wc) - q_min) / dq_grid, ta);
                    } else {
                        int nqc = cuda_floor_int((log2(wc) - q_min) / dq);
                        if (nqc < 0) nqc = 0;
                        else if (nqc >= NQ) nqc = NQ - 1;
                        s1 = (double)tab->S1u8[nqc + na * NQ];
                    }
                    Nnow += Pin * Pout * RF * geomproduct * Rayleigh_factor * a2now * s1;
                }
                /* Fine-q Rayleigh sum, :299-308 (all NQF bins). */
                const float *Im = (want_nc && !tab) ? Ifine + (int64_t)matID * NQF : NULL;
                for (int qf = 0; Im && qf < NQF; qf++) {
                    double qaxis_fine = p->q_lo + dq_fine * (0.5 + (double)qf);
                    double Rq = RF * exp(-(wvt - qaxis_fine) * (wvt - qaxis_fine) / (2.0 * sigma_wvt2)) *
                                p->rsqrt2pi / sqrt(sigma_wvt2) * dq_fine;
                    Nnow += Pin * Pout * geomproduct * Rq * (double)Im[qf] * Rayleigh_factor;
                }
                /* Coarse-q model row, :311-315. */
                if (A_row || Av_row || xv || gv) {
                    const int64_t vrow = ((int64_t)nx + (int64_t)ny * NX) * NWT;
                    for (int k = 0; k < NWT; k++) {
                        double d = wvt - cb[k].qnow;
                        double Rq = RF * exp(-d * d / (2.0 * sigma_wvt2)) * p->rsqrt2pi /
                                    sqrt(sigma_wvt2) * cb[k].dqnow;
                        double t = Pin * Pout * geomproduct * Rq * Rayleigh_factor;
                        if (A_row) A_row[(int64_t)matID * NWT + k] += t;
                        if (Av_row) Av_row[vrow + k] += t;
                        if (xv) *yv += t * xv[vrow + k];
                        if (gv) gv[vrow + k] += wgt * t;
                    }
                }
                if (!want_nc) continue;
                /* Compton, :318-356. */
                double eratio = 1.0 + ein * (1.0 - costheta);
                double eout = ein / eratio;
                double Eout1 = Esrc1 / eratio, Eout2 = Esrc2 / eratio;
                double channel_match = fmax(0.0, fmin(Eout2, Edet2) - fmax(Eout1, Edet1)) / (Eout2 - Eout1);
                double w = ein * sinthetahalf;
                double log2wvt = log2(w * sqrt(eratio + w * w) / eratio);
                int nq = cuda_floor_int((log2wvt - q_min) / dq);
                if (nq < 0) nq = 0;
                else if (nq >= NQ) nq = NQ - 1;
                if (dec_nq) dec_nq[dec_v * (2 * p->dnrg + 1) + (nrg_src - nrg_src_min)] = nq;
                f1 = eout * eout * eout;
                f2 = p->kn0 + p->kn1 * eout + p->kn2 * eout * eout;
                double Pout_c = exp(-(Av2d_x / f1 + Av2d_y / f2));
                double Compton_factor = eratio * eratio * (eratio + 1.0 / eratio - 1.0 + costheta * costheta) / 2.0;
                const double s2 = (tab && tab->bilinear)
                                      ? table_bilinear(S2u8, NQ, NA, (log2wvt - q_min) / dq_grid, ta)
                                      : (double)S2u8[nq + na * NQ];
                Cnow += channel_match * Pin * Pout_c * RF * geomproduct * Compton_factor * a2now * s2;
            }
            dec_v++;
        }
    }
    *N_out = Nnow;
    *C_out = Cnow;
}

int32_t xrdt_oracle_forward_rays(const xrdt_problem *p,
                                 const float *spectrum, const float *Ifine,
                                 const int32_t *seg, const float *a1, const float *a2,
                                 const float *S2,
                                 float q_min, float q_max, float a_min, float a_max,
                                 const int64_t *rays, int64_t n_rays,
                                 double *N_out, double *C_out, double *A_out,
                                 double *Av_out, int32_t n_threads)
{
    const int64_t nvox = (int64_t)p->nx * p->ny;
    for (int64_t i = 0; i < nvox; i++)
        if (seg[i] > p->n_mat) return -1;

    /* S2 quantised to u8 by floor and clamp, integrate_diffraction.cu:66-74. */
    const int64_t nS = (int64_t)p->nq * p->na;
    unsigned char *S2u8 = (unsigned char *)malloc((size_t)nS);
    for (int64_t i = 0; i < nS; i++) {
        int s = cuda_floor_int((double)S2[i]);
        if (s < 0) s = 0;
        else if (s > 255) s = 255;
        S2u8[i] = (unsigned char)s;
    }
    coarse_bin *cb = (coarse_bin *)malloc(sizeof(coarse_bin) * (size_t)p->nwt);
    for (int k = 0; k < p->nwt; k++) xrdt_oracle_wvt_value(p, k, &cb[k].qnow, &cb[k].dqnow);

    const int64_t arow = (int64_t)p->n_mat * p->nwt;
    const int64_t avrow = nvox * p->nwt;
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int64_t i = 0; i < n_rays; i++) {
        double *A_row = A_out ? A_out + i * arow : NULL;
        double *Av_row = Av_out ? Av_out + i * avrow : NULL;
        if (A_row) memset(A_row, 0, sizeof(double) * (size_t)arow);
        if (Av_row) memset(Av_row, 0, sizeof(double) * (size_t)avrow);
        forward_one_ray(p, spectrum, Ifine, seg, a1, a2, S2u8, cb,
                        (double)q_min, (double)q_max, (double)a_min, (double)a_max,
                        rays[i], &N_out[i], &C_out[i], A_row, Av_row, NULL, NULL, NULL, 0.0, NULL, NULL, NULL, NULL);
    }
    free(cb);
    free(S2u8);
    return 0;
}

/* The cross-section table path for the listed rays: Nphotons with the
 * coherent term of the S1 table (nearest bin, or bilinear when bilinear != 0),
 * Cphotons as xrdt_oracle_forward_rays (bilinear S2 lookups when bilinear). */
int32_t xrdt_oracle_forward_tables(const xrdt_problem *p, const float *spectrum, const int32_t *seg,
                                   const float *a1, const float *a2, const float *S1, const float *S2,
                                   float q_min, float q_max, float a_min, float a_max, int32_t bilinear,
                                   const int64_t *rays, int64_t n_rays, double *N_out, double *C_out,
                                   int32_t n_threads)
{
    const int64_t nvox = (int64_t)p->nx * p->ny;
    for (int64_t i = 0; i < nvox; i++)
        if (seg[i] > p->n_mat) return -1;
    if (p->nq < 2 || p->na < 2) return -2;
    const int64_t nS = (int64_t)p->nq * p->na;
    unsigned char *u8 = (unsigned char *)malloc(2 * (size_t)nS);
    for (int64_t i = 0; i < 2 * nS; i++) {
        int s = cuda_floor_int((double)(i < nS ? S1[i] : S2[i - nS]));
        if (s < 0) s = 0;
        else if (s > 255) s = 255;
        u8[i] = (unsigned char)s;
    }
    oracle_tables tab = {u8, bilinear ? 1 : 0};
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int64_t i = 0; i < n_rays; i++)
        forward_one_ray(p, spectrum, NULL, seg, a1, a2, u8 + nS, NULL, (double)q_min, (double)q_max,
                        (double)a_min, (double)a_max, rays[i], &N_out[i], &C_out[i], NULL, NULL, NULL, NULL,
                        NULL, 0.0, NULL, NULL, NULL, &tab);
    free(u8);
    return 0;
}

/* The integer decisions of forward_one_ray for the listed rays (every
 * non-empty voxel in loop order): the source-energy window, the ROI edge and
 * sample count of both line integrals, the Compton table bin per window
 * energy and column per voxel, and the u8 table.  walk [n][nv][4], nq
 * [n][nv][2*dnrg+1], na [nv], win [n][2], s2u8 [nq*na]. */
int32_t xrdt_oracle_decisions(const xrdt_problem *p, const float *spectrum, const float *Ifine,
                              const int32_t *seg, const float *a1, const float *a2, const float *S2,
                              float q_min, float q_max, float a_min, float a_max,
                              const int64_t *rays, int64_t n_rays, int32_t *win, int32_t *walk,
                              int32_t *na, int32_t *nq, uint8_t *s2u8, int32_t n_threads)
{
    const int64_t nvox = (int64_t)p->nx * p->ny;
    int64_t nv = 0;
    for (int64_t i = 0; i < nvox; i++) {
        if (seg[i] > p->n_mat) return -1;
        if (seg[i] > 0) nv++;
    }
    const int64_t nS = (int64_t)p->nq * p->na;
    for (int64_t i = 0; i < nS; i++) {
        int s = cuda_floor_int((double)S2[i]);
        if (s < 0) s = 0;
        else if (s > 255) s = 255;
        s2u8[i] = (uint8_t)s;
    }
    coarse_bin *cb = (coarse_bin *)malloc(sizeof(coarse_bin) * (size_t)p->nwt);
    for (int k = 0; k < p->nwt; k++) xrdt_oracle_wvt_value(p, k, &cb[k].qnow, &cb[k].dqnow);
    const int W = 2 * p->dnrg + 1;
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int64_t i = 0; i < n_rays; i++) {
        const int nrg = (int)(rays[i] / ((int64_t)p->n_src * p->n_col * p->n_row));
        int lo, hi;
        xrdt_oracle_src_nrg_range(p, nrg, &lo, &hi);
        win[2 * i] = lo;
        win[2 * i + 1] = hi;
        double nn, cc;
        forward_one_ray(p, spectrum, Ifine, seg, a1, a2, s2u8, cb, (double)q_min, (double)q_max,
                        (double)a_min, (double)a_max, rays[i], &nn, &cc, NULL, NULL, NULL, NULL, NULL, 0.0,
                        walk + i * nv * 4, nq + i * nv * W, i == 0 ? na : NULL, NULL);
    }
    free(cb);
    return 0;
}

int32_t xrdt_oracle_vox_rays(const xrdt_problem *p, const float *spectrum, const int32_t *seg,
                             const float *a1, const float *a2, const double *x, const double *w,
                             const int64_t *rays, int64_t n_rays, double *y_out, double *g_out,
                             int32_t n_threads)
{
    const int64_t nvox = (int64_t)p->nx * p->ny;
    for (int64_t i = 0; i < nvox; i++)
        if (seg[i] > p->n_mat) return -1;
    if ((x == NULL) != (y_out == NULL) || (w == NULL) != (g_out == NULL)) return -2;
    coarse_bin *cb = (coarse_bin *)malloc(sizeof(coarse_bin) * (size_t)p->nwt);
    for (int k = 0; k < p->nwt; k++) xrdt_oracle_wvt_value(p, k, &cb[k].qnow, &cb[k].dqnow);
    const int64_t ng = nvox * p->nwt;
    int nt = 1;
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
    nt = omp_get_max_threads();
#endif
    /* one adjoint accumulator per thread, summed in thread order */
    double *gpriv = g_out ? (double *)calloc((size_t)nt * (size_t)ng, sizeof(double)) : NULL;
    if (g_out && !gpriv) {
        free(cb);
        return -3;
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int64_t i = 0; i < n_rays; i++) {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
        double nn = 0.0, cc = 0.0, yy = 0.0;
        /* one pass per ray: the forward sum and the adjoint accumulation */
        forward_one_ray(p, spectrum, NULL, seg, a1, a2, NULL, cb, 0.0, 1.0, 0.0, 1.0, rays[i], &nn, &cc,
                        NULL, NULL, x, &yy, gpriv ? gpriv + (size_t)t * (size_t)ng : NULL, w ? w[i] : 0.0,
                        NULL, NULL, NULL, NULL);
        if (y_out) y_out[i] = yy;
    }
    if (g_out) {
        for (int64_t j = 0; j < ng; j++) {
            double s = 0.0;
            for (int t = 0; t < nt; t++) s += gpriv[(size_t)t * (size_t)ng + (size_t)j];
            g_out[j] = s;
        }
        free(gpriv);
    }
    free(cb);
    return 0;
}

/* Transmission through the map along the source -> pixel chord (a project
 * definition; the reference only declares these outputs): the segment is
 * clipped to [0,NX] x [0,NY] by slabs, sampled every DQ from the entry point
 * for k*DQ <= chord length (k below maxBatch*NWT), bilinear as tex2D, and
 * the energy channels weighted as in integrate_diffraction.cu:266-296. */
static void ct_one_ray(const xrdt_problem *p, const float *spectrum, const float *a1, const float *a2, int64_t ray,
                       double *T, double *G0)
{
    const int NX = p->nx, NY = p->ny, SRC = p->n_src, COL = p->n_col, DET = p->n_col * p->n_row;
    const int src = (int)(ray % SRC), det = (int)((ray / SRC) % DET), nrg = (int)(ray / ((int64_t)SRC * DET));
    const int col = det % COL, row = (det - col) / COL;
    (void)row;
    const double phi = ((double)src / (double)SRC) * p->src_arc + p->src_phi0;
    const double sphi = sin(phi), cphi = cos(phi);
    const double sx = p->cx + p->r_src * sphi, sy = p->cy - p->r_src * cphi;
    const double rdet = ((double)col - (double)COL / 2.0 + 0.5) * p->col_pitch;
    const double dx = p->cx - p->r_det * sphi + rdet * cphi, dy = p->cy + p->r_det * cphi + rdet * sphi;
    const double ex = dx - sx, ey = dy - sy;
    double t0 = 0.0, t1 = 1.0;
    const double lo[2] = {0.0, 0.0}, hi[2] = {(double)NX, (double)NY};
    const double o[2] = {sx, sy}, d[2] = {ex, ey};
    for (int a = 0; a < 2; a++) {
        if (d[a] == 0.0) {
            if (o[a] < lo[a] || o[a] > hi[a]) t1 = -1.0;
            continue;
        }
        double ta = (lo[a] - o[a]) / d[a], tb = (hi[a] - o[a]) / d[a];
        if (ta > tb) {
            const double t = ta;
            ta = tb;
            tb = t;
        }
        if (ta > t0) t0 = ta;
        if (tb < t1) t1 = tb;
    }
    double A1 = 0.0, A2 = 0.0;
    if (t1 > t0) {
        const double DQ = p->dq_step;
        const double len = sqrt(ex * ex + ey * ey);
        const double rx = sx + t0 * ex, ry = sy + t0 * ey;
        const double L = (t1 - t0) * len;
        long long k = (long long)floor(L / DQ);
        while (DQ * (double)(k + 1) <= L) k++;
        while (k >= 0 && !(DQ * (double)k <= L)) k--;
        long long n = k + 1;
        const long maxBatch = (long)ceil(sqrt((double)((int64_t)NX * NX + (int64_t)NY * NY)) / (DQ * (double)p->nwt));
        if (n > maxBatch * (long)p->nwt) n = maxBatch * (long)p->nwt;
        const double ux = ex / len, uy = ey / len;
        double s1 = 0.0, s2 = 0.0;
        for (long long j = 0; j < n; j++) {
            double v1, v2;
            const double qr = DQ * (double)j;
            tex_bilinear(a1, a2, NX, NY, rx + ux * qr, ry + uy * qr, &v1, &v2);
            s1 += v1;
            s2 += v2;
        }
        A1 = s1 * DQ;
        A2 = s2 * DQ;
    }
    int lo_e, hi_e;
    xrdt_oracle_src_nrg_range(p, nrg, &lo_e, &hi_e);
    const double dEs = (p->e_src_max - p->e_src_min) / (double)p->nrg_src;
    double t = 0.0, g = 0.0;
    for (int e = lo_e; e <= hi_e; e++) {
        const double Esrc1 = p->e_src_min + (double)e * dEs, Esrc2 = p->e_src_min + (double)(e + 1) * dEs;
        const double ein = 0.5 * (Esrc1 + Esrc2) / p->mec2;
        const double f1 = ein * ein * ein, f2 = p->kn0 + p->kn1 * ein + p->kn2 * ein * ein;
        const double RF = (double)spectrum[e + (int64_t)nrg * p->nrg_src];
        t += RF * exp(-(A1 / f1 + A2 / f2));
        g += RF;
    }
    *T = t;
    *G0 = g;
}

int32_t xrdt_oracle_ct_rays(const xrdt_problem *p, const float *spectrum, const float *a1, const float *a2,
                            const int64_t *rays, int64_t n_rays, double *T_out, double *G_out, int32_t n_threads)
{
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (int64_t i = 0; i < n_rays; i++) ct_one_ray(p, spectrum, a1, a2, rays[i], &T_out[i], &G_out[i]);
    return 0;
}
