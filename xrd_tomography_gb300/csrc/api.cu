// api.cu -- the C ABI of libxrdt.so (include/xrdt.h).
//
// Host side of the drop-in for mexFunction (Forward_XRD.cu:76-301): input
// validation, staging of host arrays, the per-call tables that the reference
// derives inside every block, and the kernel sequence.  The reference checks
// no CUDA error (Forward_XRD.cu:210-259); here every call is checked and
// reported through xrdt_status and xrdt_last_error.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "ctx.h"

using namespace xrdt;

namespace xrdt {

std::string fmt(const char *f, ...)
{
    char b[512];
    va_list ap;
    va_start(ap, f);
    vsnprintf(b, sizeof b, f, ap);
    va_end(ap);
    return std::string(b);
}

} // namespace xrdt

namespace {

enum Slot {
    S_SPEC, S_IFINE, S_SEG, S_A1, S_A2, S_S2, S_N, S_C, S_A,
    S_CELLS, S_VXY, S_VMAT, S_VNA, S_VA2, S_CNT, S_ASRC, S_S2U8,
    S_SRCG, S_ENERGY, S_RFWIN, S_OFFS, S_WINLO, S_WINN, S_FINEQ, S_COARSEQ, S_COARSEQD,
    S_RAYS, S_PAIRS, S_NC, S_CC, S_AC,
    S_MA, S_MY, S_MC, S_MX, S_MPART, S_MSENS, S_BC, S_BB, S_BI, S_ERR, S_WALK,
    S_SPFINE, S_SPSRC, S_SPDET, S_SPOUT, S_DWALK, S_DNQ,
    S_S1, S_S1U8, S_VTA,
    S_COUNT
};

int fail(xrdt_ctx *c, int status, const std::string &msg)
{
    if (c) c->err = msg;
    return status;
}

void fold_pending(xrdt_ctx *ctx)
{
    for (auto &p : ctx->pending) {
        float ms = 0.f;
        if (cudaEventSynchronize(p.b) == cudaSuccess && cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            ctx->prof_ms[p.kernel] += ms;
            ctx->prof_launches[p.kernel] += 1;
        }
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    ctx->pending.clear();
    cudaGetLastError();
}

#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return fail(ctx, XRDT_ERR_CUDA, fmt("%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                                               __FILE__, __LINE__));                      \
    } while (0)

int get_buf(xrdt_ctx *ctx, int slot, size_t bytes, void **out)
{
    if ((int)ctx->buf.size() < S_COUNT) {
        ctx->buf.assign(S_COUNT, nullptr);
        ctx->cap.assign(S_COUNT, 0);
    }
    if (bytes == 0) bytes = 16;
    if (ctx->cap[slot] < bytes) {
        if (ctx->buf[slot]) {
            cudaStreamSynchronize(ctx->stream);
            cudaFree(ctx->buf[slot]);
            ctx->buf[slot] = nullptr;
            ctx->cap[slot] = 0;
        }
        void *p = nullptr;
        if (test_alloc_fails()) return fail(ctx, XRDT_ERR_ALLOC, fmt("cudaMalloc(%zu bytes): failure injected", bytes));
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(ctx, XRDT_ERR_ALLOC, fmt("cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e)));
        }
        ctx->buf[slot] = p;
        ctx->cap[slot] = bytes;
    }
    *out = ctx->buf[slot];
    return XRDT_OK;
}

// Device view of an input: the pointer itself, or a staged copy.
int stage_in(xrdt_ctx *ctx, int slot, const void *p, size_t bytes, const void **dev)
{
    if (is_device_ptr(p)) {
        *dev = p;
        return XRDT_OK;
    }
    void *d;
    int rc = get_buf(ctx, slot, bytes, &d);
    if (rc) return rc;
    if (bytes) CK(cudaMemcpyAsync(d, p, bytes, cudaMemcpyHostToDevice, ctx->stream));
    *dev = d;
    return XRDT_OK;
}

bool finite_all(const xrdt_problem *p)
{
    const double v[] = {p->e_src_min, p->e_src_max, p->e_det_min, p->e_det_max, p->q_lo, p->q_hi,
                        p->dq0, p->hbarc, p->mec2, p->kn0, p->kn1, p->kn2, p->rsqrt2pi, p->dq_step,
                        p->cx, p->cy, p->r_src, p->r_det, p->src_arc, p->src_phi0, p->col_pitch,
                        p->row_pitch, p->z0, p->focal_spot, p->target_angle, p->wedge_angle, p->vox_side};
    for (double x : v)
        if (!std::isfinite(x)) return false;
    return true;
}

// Positions of the sources and detector pixels, as integrate_diffraction.cu:93-109.
void src_geom(const xrdt_problem *p, int src, SrcGeom *g)
{
    const double phi = ((double)src / (double)p->n_src) * p->src_arc + p->src_phi0;
    g->sphi = sin(phi);
    g->cphi = cos(phi);
    g->Rsrc_x = p->cx + p->r_src * g->sphi;
    g->Rsrc_y = p->cy - p->r_src * g->cphi;
}

bool inside_roi(const xrdt_problem *p, double x, double y)
{
    const double m = 1e-3;  // a margin of a thousandth of a voxel
    return x > -m && x < p->nx * p->vox_side + m && y > -m && y < p->ny * p->vox_side + m;
}

} // namespace

namespace xrdt {

int build_dev_problem(const xrdt_problem *p, float q_min, float q_max, float a_min, float a_max,
                      DevProblem *d, std::string *err)
{
    memset(d, 0, sizeof *d);
    d->nx = p->nx;
    d->ny = p->ny;
    d->n_src = p->n_src;
    d->n_col = p->n_col;
    d->n_row = p->n_row;
    d->n_det = p->n_col * p->n_row;
    d->nrg_src = p->nrg_src;
    d->nrg_det = p->nrg_det;
    d->dnrg = p->dnrg;
    d->nwt = p->nwt;
    d->nqf = p->nqf;
    d->n_mat = p->n_mat;
    d->nq = p->nq;
    d->na = p->na;
    d->quirk_stale = (p->quirks & XRDT_QUIRK_STALE_VOXEL_A) ? 1 : 0;
    d->dEs = (p->e_src_max - p->e_src_min) / (double)p->nrg_src;
    d->dEd = (p->e_det_max - p->e_det_min) / (double)p->nrg_det;
    d->e_src_min = p->e_src_min;
    d->e_det_min = p->e_det_min;
    d->q_lo = p->q_lo;
    d->q_hi = p->q_hi;
    d->dq0 = p->dq0;
    d->dq_fine = (p->q_hi - p->q_lo) / (double)p->nqf;
    d->hbarc = p->hbarc;
    d->mec2 = p->mec2;
    d->kn0 = p->kn0;
    d->kn1 = p->kn1;
    d->kn2 = p->kn2;
    d->rsqrt2pi = p->rsqrt2pi;
    d->DQ = p->dq_step;
    d->cx = p->cx;
    d->cy = p->cy;
    d->r_src = p->r_src;
    d->r_det = p->r_det;
    d->col_pitch = p->col_pitch;
    d->row_pitch = p->row_pitch;
    d->z0 = p->z0;
    d->focal = p->focal_spot;
    d->geomAdet = p->col_pitch * p->row_pitch;
    d->vox = p->vox_side;
    d->tan_half = tan(p->wedge_angle / 2.0);
    d->tan_full = tan(p->wedge_angle);
    d->sta = sin(p->target_angle);
    d->cta = cos(p->target_angle);
    d->q_min = q_min;
    d->q_max = q_max;
    d->a_min = a_min;
    d->a_max = a_max;
    d->dq_tab = ((double)q_max - (double)q_min) / (double)p->nq;
    d->da_tab = ((double)a_max - (double)a_min) / (double)p->na;
    d->dq_grid = p->nq > 1 ? ((double)q_max - (double)q_min) / (double)(p->nq - 1) : 0.0;
    d->da_grid = p->na > 1 ? ((double)a_max - (double)a_min) / (double)(p->na - 1) : 0.0;
    // maxBatch of integrate_diffraction.cu:160-161, times the block size
    const double diag = sqrt((double)((int64_t)p->nx * p->nx + (int64_t)p->ny * p->ny));
    d->kmax = (long long)ceil(diag / (p->dq_step * (double)p->nwt)) * (long long)p->nwt;
    const int same = (p->nrg_src == p->nrg_det && p->e_src_min == p->e_det_min && p->e_src_max == p->e_det_max);
    int lo_all = p->nrg_src, hi_all = -1;
    for (int n = 0; n < p->nrg_det; n++) {
        int lo, hi;
        src_nrg_range(*d, same, n, &lo, &hi);
        if (lo < lo_all) lo_all = lo;
        if (hi > hi_all) hi_all = hi;
    }
    d->e_lo = lo_all;
    d->e_hi = hi_all;
    (void)err;
    return XRDT_OK;
}

F32Consts make_f32_consts(const DevProblem &P)
{
    F32Consts c;
    c.vox = (float)P.vox;
    c.DQ = (float)P.DQ;
    c.inv_DQ = (float)(1.0 / P.DQ);
    c.nxf = (float)P.nx;
    c.nyf = (float)P.ny;
    c.rsqrt2pi = (float)P.rsqrt2pi;
    c.dqf_hi = (float)P.dq_fine;
    c.dqf_lo = (float)(P.dq_fine - (double)c.dqf_hi);
    c.inv_dqf = (float)(1.0 / P.dq_fine);
    c.q_lo = (float)P.q_lo;
    c.q_hi = (float)P.q_hi;
    c.kn0 = (float)P.kn0;
    c.kn1 = (float)P.kn1;
    c.kn2 = (float)P.kn2;
    c.edmin = (float)P.e_det_min;
    c.inv_dEd = (float)(1.0 / P.dEd);
    c.inv_dEs = (float)(1.0 / P.dEs);
    c.dEd = (float)P.dEd;
    c.dEs = (float)P.dEs;
    c.qmin_t = (float)P.q_min;
    c.inv_dqt = P.dq_tab > 0 ? (float)(1.0 / P.dq_tab) : 0.f;
    c.inv_dqg = P.dq_grid > 0 ? (float)(1.0 / P.dq_grid) : 0.f;
    const double NWT = (double)P.nwt;
    c.qpar_b = (float)P.dq0;
    c.qpar_a = (float)((P.q_hi - P.q_lo - P.dq0 * NWT) / (NWT * NWT));
    return c;
}

void build_host_tables(const xrdt_problem *p, const DevProblem &P, const float *spec_h, HostTables *t)
{
    const int W = 2 * p->dnrg + 1;
    // energy rows
    t->energy.resize(p->nrg_src);
    for (int e = 0; e < p->nrg_src; e++) {
        EnergyRow &r = t->energy[e];
        r.Esrc1 = P.e_src_min + (double)e * P.dEs;
        r.Esrc2 = P.e_src_min + (double)(e + 1) * P.dEs;
        r.Esrc = 0.5 * (r.Esrc1 + r.Esrc2);
        r.ein = r.Esrc / P.mec2;
        const double f1 = r.ein * r.ein * r.ein, f2 = P.kn0 + P.kn1 * r.ein + P.kn2 * r.ein * r.ein;
        r.inv_f1 = (float)(1.0 / f1);
        r.inv_f2 = (float)(1.0 / f2);
        r.inv_f1_lo = (float)(1.0 / f1 - (double)r.inv_f1);
        r.inv_f2_lo = (float)(1.0 / f2 - (double)r.inv_f2);
        const double wf = 2.0 * r.Esrc / P.hbarc;
        r.wfac_hi = (float)wf;
        r.wfac_lo = (float)(wf - (double)r.wfac_hi);
        const double c1 = (2.0 / P.hbarc) * (2.0 / P.hbarc) * P.dEs * P.dEs / 12.0;
        const double c2 = (r.Esrc / P.hbarc) * (r.Esrc / P.hbarc) / 4.0;
        r.sig_c1 = (float)c1;
        r.sig_c2 = (float)c2;
        r.sig_c1_lo = (float)(c1 - (double)r.sig_c1);
        r.sig_c2_lo = (float)(c2 - (double)r.sig_c2);
        r.einf = (float)r.ein;
        r.Esrc1f = (float)r.Esrc1;
        r.Esrc2f = (float)r.Esrc2;
    }
    // spectrum windows: detector bin n takes source bins win_lo[n] .. + W-1
    // with weights RF = spectrum[e + n*nrg_src]; win_n[e] = the detector bins
    // whose window holds e
    const int same = (p->nrg_src == p->nrg_det && p->e_src_min == p->e_det_min && p->e_src_max == p->e_det_max);
    t->rf_win.assign((size_t)p->nrg_det * W, 0.f);
    t->win_lo.assign(p->nrg_det, 0);
    t->win_n.assign(2 * (size_t)p->nrg_src, 0);
    for (int e = 0; e < p->nrg_src; e++) {
        t->win_n[2 * e] = p->nrg_det;
        t->win_n[2 * e + 1] = -1;
    }
    for (int n = 0; n < p->nrg_det; n++) {
        int lo, hi;
        src_nrg_range(P, same, n, &lo, &hi);
        t->win_lo[n] = lo;
        for (int j = 0; j < W; j++) {
            t->rf_win[(size_t)n * W + j] = spec_h[(lo + j) + (size_t)n * p->nrg_src];
            const int e = lo + j;
            if (n < t->win_n[2 * e]) t->win_n[2 * e] = n;
            if (n > t->win_n[2 * e + 1]) t->win_n[2 * e + 1] = n;
        }
    }
    // Compton slots: for source bin e, slot s is detector bin win_n(e) + s
    t->sl = 1;
    for (int e = 0; e < p->nrg_src; e++)
        if (t->win_n[2 * e + 1] >= t->win_n[2 * e]) t->sl = std::max(t->sl, t->win_n[2 * e + 1] - t->win_n[2 * e] + 1);
    t->offs_e.assign((size_t)p->nrg_src * t->sl, 0.f);
    for (int e = 0; e < p->nrg_src; e++)
        for (int s = 0; s < t->sl; s++) {
            const double Ed1 = P.e_det_min + (double)(t->win_n[2 * e] + s) * P.dEd;
            t->offs_e[(size_t)e * t->sl + s] = (float)((P.e_src_min + (double)e * P.dEs) - Ed1);
        }
    t->fine_q.resize(p->nqf);
    for (int j = 0; j < p->nqf; j++) {
        const double q = P.q_lo + P.dq_fine * (0.5 + (double)j);
        t->fine_q[j].x = (float)q;
        t->fine_q[j].y = (float)(q - (double)t->fine_q[j].x);
    }
    // coarse bins of wvt_value.cu:8-22: centre as a pair, width
    t->coarse_q.resize(p->nwt);
    for (int k = 0; k < p->nwt; k++) {
        const double NWT = (double)p->nwt;
        const double e1 = p->q_lo + (double)k * p->dq0 +
                          (p->q_hi - p->q_lo - p->dq0 * NWT) * (double)((int64_t)k * k) / (NWT * NWT);
        const double e2 = p->q_lo + (double)(k + 1) * p->dq0 +
                          (p->q_hi - p->q_lo - p->dq0 * NWT) * (double)((int64_t)(k + 1) * (k + 1)) / (NWT * NWT);
        const double q = 0.5 * (e1 + e2);
        t->coarse_q[k].x = (float)q;
        t->coarse_q[k].y = (float)(q - (double)t->coarse_q[k].x);
        t->coarse_q[k].z = (float)(e2 - e1);
        t->coarse_q[k].w = 0.f;
    }
}

} // namespace xrdt

extern "C" {

int32_t xrdt_abi_version(void) { return XRDT_ABI_VERSION; }

const char *xrdt_status_string(int32_t s)
{
    switch (s) {
    case XRDT_OK: return "ok";
    case XRDT_ERR_NULL: return "null pointer";
    case XRDT_ERR_DIMS: return "dimension out of range";
    case XRDT_ERR_GEOMETRY: return "source or detector inside the phantom";
    case XRDT_ERR_INPUT: return "invalid input values";
    case XRDT_ERR_CUDA: return "CUDA error";
    case XRDT_ERR_ALLOC: return "allocation failed";
    case XRDT_ERR_UNSUPPORTED: return "unsupported option";
    case XRDT_ERR_TIMEOUT: return "device wait timed out";
    case XRDT_ERR_IO: return "file could not be written or read";
    default: return "unknown status";
    }
}

int32_t xrdt_problem_reference(xrdt_problem *p, int32_t nx, int32_t ny)
{
    if (!p) return XRDT_ERR_NULL;
    if (nx <= 0 || ny <= 0) return XRDT_ERR_DIMS;
    memset(p, 0, sizeof *p);
    p->nx = nx;
    p->ny = ny;
    p->n_src = 32;      // Forward_XRD.cu:17-25,47-48
    p->n_col = 1024;
    p->n_row = 1;
    p->nrg_src = 64;
    p->nrg_det = 64;
    p->dnrg = 5;
    p->nwt = 256;
    p->nqf = 768;
    p->n_mat = 3;
    p->nq = 64;
    p->na = 64;
    p->quirks = XRDT_QUIRK_STALE_VOXEL_A;
    p->e_src_min = p->e_det_min = 8.0;   // integrate_diffraction.cu:138-140
    p->e_src_max = p->e_det_max = 80.0;
    p->q_lo = (double)0.5f;              // Forward_XRD.cu:39-41
    p->q_hi = (double)6.0f;
    p->dq0 = (double)0.01f;
    p->hbarc = (double)1.973269804f;     // Forward_XRD.cu:36
    p->mec2 = (double)510.99895f;        // integrate_diffraction.cu:278
    p->kn0 = (double)0.751691286166726f; // Forward_XRD.cu:51-53
    p->kn1 = (double)1.4599683207703f;
    p->kn2 = (double)-0.64597532690936f;
    p->rsqrt2pi = (double)0.398942280401433f;  // Forward_XRD.cu:34
    p->dq_step = (double)0.25f;          // Forward_XRD.cu:44
    const double mmv = (double)nx / 100.0;     // integrate_diffraction.cu:81
    const double Lx = 200.0 * mmv, Ly = 200.0 * mmv;
    p->cx = Lx / 2.0;
    p->cy = Ly / 2.0;
    p->r_src = 150.0 * mmv;              // :84-85
    p->r_det = 170.0 * mmv;
    p->src_arc = (double)6.28318530717959f;  // twopi, Forward_XRD.cu:35
    p->src_phi0 = 0.0;
    p->col_pitch = 0.5 * mmv;            // :99-101
    p->row_pitch = 1.0 * mmv;
    p->z0 = 10.0 * mmv;
    p->focal_spot = 0.5 * mmv;           // :118
    p->target_angle = (double)0.523598775598299f;   // :117
    p->wedge_angle = (double)0.00872664625997165f;  // :126
    p->vox_side = 1.0;                   // :128
    return XRDT_OK;
}

int32_t xrdt_problem_validate(const xrdt_problem *p)
{
    if (!p) return XRDT_ERR_NULL;
    if (p->nx < 1 || p->ny < 1 || p->nx > 32767 || p->ny > 32767) return XRDT_ERR_DIMS;
    if (p->n_src < 1 || p->n_src > 65535 || p->n_col < 1 || p->n_row < 1) return XRDT_ERR_DIMS;
    if ((int64_t)p->n_col * p->n_row > 2147483647LL) return XRDT_ERR_DIMS;
    if (p->dnrg < 0 || p->nrg_det < 1 || p->nrg_src < 2 * p->dnrg + 1) return XRDT_ERR_DIMS;
    if (p->nwt < 1 || p->nqf < 1 || p->n_mat < 1 || p->nq < 1 || p->na < 1) return XRDT_ERR_DIMS;
    if (p->reserved0 != 0 || (p->quirks & ~XRDT_QUIRK_STALE_VOXEL_A)) return XRDT_ERR_DIMS;
    if (!finite_all(p)) return XRDT_ERR_DIMS;
    if (!(p->e_src_max > p->e_src_min) || !(p->e_det_max > p->e_det_min) || !(p->q_hi > p->q_lo))
        return XRDT_ERR_DIMS;
    if (!(p->dq0 > 0) || !(p->dq_step > 0) || !(p->hbarc > 0) || !(p->mec2 > 0) || !(p->vox_side > 0))
        return XRDT_ERR_DIMS;
    for (int s = 0; s < p->n_src; s++) {
        SrcGeom g;
        src_geom(p, s, &g);
        if (inside_roi(p, g.Rsrc_x, g.Rsrc_y)) return XRDT_ERR_GEOMETRY;
        // the detector panel is a segment; its end pixels bound it
        for (int c = 0; c < p->n_col; c += (p->n_col > 1 ? p->n_col - 1 : 1)) {
            const double rdet = ((double)c - (double)p->n_col / 2.0 + 0.5) * p->col_pitch;
            const double x = p->cx - p->r_det * g.sphi + rdet * g.cphi;
            const double y = p->cy + p->r_det * g.cphi + rdet * g.sphi;
            if (inside_roi(p, x, y)) return XRDT_ERR_GEOMETRY;
        }
        // the segment between the end pixels must not cross the ROI either
        const double r0 = (0.0 - (double)p->n_col / 2.0 + 0.5) * p->col_pitch;
        const double r1 = ((double)(p->n_col - 1) - (double)p->n_col / 2.0 + 0.5) * p->col_pitch;
        for (int k = 1; k < 64; k++) {
            const double r = r0 + (r1 - r0) * k / 64.0;
            if (inside_roi(p, p->cx - p->r_det * g.sphi + r * g.cphi, p->cy + p->r_det * g.cphi + r * g.sphi))
                return XRDT_ERR_GEOMETRY;
        }
    }
    return XRDT_OK;
}

int64_t xrdt_problem_rays(const xrdt_problem *p)
{
    if (!p) return -1;
    return (int64_t)p->n_src * p->n_col * p->n_row * p->nrg_det;
}

int64_t xrdt_problem_amatrix_elems(const xrdt_problem *p)
{
    if (!p) return -1;
    return xrdt_problem_rays(p) * p->nwt * p->n_mat;
}

int32_t xrdt_ctx_create(xrdt_ctx **out, int32_t device, void *stream)
{
    if (!out) return XRDT_ERR_NULL;
    *out = nullptr;
    xrdt_ctx *ctx = new xrdt_ctx();
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) {
        if (stream) {
            ctx->stream = (cudaStream_t)stream;
        } else {
            e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
            ctx->own_stream = (e == cudaSuccess);
        }
    }
    if (e == cudaSuccess) e = cudaMallocHost((void **)&ctx->h_counters, 16 * sizeof(int));
    if (e != cudaSuccess) {
        cudaGetLastError();
        if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
        delete ctx;
        return XRDT_ERR_CUDA;
    }
    ctx->buf.assign(S_COUNT, nullptr);
    ctx->cap.assign(S_COUNT, 0);
    *out = ctx;
    return XRDT_OK;
}

int32_t xrdt_ctx_set_profiling(xrdt_ctx *ctx, int32_t enable)
{
    if (!ctx) return XRDT_ERR_NULL;
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    fold_pending(ctx);
    for (int k = 0; k < XRDT_KERNEL_COUNT; k++) {
        ctx->prof_launches[k] = 0;
        ctx->prof_ms[k] = 0.0;
    }
    if (enable && !ctx->d_work) {
        cudaError_t e = cudaMalloc((void **)&ctx->d_work, sizeof(unsigned long long));
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(ctx, XRDT_ERR_ALLOC, "profiling counter allocation failed");
        }
    }
    if (ctx->d_work) CK(cudaMemset(ctx->d_work, 0, sizeof(unsigned long long)));
    ctx->profiling = enable != 0;
    return XRDT_OK;
}

int32_t xrdt_ctx_kernel_stats(xrdt_ctx *ctx, int32_t kernel, int64_t *launches, double *total_ms, int64_t *work)
{
    if (!ctx) return XRDT_ERR_NULL;
    if (kernel < 0 || kernel >= XRDT_KERNEL_COUNT) return fail(ctx, XRDT_ERR_DIMS, "unknown kernel group");
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    fold_pending(ctx);
    if (launches) *launches = ctx->prof_launches[kernel];
    if (total_ms) *total_ms = ctx->prof_ms[kernel];
    if (work) {
        unsigned long long w = 0;
        if (kernel == XRDT_KERNEL_FORWARD && ctx->d_work)
            CK(cudaMemcpy(&w, ctx->d_work, sizeof w, cudaMemcpyDeviceToHost));
        *work = (int64_t)w;
    }
    return XRDT_OK;
}

int32_t xrdt_ctx_destroy(xrdt_ctx *ctx)
{
    if (!ctx) return XRDT_ERR_NULL;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    fold_pending(ctx);
    if (ctx->mlem_exec) cudaGraphExecDestroy(ctx->mlem_exec);
    if (ctx->d_work) cudaFree(ctx->d_work);
    for (void *p : ctx->buf)
        if (p) cudaFree(p);
    if (ctx->h_counters) cudaFreeHost(ctx->h_counters);
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return XRDT_OK;
}

int32_t xrdt_ctx_synchronize(xrdt_ctx *ctx)
{
    if (!ctx) return XRDT_ERR_NULL;
    CK(cudaStreamSynchronize(ctx->stream));
    return XRDT_OK;
}

const char *xrdt_last_error(const xrdt_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int64_t xrdt_ctx_launch_count(const xrdt_ctx *ctx) { return ctx ? ctx->launches : -1; }

} // extern "C"

namespace {

// Bound on the staged detector-side integrals of one tile of pairs.
constexpr int64_t kWalkTableBytes = (int64_t)4 << 30;

// Shared body of xrdt_forward (rays == NULL: every ray, the Forward_XRD
// layout) and xrdt_forward_rays (outputs per listed ray).
// tab (the cross-section table path, xrdt_forward_tables): 0 = the fine-q
// patterns Ifine; 1 = the coherent table S1, nearest bins; 2 = both tables
// read bilinearly.
int forward_impl(xrdt_ctx *ctx, const xrdt_problem *p, const float *spectrum, const float *Ifine,
                 const int32_t *seg, const float *a1, const float *a2, const float *S2, float q_min,
                 float q_max, float a_min, float a_max, const int64_t *ray_list, int64_t n_list,
                 float *Nphotons, float *Cphotons, float *Amatrix, uint32_t flags, const float *S1 = nullptr,
                 int tab = 0)
{
    if (!ctx) return XRDT_ERR_NULL;
    ctx->err.clear();
    if (!p || !spectrum || (!Ifine && !tab) || (!S1 && tab) || !seg || !a1 || !a2 || !S2 || !Nphotons || !Cphotons)
        return fail(ctx, XRDT_ERR_NULL, "a required array pointer is NULL");
    if (tab && (Amatrix || ray_list || (flags & XRDT_FWD_PLAIN_FP64)))
        return fail(ctx, XRDT_ERR_UNSUPPORTED, "the table path computes Nphotons and Cphotons of every ray");
    if (tab && (p->nq < 2 || p->na < 2)) return fail(ctx, XRDT_ERR_DIMS, "the table path needs NQ, NA >= 2");
    int rc = xrdt_problem_validate(p);
    if (rc) return fail(ctx, rc, fmt("problem rejected: %s", xrdt_status_string(rc)));
    if (flags & ~(XRDT_FWD_PLAIN_FP64 | XRDT_FWD_NO_SYNC))
        return fail(ctx, XRDT_ERR_UNSUPPORTED, "unknown flag bits");
    if (!std::isfinite(q_min) || !std::isfinite(q_max) || !std::isfinite(a_min) || !std::isfinite(a_max))
        return fail(ctx, XRDT_ERR_INPUT, "table edges must be finite");
    const bool plain = flags & XRDT_FWD_PLAIN_FP64;
    if (plain && (p->nwt % 32 != 0 || p->nwt > 1024))
        return fail(ctx, XRDT_ERR_UNSUPPORTED, "the reference launch shape needs NWT a multiple of 32, <= 1024");
    DevProblem P;
    std::string err;
    build_dev_problem(p, q_min, q_max, a_min, a_max, &P, &err);
    if (!plain && P.e_hi - P.e_lo + 1 > 128)
        return fail(ctx, XRDT_ERR_UNSUPPORTED, "more than 128 source energy bins in the windows");
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;

    const int64_t nvox = (int64_t)p->nx * p->ny;
    const int64_t all_rays = xrdt_problem_rays(p);
    const int64_t MW = (int64_t)p->nwt * p->n_mat;
    if (ray_list) {
        if (n_list < 0 || n_list > 2147483647LL) return fail(ctx, XRDT_ERR_DIMS, "bad ray count");
        if (is_device_ptr(ray_list)) return fail(ctx, XRDT_ERR_UNSUPPORTED, "the ray list must be host memory");
        for (int64_t i = 0; i < n_list; i++)
            if (ray_list[i] < 0 || ray_list[i] >= all_rays)
                return fail(ctx, XRDT_ERR_INPUT, fmt("ray %lld out of range", (long long)ray_list[i]));
    }
    // output element counts
    const int64_t rays = ray_list ? n_list : all_rays;
    const int64_t aelems = rays * MW;

    // ---- inputs ----
    const void *d_spec, *d_ifine, *d_seg, *d_a1, *d_a2, *d_S2;
    if ((rc = stage_in(ctx, S_SPEC, spectrum, sizeof(float) * p->nrg_src * p->nrg_det, &d_spec))) return rc;
    d_ifine = nullptr;
    if (!tab && (rc = stage_in(ctx, S_IFINE, Ifine, sizeof(float) * (size_t)p->nqf * p->n_mat, &d_ifine))) return rc;
    const void *d_S1 = nullptr;
    if (tab && (rc = stage_in(ctx, S_S1, S1, sizeof(float) * (size_t)p->nq * p->na, &d_S1))) return rc;
    if ((rc = stage_in(ctx, S_SEG, seg, sizeof(int32_t) * nvox, &d_seg))) return rc;
    if ((rc = stage_in(ctx, S_A1, a1, sizeof(float) * nvox, &d_a1))) return rc;
    if ((rc = stage_in(ctx, S_A2, a2, sizeof(float) * nvox, &d_a2))) return rc;
    if ((rc = stage_in(ctx, S_S2, S2, sizeof(float) * (size_t)p->nq * p->na, &d_S2))) return rc;
    const bool hostN = !is_device_ptr(Nphotons), hostC = !is_device_ptr(Cphotons);
    const bool hostA = Amatrix && !is_device_ptr(Amatrix);
    if ((flags & XRDT_FWD_NO_SYNC) && (hostN || hostC || hostA))
        return fail(ctx, XRDT_ERR_UNSUPPORTED, "XRDT_FWD_NO_SYNC needs device outputs");
    float *dN = Nphotons, *dC = Cphotons, *dA = Amatrix;
    void *tmp;
    if (hostN) { if ((rc = get_buf(ctx, S_N, sizeof(float) * rays, &tmp))) return rc; dN = (float *)tmp; }
    if (hostC) { if ((rc = get_buf(ctx, S_C, sizeof(float) * rays, &tmp))) return rc; dC = (float *)tmp; }
    if (hostA) { if ((rc = get_buf(ctx, S_A, sizeof(float) * aelems, &tmp))) return rc; dA = (float *)tmp; }

    // ---- per-call tables (host, double) ----
    std::vector<SrcGeom> hsg(p->n_src);
    for (int s = 0; s < p->n_src; s++) src_geom(p, s, &hsg[s]);
    PrepBuffers B;
    void *d_srcg;
    if ((rc = get_buf(ctx, S_SRCG, sizeof(SrcGeom) * p->n_src, &d_srcg))) return rc;
    CK(cudaMemcpyAsync(d_srcg, hsg.data(), sizeof(SrcGeom) * p->n_src, cudaMemcpyHostToDevice, st));
    if ((rc = get_buf(ctx, S_CELLS, sizeof(float4) * 4 * (size_t)(p->nx + 1) * (p->ny + 1), &tmp))) return rc;
    B.cells = (float4 *)tmp;
    if ((rc = get_buf(ctx, S_VXY, sizeof(int) * nvox, &tmp))) return rc;
    B.vox_xy = (int *)tmp;
    if ((rc = get_buf(ctx, S_VMAT, sizeof(int) * nvox, &tmp))) return rc;
    B.vox_mat = (int *)tmp;
    if ((rc = get_buf(ctx, S_VNA, sizeof(int) * nvox, &tmp))) return rc;
    B.vox_na = (int *)tmp;
    if ((rc = get_buf(ctx, S_VA2, sizeof(float) * nvox, &tmp))) return rc;
    B.vox_a2 = (float *)tmp;
    if ((rc = get_buf(ctx, S_CNT, sizeof(int) * 4, &tmp))) return rc;
    B.counters = (int *)tmp;
    if ((rc = get_buf(ctx, S_S2U8, (size_t)p->nq * p->na, &tmp))) return rc;
    B.s2u8 = (unsigned char *)tmp;
    B.atten_src = nullptr;
    if (tab) {
        if ((rc = get_buf(ctx, S_S1U8, (size_t)p->nq * p->na, &tmp))) return rc;
        B.s1u8 = (unsigned char *)tmp;
    }
    if (tab == 2) {
        if ((rc = get_buf(ctx, S_VTA, sizeof(float) * nvox, &tmp))) return rc;
        B.vox_ta = (float *)tmp;
    }

    { ProfScope ps(ctx, XRDT_KERNEL_PREP_VOXELS);
    CK(launch_prep_voxels(P, (const int32_t *)d_seg, (const float *)d_a1, (const float *)d_a2, B, st,
                          &ctx->launches)); }
    CK(cudaMemcpyAsync(ctx->h_counters, B.counters, sizeof(int) * 2, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    const int nv = ctx->h_counters[0];
    if (ctx->h_counters[1])
        return fail(ctx, XRDT_ERR_INPUT, fmt("segmentation holds a material id above n_mat = %d", p->n_mat));

    if (plain) {
        std::vector<double> cq(2 * (size_t)p->nwt);
        for (int k = 0; k < p->nwt; k++) {
            const double NWT = (double)p->nwt;
            const double e1 = p->q_lo + (double)k * p->dq0 +
                              (p->q_hi - p->q_lo - p->dq0 * NWT) * (double)((int64_t)k * k) / (NWT * NWT);
            const double e2 = p->q_lo + (double)(k + 1) * p->dq0 +
                              (p->q_hi - p->q_lo - p->dq0 * NWT) * (double)((int64_t)(k + 1) * (k + 1)) / (NWT * NWT);
            cq[2 * k] = 0.5 * (e1 + e2);
            cq[2 * k + 1] = e2 - e1;
        }
        if ((rc = get_buf(ctx, S_COARSEQD, sizeof(double) * cq.size(), &tmp))) return rc;
        CK(cudaMemcpyAsync(tmp, cq.data(), sizeof(double) * cq.size(), cudaMemcpyHostToDevice, st));
        const int64_t *d_rays = nullptr;
        if (ray_list) {
            void *dr;
            if ((rc = get_buf(ctx, S_RAYS, sizeof(int64_t) * (n_list ? n_list : 1), &dr))) return rc;
            if (n_list) CK(cudaMemcpyAsync(dr, ray_list, sizeof(int64_t) * n_list, cudaMemcpyHostToDevice, st));
            d_rays = (const int64_t *)dr;
        }
        ProfScope ps(ctx, XRDT_KERNEL_PLAIN);
        CK(launch_plain_forward(P, (const SrcGeom *)d_srcg, (const float *)d_spec, (const float *)d_ifine,
                                (const int32_t *)d_seg, (const float *)d_a1, (const float *)d_a2,
                                (const float *)d_S2, (const double *)tmp, d_rays, n_list, dN, dC, dA, st,
                                &ctx->launches));
    } else if (nv == 0) {
        // empty phantom: every output is zero (integrate_diffraction.cu:148-150,364-409)
        CK(cudaMemsetAsync(dN, 0, sizeof(float) * rays, st));
        CK(cudaMemsetAsync(dC, 0, sizeof(float) * rays, st));
        if (dA) CK(cudaMemsetAsync(dA, 0, sizeof(float) * aelems, st));
    } else {
        std::vector<float> hspec;
        const float *spec_h = spectrum;
        if (is_device_ptr(spectrum)) {
            hspec.resize((size_t)p->nrg_src * p->nrg_det);
            CK(cudaMemcpy(hspec.data(), spectrum, sizeof(float) * hspec.size(), cudaMemcpyDeviceToHost));
            spec_h = hspec.data();
        }
        HostTables ht;
        build_host_tables(p, P, spec_h, &ht);
        const std::vector<EnergyRow> &er = ht.energy;
        const std::vector<float> &rfw = ht.rf_win, &offs_e = ht.offs_e;
        const std::vector<int> &wlo = ht.win_lo, &wn = ht.win_n;
        const std::vector<float2> &fq = ht.fine_q;
        const std::vector<float4> &cqf = ht.coarse_q;
        const int sl = ht.sl;
        FwdTables T;
        void *d;
        if ((rc = get_buf(ctx, S_ENERGY, sizeof(EnergyRow) * er.size(), &d))) return rc;
        CK(cudaMemcpyAsync(d, er.data(), sizeof(EnergyRow) * er.size(), cudaMemcpyHostToDevice, st));
        T.energy = (const EnergyRow *)d;
        if ((rc = get_buf(ctx, S_RFWIN, sizeof(float) * rfw.size(), &d))) return rc;
        CK(cudaMemcpyAsync(d, rfw.data(), sizeof(float) * rfw.size(), cudaMemcpyHostToDevice, st));
        T.rf_win = (const float *)d;
        if ((rc = get_buf(ctx, S_OFFS, sizeof(float) * offs_e.size(), &d))) return rc;
        CK(cudaMemcpyAsync(d, offs_e.data(), sizeof(float) * offs_e.size(), cudaMemcpyHostToDevice, st));
        T.offs_e = (const float *)d;
        T.sl = sl;
        if ((rc = get_buf(ctx, S_WINLO, sizeof(int) * wlo.size(), &d))) return rc;
        CK(cudaMemcpyAsync(d, wlo.data(), sizeof(int) * wlo.size(), cudaMemcpyHostToDevice, st));
        T.win_lo = (const int *)d;
        if ((rc = get_buf(ctx, S_WINN, sizeof(int) * wn.size(), &d))) return rc;
        CK(cudaMemcpyAsync(d, wn.data(), sizeof(int) * wn.size(), cudaMemcpyHostToDevice, st));
        T.win_n = (const int *)d;
        if ((rc = get_buf(ctx, S_FINEQ, sizeof(float2) * fq.size(), &d))) return rc;
        CK(cudaMemcpyAsync(d, fq.data(), sizeof(float2) * fq.size(), cudaMemcpyHostToDevice, st));
        T.fine_q = (const float2 *)d;
        if ((rc = get_buf(ctx, S_COARSEQ, sizeof(float4) * cqf.size(), &d))) return rc;
        CK(cudaMemcpyAsync(d, cqf.data(), sizeof(float4) * cqf.size(), cudaMemcpyHostToDevice, st));
        T.coarse_q = (const float4 *)d;

        if ((rc = get_buf(ctx, S_ASRC, sizeof(float2) * (size_t)p->n_src * nv, &tmp))) return rc;
        B.atten_src = (float2 *)tmp;
        { ProfScope ps(ctx, XRDT_KERNEL_PREP_MAP);
          CK(launch_prep_map(P, (const float *)d_a1, (const float *)d_a2, (const float *)d_S2, B, st, &ctx->launches,
                             (const float *)d_S1)); }
        { ProfScope ps(ctx, XRDT_KERNEL_SRC_ATTEN);
          CK(launch_src_atten(P, (const SrcGeom *)d_srcg, nv, B, st, &ctx->launches)); }
        T.work = ctx->profiling ? ctx->d_work : nullptr;
        // pairs go through in tiles: the detector-side integrals of a tile
        // (k_walk.cu), then the projector over the same pairs
        auto project = [&](const int2 *list, int64_t n_total, float *oN, float *oC, float *oA) -> int {
            // whole groups of 32 pixels of every view (32 entries of a list)
            const int64_t unit = list ? 32 : 32 * (int64_t)p->n_src;
            const int64_t fit = std::min<int64_t>(kWalkTableBytes / ((int64_t)nv * (int64_t)sizeof(float2)),
                                                  (int64_t)1 << 30);
            const int64_t tile = std::min<int64_t>(n_total, std::max<int64_t>(unit, fit / unit * unit));
            void *dtab;
            int r = get_buf(ctx, S_WALK, sizeof(float2) * (size_t)tile * nv, &dtab);
            if (r) return r;
            for (int64_t p0 = 0; p0 < n_total; p0 += tile) {
                const int64_t n = std::min(tile, n_total - p0);
                {
                    ProfScope ps(ctx, XRDT_KERNEL_WALK);
                    CK(launch_det_walk(P, (const SrcGeom *)d_srcg, list ? list + p0 : nullptr, p0, n, B.vox_xy, nv,
                                       B.cells, (float2 *)dtab, st, &ctx->launches));
                }
                ProfScope ps(ctx, XRDT_KERNEL_FORWARD);
                CK(launch_fast_forward(P, (const SrcGeom *)d_srcg, T, B, nv, (const float *)d_ifine, list, n_total,
                                       p0, (int)n, (const float2 *)dtab, oN, oC, oA, st, &ctx->launches, tab));
            }
            return XRDT_OK;
        };
        if (!ray_list) {
            if ((rc = project(nullptr, (int64_t)p->n_src * P.n_det, dN, dC, dA))) return rc;
        } else if (n_list > 0) {
            // the (src, det) pairs the listed rays need, then a gather
            std::vector<int64_t> cols(n_list);
            for (int64_t i = 0; i < n_list; i++) cols[i] = ray_list[i] % ((int64_t)p->n_src * P.n_det);
            std::vector<int64_t> uniq(cols);
            std::sort(uniq.begin(), uniq.end());
            uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
            const int np = (int)uniq.size();
            std::vector<int2> pairs(np);
            for (int i = 0; i < np; i++) pairs[i] = make_int2((int)(uniq[i] % p->n_src), (int)(uniq[i] / p->n_src));
            std::vector<int64_t> idx(n_list);
            for (int64_t i = 0; i < n_list; i++) {
                const int64_t pi = std::lower_bound(uniq.begin(), uniq.end(), cols[i]) - uniq.begin();
                const int64_t nrg = ray_list[i] / ((int64_t)p->n_src * P.n_det);
                idx[i] = pi + nrg * np;
            }
            void *dpairs, *didx, *dNc, *dCc, *dAc = nullptr;
            const int64_t ncomp = (int64_t)np * p->nrg_det;
            if ((rc = get_buf(ctx, S_PAIRS, sizeof(int2) * np, &dpairs))) return rc;
            if ((rc = get_buf(ctx, S_RAYS, sizeof(int64_t) * n_list, &didx))) return rc;
            if ((rc = get_buf(ctx, S_NC, sizeof(float) * ncomp, &dNc))) return rc;
            if ((rc = get_buf(ctx, S_CC, sizeof(float) * ncomp, &dCc))) return rc;
            if (dA && (rc = get_buf(ctx, S_AC, sizeof(float) * ncomp * MW, &dAc))) return rc;
            CK(cudaMemcpyAsync(dpairs, pairs.data(), sizeof(int2) * np, cudaMemcpyHostToDevice, st));
            CK(cudaMemcpyAsync(didx, idx.data(), sizeof(int64_t) * n_list, cudaMemcpyHostToDevice, st));
            if ((rc = project((const int2 *)dpairs, np, (float *)dNc, (float *)dCc, (float *)dAc))) return rc;
            ProfScope ps(ctx, XRDT_KERNEL_GATHER);
            CK(launch_gather_rays((const int64_t *)didx, n_list, (const float *)dNc, (const float *)dCc,
                                  (const float *)dAc, (int)MW, dN, dC, dA, st, &ctx->launches));
            // the pair list and index buffers are read asynchronously
            CK(cudaStreamSynchronize(st));
        }
    }

    // ---- outputs ----
    if (hostN) CK(cudaMemcpyAsync(Nphotons, dN, sizeof(float) * rays, cudaMemcpyDeviceToHost, st));
    if (hostC) CK(cudaMemcpyAsync(Cphotons, dC, sizeof(float) * rays, cudaMemcpyDeviceToHost, st));
    if (hostA) CK(cudaMemcpyAsync(Amatrix, dA, sizeof(float) * aelems, cudaMemcpyDeviceToHost, st));
    if (!(flags & XRDT_FWD_NO_SYNC)) CK(cudaStreamSynchronize(st));
    return XRDT_OK;
}

} // namespace

extern "C" {

int32_t xrdt_forward(xrdt_ctx *ctx, const xrdt_problem *p, const float *spectrum, const float *Ifine,
                     const int32_t *seg, const float *a1, const float *a2, const float *S2, float q_min,
                     float q_max, float a_min, float a_max, float *Nphotons, float *Cphotons,
                     float *Amatrix, uint32_t flags)
{
    return forward_impl(ctx, p, spectrum, Ifine, seg, a1, a2, S2, q_min, q_max, a_min, a_max, nullptr, 0,
                        Nphotons, Cphotons, Amatrix, flags);
}

int32_t xrdt_forward_tables(xrdt_ctx *ctx, const xrdt_problem *p, const float *spectrum, const int32_t *seg,
                            const float *a1, const float *a2, const float *S1, const float *S2, float q_min,
                            float q_max, float a_min, float a_max, float *Nphotons, float *Cphotons,
                            uint32_t flags)
{
    if (!ctx) return XRDT_ERR_NULL;
    if (flags & ~(XRDT_TAB_BILINEAR | XRDT_FWD_NO_SYNC)) return fail(ctx, XRDT_ERR_UNSUPPORTED, "unknown flag bits");
    const int tab = (flags & XRDT_TAB_BILINEAR) ? 2 : 1;
    return forward_impl(ctx, p, spectrum, nullptr, seg, a1, a2, S2, q_min, q_max, a_min, a_max, nullptr, 0,
                        Nphotons, Cphotons, nullptr, flags & XRDT_FWD_NO_SYNC, S1, tab);
}

int32_t xrdt_forward_rays(xrdt_ctx *ctx, const xrdt_problem *p, const float *spectrum, const float *Ifine,
                          const int32_t *seg, const float *a1, const float *a2, const float *S2, float q_min,
                          float q_max, float a_min, float a_max, const int64_t *rays, int64_t n_rays,
                          float *Nphotons, float *Cphotons, float *A_rows, uint32_t flags)
{
    if (!rays && n_rays) return fail(ctx, XRDT_ERR_NULL, "ray list is NULL");
    static const int64_t none = 0;
    return forward_impl(ctx, p, spectrum, Ifine, seg, a1, a2, S2, q_min, q_max, a_min, a_max,
                        rays ? rays : &none, n_rays, Nphotons, Cphotons, A_rows, flags);
}

int32_t xrdt_debug_decisions(xrdt_ctx *ctx, const xrdt_problem *p, const float *spectrum, const int32_t *seg,
                             const float *a1, const float *a2, const float *S2, float q_min, float q_max,
                             float a_min, float a_max, const int64_t *rays, int64_t n_rays, int32_t *win,
                             int32_t *walk, int32_t *na, int32_t *nq, uint8_t *s2u8, int64_t *nv_out)
{
    if (!ctx) return XRDT_ERR_NULL;
    ctx->err.clear();
    if (!p || !spectrum || !seg || !a1 || !a2 || !S2 || !nv_out || (n_rays && (!rays || !win || !walk || !nq)) ||
        !na || !s2u8)
        return fail(ctx, XRDT_ERR_NULL, "a required array pointer is NULL");
    int rc = xrdt_problem_validate(p);
    if (rc) return fail(ctx, rc, fmt("problem rejected: %s", xrdt_status_string(rc)));
    if (n_rays < 0 || n_rays > 65535) return fail(ctx, XRDT_ERR_DIMS, "need 0 <= n_rays <= 65535");
    const int64_t all_rays = xrdt_problem_rays(p);
    for (int64_t i = 0; i < n_rays; i++)
        if (rays[i] < 0 || rays[i] >= all_rays)
            return fail(ctx, XRDT_ERR_INPUT, fmt("ray %lld out of range", (long long)rays[i]));
    for (const void *q : {(const void *)rays, (const void *)win, (const void *)walk, (const void *)na,
                          (const void *)nq, (const void *)s2u8})
        if (q && is_device_ptr(q)) return fail(ctx, XRDT_ERR_UNSUPPORTED, "lists and outputs must be host memory");
    DevProblem P;
    std::string err;
    build_dev_problem(p, q_min, q_max, a_min, a_max, &P, &err);
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const int64_t nvox = (int64_t)p->nx * p->ny;
    const void *d_spec, *d_seg, *d_a1, *d_a2, *d_S2;
    if ((rc = stage_in(ctx, S_SPEC, spectrum, sizeof(float) * p->nrg_src * p->nrg_det, &d_spec))) return rc;
    if ((rc = stage_in(ctx, S_SEG, seg, sizeof(int32_t) * nvox, &d_seg))) return rc;
    if ((rc = stage_in(ctx, S_A1, a1, sizeof(float) * nvox, &d_a1))) return rc;
    if ((rc = stage_in(ctx, S_A2, a2, sizeof(float) * nvox, &d_a2))) return rc;
    if ((rc = stage_in(ctx, S_S2, S2, sizeof(float) * (size_t)p->nq * p->na, &d_S2))) return rc;
    // the production preparation: voxel list, Compton columns, cell map, u8 table
    std::vector<SrcGeom> hsg(p->n_src);
    for (int s = 0; s < p->n_src; s++) src_geom(p, s, &hsg[s]);
    void *d_srcg, *tmp;
    if ((rc = get_buf(ctx, S_SRCG, sizeof(SrcGeom) * p->n_src, &d_srcg))) return rc;
    CK(cudaMemcpyAsync(d_srcg, hsg.data(), sizeof(SrcGeom) * p->n_src, cudaMemcpyHostToDevice, st));
    PrepBuffers B;
    memset(&B, 0, sizeof B);
    if ((rc = get_buf(ctx, S_CELLS, sizeof(float4) * 4 * (size_t)(p->nx + 1) * (p->ny + 1), &tmp))) return rc;
    B.cells = (float4 *)tmp;
    if ((rc = get_buf(ctx, S_VXY, sizeof(int) * nvox, &tmp))) return rc;
    B.vox_xy = (int *)tmp;
    if ((rc = get_buf(ctx, S_VMAT, sizeof(int) * nvox, &tmp))) return rc;
    B.vox_mat = (int *)tmp;
    if ((rc = get_buf(ctx, S_VNA, sizeof(int) * nvox, &tmp))) return rc;
    B.vox_na = (int *)tmp;
    if ((rc = get_buf(ctx, S_VA2, sizeof(float) * nvox, &tmp))) return rc;
    B.vox_a2 = (float *)tmp;
    if ((rc = get_buf(ctx, S_CNT, sizeof(int) * 4, &tmp))) return rc;
    B.counters = (int *)tmp;
    if ((rc = get_buf(ctx, S_S2U8, (size_t)p->nq * p->na, &tmp))) return rc;
    B.s2u8 = (unsigned char *)tmp;
    CK(launch_prep_voxels(P, (const int32_t *)d_seg, (const float *)d_a1, (const float *)d_a2, B, st,
                          &ctx->launches));
    CK(launch_prep_map(P, (const float *)d_a1, (const float *)d_a2, (const float *)d_S2, B, st, &ctx->launches));
    CK(cudaMemcpyAsync(ctx->h_counters, B.counters, sizeof(int) * 2, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    const int nv = ctx->h_counters[0];
    if (ctx->h_counters[1])
        return fail(ctx, XRDT_ERR_INPUT, fmt("segmentation holds a material id above n_mat = %d", p->n_mat));
    *nv_out = nv;
    std::vector<float> hspec((size_t)p->nrg_src * p->nrg_det);
    CK(cudaMemcpy(hspec.data(), d_spec, sizeof(float) * hspec.size(), cudaMemcpyDeviceToHost));
    HostTables ht;
    build_host_tables(p, P, hspec.data(), &ht);
    const int W = 2 * p->dnrg + 1;
    for (int64_t i = 0; i < n_rays; i++) {
        const int nrg = (int)(rays[i] / ((int64_t)p->n_src * P.n_det));
        win[2 * i] = ht.win_lo[nrg];
        win[2 * i + 1] = ht.win_lo[nrg] + W - 1;
    }
    CK(cudaMemcpyAsync(s2u8, B.s2u8, (size_t)p->nq * p->na, cudaMemcpyDeviceToHost, st));
    if (nv > 0) CK(cudaMemcpyAsync(na, B.vox_na, sizeof(int) * nv, cudaMemcpyDeviceToHost, st));
    if (n_rays > 0 && nv > 0) {
        void *d_energy, *d_wlo, *d_rays, *d_walk, *d_nq;
        if ((rc = get_buf(ctx, S_ENERGY, sizeof(EnergyRow) * ht.energy.size(), &d_energy))) return rc;
        CK(cudaMemcpyAsync(d_energy, ht.energy.data(), sizeof(EnergyRow) * ht.energy.size(), cudaMemcpyHostToDevice,
                           st));
        if ((rc = get_buf(ctx, S_WINLO, sizeof(int) * ht.win_lo.size(), &d_wlo))) return rc;
        CK(cudaMemcpyAsync(d_wlo, ht.win_lo.data(), sizeof(int) * ht.win_lo.size(), cudaMemcpyHostToDevice, st));
        if ((rc = get_buf(ctx, S_RAYS, sizeof(int64_t) * n_rays, &d_rays))) return rc;
        CK(cudaMemcpyAsync(d_rays, rays, sizeof(int64_t) * n_rays, cudaMemcpyHostToDevice, st));
        if ((rc = get_buf(ctx, S_DWALK, sizeof(int4) * (size_t)n_rays * nv, &d_walk))) return rc;
        if ((rc = get_buf(ctx, S_DNQ, sizeof(int) * (size_t)n_rays * nv * W, &d_nq))) return rc;
        CK(launch_decisions(P, (const SrcGeom *)d_srcg, (const EnergyRow *)d_energy, (const int *)d_wlo,
                            (const int64_t *)d_rays, (int)n_rays, B.vox_xy, nv, (int4 *)d_walk, (int *)d_nq, st,
                            &ctx->launches));
        CK(cudaMemcpyAsync(walk, d_walk, sizeof(int4) * (size_t)n_rays * nv, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(nq, d_nq, sizeof(int) * (size_t)n_rays * nv * W, cudaMemcpyDeviceToHost, st));
    }
    CK(cudaStreamSynchronize(st));
    return XRDT_OK;
}

int32_t xrdt_basis_expand(xrdt_ctx *ctx, const float *C, int64_t M, int32_t K, const float *B, int32_t N, float *I,
                          uint32_t flags)
{
    if (!ctx) return XRDT_ERR_NULL;
    ctx->err.clear();
    if (!C || !B || !I) return fail(ctx, XRDT_ERR_NULL, "C, B and I are required");
    if (M < 1 || M > ((int64_t)1 << 40) || K < 8 || K > 64 || (K & 7) || N < 16 || N > 256 || (N & 15))
        return fail(ctx, XRDT_ERR_DIMS, "need M >= 1, K a multiple of 8 in [8, 64], N a multiple of 16 in [16, 256]");
    if (flags) return fail(ctx, XRDT_ERR_UNSUPPORTED, "unknown flag bits");
    CK(cudaSetDevice(ctx->device));
    int optin = 0;
    CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
    if ((int64_t)basis_smem(K, N) > optin) return fail(ctx, XRDT_ERR_UNSUPPORTED, "basis too large for one block");
    cudaStream_t st = ctx->stream;
    int rc;
    const void *dC, *dB;
    if ((rc = stage_in(ctx, S_BC, C, sizeof(float) * (size_t)M * K, &dC))) return rc;
    if ((rc = stage_in(ctx, S_BB, B, sizeof(float) * (size_t)K * N, &dB))) return rc;
    const bool hostI = !is_device_ptr(I);
    float *dI = I;
    void *tmp;
    if (hostI) {
        if ((rc = get_buf(ctx, S_BI, sizeof(float) * (size_t)M * N, &tmp))) return rc;
        dI = (float *)tmp;
    }
    if ((rc = get_buf(ctx, S_ERR, sizeof(unsigned), &tmp))) return rc;
    unsigned *derr = (unsigned *)tmp;
    CK(cudaMemsetAsync(derr, 0, sizeof(unsigned), st));
    {
        ProfScope ps(ctx, XRDT_KERNEL_BASIS);
        CK(launch_basis_expand((const float *)dC, M, K, (const float *)dB, N, dI, derr, st, &ctx->launches));
    }
    CK(cudaMemcpyAsync(ctx->h_counters + 2, derr, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    if (hostI) CK(cudaMemcpyAsync(I, dI, sizeof(float) * (size_t)M * N, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (ctx->h_counters[2]) return fail(ctx, XRDT_ERR_TIMEOUT, "the tensor-core accumulator never completed");
    return XRDT_OK;
}

int32_t xrdt_spectrum_build(xrdt_ctx *ctx, const float *e_hd, const float *n_hd, int32_t n_hd_bins,
                            const float *src_edges, int32_t ns, const float *det_edges, int32_t nd, double sigma0,
                            double sigma1, float *spectrum, uint32_t flags)
{
    if (!ctx) return XRDT_ERR_NULL;
    ctx->err.clear();
    if (!e_hd || !n_hd || !src_edges || !det_edges || !spectrum)
        return fail(ctx, XRDT_ERR_NULL, "a required array pointer is NULL");
    if (n_hd_bins < 1 || ns < 1 || nd < 1 || nd > 65535)
        return fail(ctx, XRDT_ERR_DIMS, "need n_hd_bins >= 1, ns >= 1 and 1 <= nd <= 65535");
    if (flags) return fail(ctx, XRDT_ERR_UNSUPPORTED, "unknown flag bits");
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    // the inputs are small: read them to the host (from either memory)
    std::vector<float> e((size_t)n_hd_bins + 1), n((size_t)n_hd_bins), es((size_t)ns + 1), ed((size_t)nd + 1);
    CK(cudaMemcpy(e.data(), e_hd, sizeof(float) * e.size(), cudaMemcpyDefault));
    CK(cudaMemcpy(n.data(), n_hd, sizeof(float) * n.size(), cudaMemcpyDefault));
    CK(cudaMemcpy(es.data(), src_edges, sizeof(float) * es.size(), cudaMemcpyDefault));
    CK(cudaMemcpy(ed.data(), det_edges, sizeof(float) * ed.size(), cudaMemcpyDefault));
    auto increasing = [](const std::vector<float> &v) {
        for (size_t i = 0; i < v.size(); i++) {
            if (!std::isfinite(v[i])) return false;
            if (i && !(v[i] > v[i - 1])) return false;
        }
        return true;
    };
    if (!increasing(e) || !increasing(es) || !increasing(ed))
        return fail(ctx, XRDT_ERR_INPUT, "bin edges must be finite and increasing");
    // fine bins (spectrum_builder.m:26, :65, :75)
    std::vector<SpecFineBin> fb((size_t)n_hd_bins);
    const double rsqrt2pi = 1.0 / std::sqrt(2.0 * 3.14159265358979323846);
    for (int h = 0; h < n_hd_bins; h++) {
        const double l = e[h], r = e[h + 1], c = 0.5 * (l + r);
        const double sig = sigma0 + sigma1 * c;
        if (!(sig > 0.0) || !std::isfinite(sig) || !std::isfinite((double)n[h]))
            return fail(ctx, XRDT_ERR_INPUT, fmt("sigma(E) = %g at fine bin %d: need a positive width and finite counts",
                                                 sig, h));
        fb[h] = SpecFineBin{l, r, c, 1.0 / (2.0 * sig * sig), (double)n[h] * rsqrt2pi / sig};
    }
    // coarse bins with the range of fine bins that overlap them
    auto coarse = [&](const std::vector<float> &edges) {
        std::vector<SpecCoarseBin> cb(edges.size() - 1);
        int h0 = 0;
        for (size_t k = 0; k + 1 < edges.size(); k++) {
            const double e1 = edges[k], e2 = edges[k + 1];
            while (h0 < n_hd_bins && !(fb[h0].right > e1)) h0++;
            int h1 = h0;
            while (h1 < n_hd_bins && fb[h1].left < e2) h1++;
            cb[k] = SpecCoarseBin{e1, e2, h0, h1};
        }
        return cb;
    };
    const std::vector<SpecCoarseBin> sb = coarse(es), db = coarse(ed);
    int rc;
    void *dfb, *dsb, *ddb;
    if ((rc = get_buf(ctx, S_SPFINE, sizeof(SpecFineBin) * fb.size(), &dfb)) ||
        (rc = get_buf(ctx, S_SPSRC, sizeof(SpecCoarseBin) * sb.size(), &dsb)) ||
        (rc = get_buf(ctx, S_SPDET, sizeof(SpecCoarseBin) * db.size(), &ddb)))
        return rc;
    CK(cudaMemcpyAsync(dfb, fb.data(), sizeof(SpecFineBin) * fb.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dsb, sb.data(), sizeof(SpecCoarseBin) * sb.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(ddb, db.data(), sizeof(SpecCoarseBin) * db.size(), cudaMemcpyHostToDevice, st));
    const size_t out_bytes = sizeof(float) * (size_t)ns * nd;
    const bool host_out = !is_device_ptr(spectrum);
    float *dout = spectrum;
    if (host_out) {
        void *tmp;
        if ((rc = get_buf(ctx, S_SPOUT, out_bytes, &tmp))) return rc;
        dout = (float *)tmp;
    }
    {
        ProfScope ps(ctx, XRDT_KERNEL_SPECTRUM);
        CK(launch_spectrum((const SpecFineBin *)dfb, (const SpecCoarseBin *)dsb, ns, (const SpecCoarseBin *)ddb, nd,
                           dout, st, &ctx->launches));
    }
    if (host_out) CK(cudaMemcpyAsync(spectrum, dout, out_bytes, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));   // the host tables above leave scope
    return XRDT_OK;
}

int32_t xrdt_ct_sinogram(xrdt_ctx *ctx, const xrdt_problem *p, const float *spectrum, const float *a1, const float *a2,
                         float *Tphotons, float *gain0, uint32_t flags)
{
    if (!ctx) return XRDT_ERR_NULL;
    ctx->err.clear();
    if (!p || !spectrum || !a1 || !a2 || !Tphotons || !gain0)
        return fail(ctx, XRDT_ERR_NULL, "a required array pointer is NULL");
    int rc = xrdt_problem_validate(p);
    if (rc) return fail(ctx, rc, fmt("problem rejected: %s", xrdt_status_string(rc)));
    if (flags) return fail(ctx, XRDT_ERR_UNSUPPORTED, "unknown flag bits");
    DevProblem P;
    std::string err;
    build_dev_problem(p, 0.f, 1.f, 0.f, 1.f, &P, &err);
    P.nq = 0;   // no Compton table
    P.na = 0;
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const int64_t nvox = (int64_t)p->nx * p->ny;
    const int64_t rays = xrdt_problem_rays(p);
    const void *d_spec, *d_a1, *d_a2;
    if ((rc = stage_in(ctx, S_SPEC, spectrum, sizeof(float) * p->nrg_src * p->nrg_det, &d_spec))) return rc;
    if ((rc = stage_in(ctx, S_A1, a1, sizeof(float) * nvox, &d_a1))) return rc;
    if ((rc = stage_in(ctx, S_A2, a2, sizeof(float) * nvox, &d_a2))) return rc;
    const bool hostT = !is_device_ptr(Tphotons), hostG = !is_device_ptr(gain0);
    float *dT = Tphotons, *dG = gain0;
    void *tmp;
    if (hostT) { if ((rc = get_buf(ctx, S_N, sizeof(float) * rays, &tmp))) return rc; dT = (float *)tmp; }
    if (hostG) { if ((rc = get_buf(ctx, S_C, sizeof(float) * rays, &tmp))) return rc; dG = (float *)tmp; }
    std::vector<float> hspec((size_t)p->nrg_src * p->nrg_det);
    CK(cudaMemcpy(hspec.data(), spectrum, sizeof(float) * hspec.size(), cudaMemcpyDefault));
    HostTables ht;
    build_host_tables(p, P, hspec.data(), &ht);
    std::vector<SrcGeom> hsg(p->n_src);
    for (int s = 0; s < p->n_src; s++) src_geom(p, s, &hsg[s]);
    void *d_srcg, *d_energy, *d_rf, *d_wlo;
    if ((rc = get_buf(ctx, S_SRCG, sizeof(SrcGeom) * p->n_src, &d_srcg))) return rc;
    if ((rc = get_buf(ctx, S_ENERGY, sizeof(EnergyRow) * ht.energy.size(), &d_energy))) return rc;
    if ((rc = get_buf(ctx, S_RFWIN, sizeof(float) * ht.rf_win.size(), &d_rf))) return rc;
    if ((rc = get_buf(ctx, S_WINLO, sizeof(int) * ht.win_lo.size(), &d_wlo))) return rc;
    CK(cudaMemcpyAsync(d_srcg, hsg.data(), sizeof(SrcGeom) * p->n_src, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d_energy, ht.energy.data(), sizeof(EnergyRow) * ht.energy.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d_rf, ht.rf_win.data(), sizeof(float) * ht.rf_win.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d_wlo, ht.win_lo.data(), sizeof(int) * ht.win_lo.size(), cudaMemcpyHostToDevice, st));
    PrepBuffers B;
    memset(&B, 0, sizeof B);
    if ((rc = get_buf(ctx, S_CELLS, sizeof(float4) * 4 * (size_t)(p->nx + 1) * (p->ny + 1), &tmp))) return rc;
    B.cells = (float4 *)tmp;
    {
        ProfScope ps(ctx, XRDT_KERNEL_PREP_MAP);
        CK(launch_prep_map(P, (const float *)d_a1, (const float *)d_a2, nullptr, B, st, &ctx->launches));
    }
    {
        ProfScope ps(ctx, XRDT_KERNEL_CT);
        CK(launch_ct_sinogram(P, (const SrcGeom *)d_srcg, B.cells, (const EnergyRow *)d_energy, (const float *)d_rf,
                              (const int *)d_wlo, dT, dG, st, &ctx->launches));
    }
    if (hostT) CK(cudaMemcpyAsync(Tphotons, dT, sizeof(float) * rays, cudaMemcpyDeviceToHost, st));
    if (hostG) CK(cudaMemcpyAsync(gain0, dG, sizeof(float) * rays, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return XRDT_OK;
}

int32_t xrdt_mlem_matrix(xrdt_ctx *ctx, const float *A, int64_t rays, int32_t K, const float *y, const float *c,
                         float *x, int32_t iters, uint32_t flags)
{
    if (!ctx) return XRDT_ERR_NULL;
    ctx->err.clear();
    if (!A || !y || !c || !x) return fail(ctx, XRDT_ERR_NULL, "a required array pointer is NULL");
    if (rays < 1 || K < 4 || K > 1024 || (K & 3) || iters < 0)
        return fail(ctx, XRDT_ERR_DIMS, "need rays >= 1, K a multiple of 4 in [4, 1024], iters >= 0");
    if (flags) return fail(ctx, XRDT_ERR_UNSUPPORTED, "unknown flag bits");
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    int rc;
    const void *dA, *dy, *dc;
    if ((rc = stage_in(ctx, S_MA, A, sizeof(float) * (size_t)rays * K, &dA))) return rc;
    if ((rc = stage_in(ctx, S_MY, y, sizeof(float) * (size_t)rays, &dy))) return rc;
    if ((rc = stage_in(ctx, S_MC, c, sizeof(float) * (size_t)rays, &dc))) return rc;
    const bool hostX = !is_device_ptr(x);
    float *dx = x;
    void *tmp;
    if (hostX) {
        if ((rc = get_buf(ctx, S_MX, sizeof(float) * K, &tmp))) return rc;
        dx = (float *)tmp;
        CK(cudaMemcpyAsync(dx, x, sizeof(float) * K, cudaMemcpyHostToDevice, st));
    }
    if (((uintptr_t)dA | (uintptr_t)dx) & 15)
        return fail(ctx, XRDT_ERR_UNSUPPORTED, "device arrays A and x must be 16-byte aligned");
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    const int nparts = mlem_pass_blocks(sms, K);
    void *dpart, *dsens;
    if ((rc = get_buf(ctx, S_MPART, sizeof(float) * (size_t)nparts * K, &dpart))) return rc;
    if ((rc = get_buf(ctx, S_MSENS, sizeof(double) * K, &dsens))) return rc;
    {
        ProfScope ps(ctx, XRDT_KERNEL_MLEM);
        CK(launch_mlem_sensitivity((const float *)dA, rays, K, (float *)dpart, nparts, (double *)dsens, st,
                                   &ctx->launches));
    }
    if (iters > 0) {
        const void *key[6] = {dA, dy, dc, dx, dpart, dsens};
        bool same = ctx->mlem_exec && ctx->mlem_rays == rays && ctx->mlem_K == K;
        for (int i = 0; i < 6 && same; i++) same = ctx->mlem_key[i] == key[i];
        if (!same) {
            if (ctx->mlem_exec) {
                cudaGraphExecDestroy(ctx->mlem_exec);
                ctx->mlem_exec = nullptr;
            }
            cudaGraph_t graph;
            CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            int64_t dummy = 0;
            cudaError_t le = launch_mlem_iteration((const float *)dA, rays, K, (const float *)dy,
                                                   (const float *)dc, dx, (float *)dpart, nparts,
                                                   (const double *)dsens, st, &dummy);
            cudaError_t ce = cudaStreamEndCapture(st, &graph);
            if (le != cudaSuccess) return fail(ctx, XRDT_ERR_CUDA, fmt("MLEM capture: %s", cudaGetErrorString(le)));
            CK(ce);
            cudaError_t ie = cudaGraphInstantiate(&ctx->mlem_exec, graph, 0);
            cudaGraphDestroy(graph);
            CK(ie);
            for (int i = 0; i < 6; i++) ctx->mlem_key[i] = key[i];
            ctx->mlem_rays = rays;
            ctx->mlem_K = K;
        }
        ProfScope ps(ctx, XRDT_KERNEL_MLEM);
        for (int it = 0; it < iters; it++) CK(cudaGraphLaunch(ctx->mlem_exec, st));
        ctx->launches += 2 * (int64_t)iters;
    }
    if (hostX) CK(cudaMemcpyAsync(x, dx, sizeof(float) * K, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return XRDT_OK;
}

} // extern "C"
