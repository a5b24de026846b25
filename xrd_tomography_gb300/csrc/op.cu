// op.cu -- C ABI of the per-voxel-coefficient operator (xrdt_op_*).
//
// An operator holds everything about one phantom and scanner that does not
// change between forward and adjoint calls: the bilinear attenuation cells,
// the non-empty voxels in the reference's loop order, the table of
// (source, pixel) pairs, the source-side line integrals and the per-energy
// tables.  The unknowns live in the compact voxel order [nv][NWT] on the
// device; calls convert from and to the full-grid layout [NX*NY][NWT].
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "ctx.h"

using namespace xrdt;

struct xrdt_op {
    xrdt_ctx *ctx = nullptr;
    xrdt_problem p;
    VoxOp v;
    std::vector<void *> allocs;
    int groups = 1;
    int64_t rays = 0;
    bool sens_ready = false;              // sens holds Av^T 1
    // device buffers
    int32_t *seg = nullptr;
    float *a1 = nullptr, *a2 = nullptr;
    float *xc = nullptr, *xd = nullptr;   // unknowns, compact; xd = x * dq
    float *what = nullptr;                // [pairs][E]
    float *part = nullptr;                // [groups][nv][NWT]
    double *sens = nullptr;               // [nv][NWT]
    float *xfull = nullptr;               // staging of the full-grid layout
    float *ray_a = nullptr, *ray_b = nullptr;   // staging of ray vectors
    // inputs of the FP64 kernel at the reference launch shape
    const SrcGeom *src = nullptr;
    float *spectrum = nullptr;
    double *coarse_qd = nullptr;          // [nwt] (centre, width) in double
    double *gd = nullptr;                 // [NX*NY*NWT] FP64 adjoint accumulator
    int64_t *rays_d = nullptr;            // staged ray list
    int64_t rays_cap = 0;
    // MLEM iteration as a graph, keyed by the ray vectors it reads
    cudaGraphExec_t mlem_exec = nullptr;
    const void *mlem_key[2] = {};
};

namespace {

int fail(xrdt_ctx *c, int status, const std::string &msg)
{
    if (c) c->err = msg;
    return status;
}

#define CK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return fail(ctx, XRDT_ERR_CUDA, fmt("%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                                               __LINE__));                                         \
    } while (0)

int op_alloc(xrdt_op *op, size_t bytes, void **out)
{
    void *p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes ? bytes : 16);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(op->ctx, XRDT_ERR_ALLOC, fmt("cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e)));
    }
    op->allocs.push_back(p);
    *out = p;
    return XRDT_OK;
}

template <class T>
int op_alloc_t(xrdt_op *op, size_t count, T **out)
{
    void *p;
    int rc = op_alloc(op, sizeof(T) * count, &p);
    if (rc == XRDT_OK) *out = (T *)p;
    return rc;
}

void op_free(xrdt_op *op)
{
    if (op->mlem_exec) cudaGraphExecDestroy(op->mlem_exec);
    for (void *p : op->allocs) cudaFree(p);
    op->allocs.clear();
}

// Positions of the sources (integrate_diffraction.cu:93-97), as api.cu builds them.
void src_geom_host(const xrdt_problem *p, int src, SrcGeom *g)
{
    const double phi = ((double)src / (double)p->n_src) * p->src_arc + p->src_phi0;
    g->sphi = sin(phi);
    g->cphi = cos(phi);
    g->Rsrc_x = p->cx + p->r_src * g->sphi;
    g->Rsrc_y = p->cy - p->r_src * g->cphi;
}

// Device view of a caller array: the pointer itself, or `stage` filled from it.
int view_in(xrdt_op *op, const float *src, size_t n, float *stage, const float **dev)
{
    xrdt_ctx *ctx = op->ctx;
    if (is_device_ptr(src)) {
        *dev = src;
        return XRDT_OK;
    }
    CK(cudaMemcpyAsync(stage, src, sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream));
    *dev = stage;
    return XRDT_OK;
}

int begin(xrdt_op *op)
{
    if (!op || !op->ctx) return XRDT_ERR_NULL;
    xrdt_ctx *ctx = op->ctx;
    ctx->err.clear();
    CK(cudaSetDevice(ctx->device));
    return XRDT_OK;
}

// Sensitivity Av^T 1, once per operator.
int ensure_sens(xrdt_op *op)
{
    xrdt_ctx *ctx = op->ctx;
    if (op->sens_ready) return XRDT_OK;
    cudaStream_t st = ctx->stream;
    {
        ProfScope ps(ctx, XRDT_KERNEL_VOX_UPDATE);
        CK(launch_vox_wtab(op->v, nullptr, op->what, st, &ctx->launches));
    }
    {
        ProfScope ps(ctx, XRDT_KERNEL_VOX_ADJOINT);
        CK(launch_vox_adjoint(op->v, op->what, op->part, op->groups, st, &ctx->launches));
    }
    {
        ProfScope ps(ctx, XRDT_KERNEL_VOX_UPDATE);
        CK(launch_vox_reduce(op->v, op->part, op->groups, 0, op->sens, nullptr, nullptr, nullptr, st,
                             &ctx->launches));
    }
    op->sens_ready = true;
    return XRDT_OK;
}

} // namespace

extern "C" {

int32_t xrdt_op_create(xrdt_ctx *ctx, const xrdt_problem *p, const float *spectrum, const int32_t *seg,
                       const float *a1, const float *a2, xrdt_op **out)
{
    if (!ctx || !out) return XRDT_ERR_NULL;
    *out = nullptr;
    ctx->err.clear();
    if (!p || !spectrum || !seg || !a1 || !a2) return fail(ctx, XRDT_ERR_NULL, "a required array pointer is NULL");
    int rc = xrdt_problem_validate(p);
    if (rc) return fail(ctx, rc, fmt("problem rejected: %s", xrdt_status_string(rc)));
    if (p->nwt > 1024) return fail(ctx, XRDT_ERR_UNSUPPORTED, "the operator takes NWT <= 1024");
    DevProblem P;
    std::string err;
    build_dev_problem(p, 0.f, 1.f, 0.f, 1.f, &P, &err);
    if (P.e_hi - P.e_lo + 1 > 128)
        return fail(ctx, XRDT_ERR_UNSUPPORTED, "more than 128 source energy bins in the windows");
    P.nq = 0;   // no Compton table: the operator models the coherent term only
    P.na = 0;
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;

    xrdt_op *op = new xrdt_op();
    op->ctx = ctx;
    op->p = *p;
    op->rays = xrdt_problem_rays(p);
    const int64_t nvox = (int64_t)p->nx * p->ny;
    const int64_t npairs = (int64_t)p->n_src * P.n_det;
    const int E = P.e_hi - P.e_lo + 1;
    const int K = p->nwt;
    auto bail = [&](int status) {
        cudaStreamSynchronize(st);
        op_free(op);
        delete op;
        return status;
    };

    // inputs
    std::vector<float> hspec((size_t)p->nrg_src * p->nrg_det);
    if ((rc = op_alloc_t(op, nvox, &op->seg)) || (rc = op_alloc_t(op, nvox, &op->a1)) ||
        (rc = op_alloc_t(op, nvox, &op->a2)))
        return bail(rc);
    cudaError_t e = cudaMemcpy(hspec.data(), spectrum, sizeof(float) * hspec.size(), cudaMemcpyDefault);
    if (e == cudaSuccess) e = cudaMemcpyAsync(op->seg, seg, sizeof(int32_t) * nvox, cudaMemcpyDefault, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(op->a1, a1, sizeof(float) * nvox, cudaMemcpyDefault, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(op->a2, a2, sizeof(float) * nvox, cudaMemcpyDefault, st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        fail(ctx, XRDT_ERR_CUDA, fmt("staging the operator inputs: %s", cudaGetErrorString(e)));
        return bail(XRDT_ERR_CUDA);
    }

    // voxel list, cells, pairs, source-side integrals
    PrepBuffers B;
    memset(&B, 0, sizeof B);
    SrcGeom *d_src;
    PairRec *d_pairs;
    if ((rc = op_alloc_t(op, 2 * (size_t)(p->nx + 1) * (p->ny + 1), &B.cells)) ||
        (rc = op_alloc_t(op, nvox, &B.vox_xy)) || (rc = op_alloc_t(op, nvox, &B.vox_mat)) ||
        (rc = op_alloc_t(op, 4, &B.counters)) || (rc = op_alloc_t(op, p->n_src, &d_src)))
        return bail(rc);
    void *pp;
    if ((rc = op_alloc(op, pair_rec_bytes() * npairs, &pp))) return bail(rc);
    d_pairs = (PairRec *)pp;
    std::vector<SrcGeom> hsg(p->n_src);
    for (int s = 0; s < p->n_src; s++) src_geom_host(p, s, &hsg[s]);
    e = cudaMemcpyAsync(d_src, hsg.data(), sizeof(SrcGeom) * p->n_src, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = launch_compact_voxels(P, op->seg, B, st, &ctx->launches);
    if (e == cudaSuccess) e = launch_prep_map(P, op->a1, op->a2, nullptr, B, st, &ctx->launches);
    if (e == cudaSuccess) e = launch_pair_table(P, d_src, d_pairs, st, &ctx->launches);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ctx->h_counters, B.counters, sizeof(int) * 2, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        fail(ctx, XRDT_ERR_CUDA, fmt("operator set-up: %s", cudaGetErrorString(e)));
        return bail(XRDT_ERR_CUDA);
    }
    const int nv = ctx->h_counters[0];
    if (ctx->h_counters[1]) {
        fail(ctx, XRDT_ERR_INPUT, fmt("segmentation holds a material id above n_mat = %d", p->n_mat));
        return bail(XRDT_ERR_INPUT);
    }
    if ((rc = op_alloc_t(op, (size_t)p->n_src * std::max(nv, 1), &B.atten_src))) return bail(rc);
    if (nv > 0 && (e = launch_src_atten(P, d_src, nv, B, st, &ctx->launches)) != cudaSuccess) {
        cudaGetLastError();
        fail(ctx, XRDT_ERR_CUDA, fmt("source-side integrals: %s", cudaGetErrorString(e)));
        return bail(XRDT_ERR_CUDA);
    }

    // per-energy tables
    HostTables ht;
    build_host_tables(p, P, hspec.data(), &ht);
    EnergyRow *d_energy;
    float *d_rf;
    int *d_wlo, *d_wn;
    float4 *d_cq;
    if ((rc = op_alloc_t(op, ht.energy.size(), &d_energy)) || (rc = op_alloc_t(op, ht.rf_win.size(), &d_rf)) ||
        (rc = op_alloc_t(op, ht.win_lo.size(), &d_wlo)) || (rc = op_alloc_t(op, ht.win_n.size(), &d_wn)) ||
        (rc = op_alloc_t(op, ht.coarse_q.size(), &d_cq)))
        return bail(rc);
    e = cudaMemcpyAsync(d_energy, ht.energy.data(), sizeof(EnergyRow) * ht.energy.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_rf, ht.rf_win.data(), sizeof(float) * ht.rf_win.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_wlo, ht.win_lo.data(), sizeof(int) * ht.win_lo.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_wn, ht.win_n.data(), sizeof(int) * ht.win_n.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_cq, ht.coarse_q.data(), sizeof(float4) * ht.coarse_q.size(), cudaMemcpyHostToDevice, st);

    op->src = d_src;
    {
        std::vector<double> cqd(2 * (size_t)K);
        for (int k = 0; k < K; k++) {
            const double NWT = (double)K;
            const double e1 = p->q_lo + (double)k * p->dq0 +
                              (p->q_hi - p->q_lo - p->dq0 * NWT) * (double)((int64_t)k * k) / (NWT * NWT);
            const double e2 = p->q_lo + (double)(k + 1) * p->dq0 +
                              (p->q_hi - p->q_lo - p->dq0 * NWT) * (double)((int64_t)(k + 1) * (k + 1)) / (NWT * NWT);
            cqd[2 * k] = 0.5 * (e1 + e2);
            cqd[2 * k + 1] = e2 - e1;
        }
        if ((rc = op_alloc_t(op, cqd.size(), &op->coarse_qd)) || (rc = op_alloc_t(op, hspec.size(), &op->spectrum)))
            return bail(rc);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(op->coarse_qd, cqd.data(), sizeof(double) * cqd.size(), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(op->spectrum, hspec.data(), sizeof(float) * hspec.size(), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);   // cqd leaves scope
    }
    op->v.P = P;
    op->v.nv = nv;
    op->v.pairs = d_pairs;
    op->v.energy = d_energy;
    op->v.rf_win = d_rf;
    op->v.win_lo = d_wlo;
    op->v.win_n = d_wn;
    op->v.coarse_q = d_cq;
    op->v.vox_xy = B.vox_xy;
    op->v.cells = B.cells;
    op->v.atten_src = B.atten_src;

    // work buffers
    int sms = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    if (e != cudaSuccess) {
        cudaGetLastError();
        fail(ctx, XRDT_ERR_CUDA, fmt("operator tables: %s", cudaGetErrorString(e)));
        return bail(XRDT_ERR_CUDA);
    }
    op->groups = vox_adj_groups(op->v, sms);
    const size_t nx_k = (size_t)std::max(nv, 1) * K;
    if ((rc = op_alloc_t(op, nx_k, &op->xc)) || (rc = op_alloc_t(op, nx_k, &op->xd)) ||
        (rc = op_alloc_t(op, (size_t)npairs * E, &op->what)) ||
        (rc = op_alloc_t(op, (size_t)op->groups * nx_k, &op->part)) || (rc = op_alloc_t(op, nx_k, &op->sens)) ||
        (rc = op_alloc_t(op, (size_t)nvox * K, &op->xfull)) || (rc = op_alloc_t(op, (size_t)op->rays, &op->ray_a)) ||
        (rc = op_alloc_t(op, (size_t)op->rays, &op->ray_b)))
        return bail(rc);
    int optin = 0;
    e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
    if (e == cudaSuccess && ((int64_t)(vox_fwd_smem(P) + vox_fwd_static_smem()) > optin ||
                           (int64_t)vox_adj_smem(P, vox_adj_warps(K)) > optin)) {
        fail(ctx, XRDT_ERR_UNSUPPORTED, "the problem's tables exceed the shared memory of one block");
        return bail(XRDT_ERR_UNSUPPORTED);
    }
    if (e == cudaSuccess) e = vox_set_attributes(optin);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        fail(ctx, XRDT_ERR_CUDA, fmt("operator set-up: %s", cudaGetErrorString(e)));
        return bail(XRDT_ERR_CUDA);
    }
    *out = op;
    return XRDT_OK;
}

int32_t xrdt_op_destroy(xrdt_op *op)
{
    if (!op) return XRDT_ERR_NULL;
    if (op->ctx) {
        cudaSetDevice(op->ctx->device);
        cudaStreamSynchronize(op->ctx->stream);
    }
    op_free(op);
    delete op;
    return XRDT_OK;
}

int64_t xrdt_op_voxels(const xrdt_op *op) { return op ? (int64_t)op->v.nv : -1; }

int32_t xrdt_op_forward(xrdt_op *op, const float *x, float *y, uint32_t flags)
{
    int rc = begin(op);
    if (rc) return rc;
    xrdt_ctx *ctx = op->ctx;
    if (!x || !y) return fail(ctx, XRDT_ERR_NULL, "x and y are required");
    if (flags) return fail(ctx, XRDT_ERR_UNSUPPORTED, "unknown flag bits");
    cudaStream_t st = ctx->stream;
    const int K = op->p.nwt;
    const size_t nfull = (size_t)op->p.nx * op->p.ny * K;
    const bool hostY = !is_device_ptr(y);
    float *dy = hostY ? op->ray_a : y;
    if (op->v.nv == 0) {
        CK(cudaMemsetAsync(dy, 0, sizeof(float) * op->rays, st));
    } else {
        const float *dx;
        if ((rc = view_in(op, x, nfull, op->xfull, &dx))) return rc;
        {
            ProfScope ps(ctx, XRDT_KERNEL_VOX_UPDATE);
            CK(launch_vox_gather(op->v, dx, nullptr, op->xd, st, &ctx->launches));
        }
        ProfScope ps(ctx, XRDT_KERNEL_VOX_FORWARD);
        CK(launch_vox_forward(op->v, op->xd, dy, nullptr, nullptr, nullptr, st, &ctx->launches));
    }
    if (hostY) CK(cudaMemcpyAsync(y, dy, sizeof(float) * op->rays, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return XRDT_OK;
}

int32_t xrdt_op_adjoint(xrdt_op *op, const float *w, float *g, uint32_t flags)
{
    int rc = begin(op);
    if (rc) return rc;
    xrdt_ctx *ctx = op->ctx;
    if (!w || !g) return fail(ctx, XRDT_ERR_NULL, "w and g are required");
    if (flags) return fail(ctx, XRDT_ERR_UNSUPPORTED, "unknown flag bits");
    cudaStream_t st = ctx->stream;
    const int K = op->p.nwt;
    const size_t nfull = (size_t)op->p.nx * op->p.ny * K;
    const bool hostG = !is_device_ptr(g);
    float *dg = hostG ? op->xfull : g;
    CK(cudaMemsetAsync(dg, 0, sizeof(float) * nfull, st));
    if (op->v.nv > 0) {
        const float *dw;
        if ((rc = view_in(op, w, op->rays, op->ray_a, &dw))) return rc;
        {
            ProfScope ps(ctx, XRDT_KERNEL_VOX_UPDATE);
            CK(launch_vox_wtab(op->v, dw, op->what, st, &ctx->launches));
        }
        {
            ProfScope ps(ctx, XRDT_KERNEL_VOX_ADJOINT);
            CK(launch_vox_adjoint(op->v, op->what, op->part, op->groups, st, &ctx->launches));
        }
        ProfScope ps(ctx, XRDT_KERNEL_VOX_UPDATE);
        CK(launch_vox_reduce(op->v, op->part, op->groups, 2, nullptr, nullptr, nullptr, dg, st, &ctx->launches));
    }
    if (hostG) CK(cudaMemcpyAsync(g, dg, sizeof(float) * nfull, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return XRDT_OK;
}

} // extern "C"

namespace {

// Stages a host ray list, checking each index.
int stage_rays(xrdt_op *op, const int64_t *rays, int64_t n_rays)
{
    xrdt_ctx *ctx = op->ctx;
    if (n_rays < 0 || n_rays > 2147483647LL) return fail(ctx, XRDT_ERR_DIMS, "bad ray count");
    if (n_rays && !rays) return fail(ctx, XRDT_ERR_NULL, "ray list is NULL");
    if (n_rays && is_device_ptr(rays)) return fail(ctx, XRDT_ERR_UNSUPPORTED, "the ray list must be host memory");
    for (int64_t i = 0; i < n_rays; i++)
        if (rays[i] < 0 || rays[i] >= op->rays)
            return fail(ctx, XRDT_ERR_INPUT, fmt("ray %lld out of range", (long long)rays[i]));
    if (n_rays > op->rays_cap) {
        int rc = op_alloc_t(op, (size_t)n_rays, &op->rays_d);
        if (rc) return rc;
        op->rays_cap = n_rays;
    }
    if (n_rays) CK(cudaMemcpyAsync(op->rays_d, rays, sizeof(int64_t) * n_rays, cudaMemcpyHostToDevice, ctx->stream));
    return XRDT_OK;
}

int plain_ok(xrdt_op *op, uint32_t flags)
{
    if (flags != XRDT_OP_PLAIN_FP64)
        return fail(op->ctx, XRDT_ERR_UNSUPPORTED, "ray-list calls run the FP64 kernel: pass XRDT_OP_PLAIN_FP64");
    if (op->p.nwt % 32 != 0 || op->p.nwt > 1024)
        return fail(op->ctx, XRDT_ERR_UNSUPPORTED, "the reference launch shape needs NWT a multiple of 32, <= 1024");
    return XRDT_OK;
}

__global__ void k_double_to_float(const double *__restrict__ a, float *__restrict__ b, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

} // namespace

extern "C" {

int32_t xrdt_op_forward_rays(xrdt_op *op, const float *x, const int64_t *rays, int64_t n_rays, float *y,
                             uint32_t flags)
{
    int rc = begin(op);
    if (rc) return rc;
    xrdt_ctx *ctx = op->ctx;
    if (!x || !y) return fail(ctx, XRDT_ERR_NULL, "x and y are required");
    if ((rc = plain_ok(op, flags)) || (rc = stage_rays(op, rays, n_rays))) return rc;
    cudaStream_t st = ctx->stream;
    const size_t nfull = (size_t)op->p.nx * op->p.ny * op->p.nwt;
    const float *dx;
    if ((rc = view_in(op, x, nfull, op->xfull, &dx))) return rc;
    const bool hostY = !is_device_ptr(y);
    float *dy = hostY ? op->ray_a : y;   // n_rays <= rays
    {
        ProfScope ps(ctx, XRDT_KERNEL_PLAIN);
        CK(launch_plain_vox(op->v.P, op->src, op->spectrum, op->seg, op->a1, op->a2, op->coarse_qd, op->rays_d,
                            n_rays, dx, dy, nullptr, nullptr, st, &ctx->launches));
    }
    if (hostY && n_rays) CK(cudaMemcpyAsync(y, dy, sizeof(float) * n_rays, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return XRDT_OK;
}

int32_t xrdt_op_adjoint_rays(xrdt_op *op, const float *w, const int64_t *rays, int64_t n_rays, float *g,
                             uint32_t flags)
{
    int rc = begin(op);
    if (rc) return rc;
    xrdt_ctx *ctx = op->ctx;
    if (!w || !g) return fail(ctx, XRDT_ERR_NULL, "w and g are required");
    if ((rc = plain_ok(op, flags)) || (rc = stage_rays(op, rays, n_rays))) return rc;
    cudaStream_t st = ctx->stream;
    const size_t nfull = (size_t)op->p.nx * op->p.ny * op->p.nwt;
    if (!op->gd && (rc = op_alloc_t(op, nfull, &op->gd))) return rc;
    const float *dw;
    if ((rc = view_in(op, w, (size_t)n_rays, op->ray_a, &dw))) return rc;
    const bool hostG = !is_device_ptr(g);
    float *dg = hostG ? op->xfull : g;
    CK(cudaMemsetAsync(op->gd, 0, sizeof(double) * nfull, st));
    {
        ProfScope ps(ctx, XRDT_KERNEL_PLAIN);
        CK(launch_plain_vox(op->v.P, op->src, op->spectrum, op->seg, op->a1, op->a2, op->coarse_qd, op->rays_d,
                            n_rays, nullptr, nullptr, dw, op->gd, st, &ctx->launches));
    }
    k_double_to_float<<<256, 256, 0, st>>>(op->gd, dg, (int64_t)nfull);
    CK(cudaGetLastError());
    ctx->launches++;
    if (hostG) CK(cudaMemcpyAsync(g, dg, sizeof(float) * nfull, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return XRDT_OK;
}


int32_t xrdt_op_mlem(xrdt_op *op, const float *y, const float *c, float *x, int32_t iters, uint32_t flags)
{
    int rc = begin(op);
    if (rc) return rc;
    xrdt_ctx *ctx = op->ctx;
    if (!y || !c || !x) return fail(ctx, XRDT_ERR_NULL, "y, c and x are required");
    if (iters < 0) return fail(ctx, XRDT_ERR_DIMS, "iters must be >= 0");
    if (flags) return fail(ctx, XRDT_ERR_UNSUPPORTED, "unknown flag bits");
    cudaStream_t st = ctx->stream;
    const int K = op->p.nwt;
    const size_t nfull = (size_t)op->p.nx * op->p.ny * K;
    if (iters == 0) return XRDT_OK;
    const bool hostX = !is_device_ptr(x);
    float *dx = hostX ? op->xfull : x;
    if (hostX) CK(cudaMemcpyAsync(dx, x, sizeof(float) * nfull, cudaMemcpyHostToDevice, st));
    if (op->v.nv > 0) {
        const float *dy, *dc;
        if ((rc = view_in(op, y, op->rays, op->ray_a, &dy))) return rc;
        if ((rc = view_in(op, c, op->rays, op->ray_b, &dc))) return rc;
        if ((rc = ensure_sens(op))) return rc;
        {
            ProfScope ps(ctx, XRDT_KERNEL_VOX_UPDATE);
            CK(launch_vox_gather(op->v, dx, op->xc, op->xd, st, &ctx->launches));
        }
        const void *key[2] = {dy, dc};
        if (!op->mlem_exec || op->mlem_key[0] != key[0] || op->mlem_key[1] != key[1]) {
            if (op->mlem_exec) {
                cudaGraphExecDestroy(op->mlem_exec);
                op->mlem_exec = nullptr;
            }
            cudaGraph_t graph;
            CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            int64_t dummy = 0;
            cudaError_t le = launch_vox_forward(op->v, op->xd, nullptr, dy, dc, op->what, st, &dummy);
            if (le == cudaSuccess) le = launch_vox_adjoint(op->v, op->what, op->part, op->groups, st, &dummy);
            if (le == cudaSuccess)
                le = launch_vox_reduce(op->v, op->part, op->groups, 1, op->sens, op->xc, op->xd, nullptr, st, &dummy);
            cudaError_t ce = cudaStreamEndCapture(st, &graph);
            if (le != cudaSuccess) {
                if (ce == cudaSuccess) cudaGraphDestroy(graph);
                cudaGetLastError();
                return fail(ctx, XRDT_ERR_CUDA, fmt("MLEM capture: %s", cudaGetErrorString(le)));
            }
            CK(ce);
            cudaError_t ie = cudaGraphInstantiate(&op->mlem_exec, graph, 0);
            cudaGraphDestroy(graph);
            CK(ie);
            op->mlem_key[0] = key[0];
            op->mlem_key[1] = key[1];
        }
        {
            ProfScope ps(ctx, XRDT_KERNEL_VOX_FORWARD);   // the whole iteration (three kernels)
            for (int it = 0; it < iters; it++) CK(cudaGraphLaunch(op->mlem_exec, st));
        }
        ctx->launches += 3 * (int64_t)iters;
        // empty voxels have no sensitivity: the update sets them to 0
        CK(cudaMemsetAsync(dx, 0, sizeof(float) * nfull, st));
        ProfScope ps(ctx, XRDT_KERNEL_VOX_UPDATE);
        CK(launch_vox_scatter(op->v, op->xc, dx, st, &ctx->launches));
    } else {
        CK(cudaMemsetAsync(dx, 0, sizeof(float) * nfull, st));
    }
    if (hostX) CK(cudaMemcpyAsync(x, dx, sizeof(float) * nfull, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return XRDT_OK;
}

} // extern "C"
