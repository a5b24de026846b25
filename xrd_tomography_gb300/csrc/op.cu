// op.cu -- C ABI of the per-voxel-coefficient operator (xrdt_op_*), of
// batches of operators (xrdt_batch_*) and of the dense-basis operator
// (xrdt_bop_*).
//
// An operator holds everything about one phantom and scanner that does not
// change between forward and adjoint calls: the bilinear attenuation cells,
// the non-empty voxels in the reference's loop order, the table of
// (source, pixel) pairs, the source-side line integrals, the per-energy
// tables and, when it fits, the detector-side integrals of every (pair,
// voxel).  The unknowns live in the compact voxel order [nv][NWT] on the
// device; calls convert from and to the full-grid layout [NX*NY][NWT].
//
// Calls run through a Plan: the batch's job descriptors and work offsets,
// the autotuned adjoint split, and -- for operators without a table of
// their own -- the tiles of whole pixels whose detector-side integrals are
// walked into a shared buffer inside each call (the forward, the adjoint
// and each MLEM iteration walk every tile once).  Each MLEM iteration of a
// plan is one CUDA graph.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "ctx.h"

using namespace xrdt;

struct xrdt_op {
    xrdt_ctx *ctx = nullptr;
    xrdt_problem p;
    VoxOp v;
    std::vector<void *> allocs;
    int groups_cap = 1;                   // rows of part: the most adjoint pair groups
    int64_t rays = 0;
    int64_t walk_bytes = 0;               // kept detector-side integrals
    bool sens_ready = false;              // sens holds Av^T 1
    // device buffers
    int32_t *seg = nullptr;
    float *a1 = nullptr, *a2 = nullptr;
    float *xc = nullptr, *xd = nullptr;   // unknowns, compact; xd = x * dq
    float *what = nullptr;                // [pairs][E]
    float2 *part = nullptr;               // [groups][nv][NWT] as float pairs
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
    struct Plan *plan = nullptr;          // the operator as a batch of one (created on first use)
};

// A batch of operators as the kernels see it: the job descriptors (a pinned
// host mirror and its device copy), the work offsets, the adjoint split and
// the persistent grids, and the MLEM iteration captured as a graph.
struct Plan {
    xrdt_ctx *ctx = nullptr;
    std::vector<xrdt_op *> ops;
    VoxJob *jobs_h = nullptr;
    VoxJob *jobs_d = nullptr;
    int64_t *off_d = nullptr;
    unsigned long long *counters_d = nullptr;
    std::vector<int64_t> off;          // 5 x (n + 1)
    int sms = 0;
    int adj_warps = 1;
    int64_t adj_tiles = 0;             // target number of adjoint tiles
    int fwd_grid = 1, adj_grid = 1;
    size_t fwd_smem = 0, adj_smem = 0;
    bool tuned = false;
    cudaGraphExec_t mlem_exec = nullptr;
    int64_t mlem_cfg[3] = {};          // adj_warps, adj_tiles, fwd_grid of the captured graph
    int64_t mlem_launches = 0;         // kernels in one iteration's graph
    // Streaming: operators that keep no detector-side table of their own have
    // their pairs cut into segments whose tables are walked, tile by tile,
    // into one shared buffer within every call; each tile is then projected
    // and back-projected before the next one is walked.
    struct Seg {
        int op;
        int64_t p0, p1;      // pairs [p0, p1) of the operator
        int64_t woff;        // first float2 of its rows in walkbuf; -1: the operator's own table
    };
    struct Tile {
        std::vector<Seg> segs;
        VoxJob *jobs_h = nullptr, *jobs_d = nullptr;
        int64_t *off_d = nullptr;
        std::vector<int64_t> off;   // 5 x (segments + 1), rows 0 and 1 used
    };
    bool streamed = false;
    int64_t tile_budget = 0;           // bytes of walkbuf
    std::vector<Tile> tiles;
    float2 *walkbuf = nullptr;
    std::vector<int> rows;             // partial-sum rows each operator's tiles use
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
    if (test_alloc_fails())
        return fail(op->ctx, XRDT_ERR_ALLOC, fmt("cudaMalloc(%zu bytes): failure injected", bytes));
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

void plan_free(Plan *pl)
{
    if (!pl) return;
    for (Plan::Tile &t : pl->tiles) {
        if (t.jobs_h) cudaFreeHost(t.jobs_h);
        if (t.jobs_d) cudaFree(t.jobs_d);
        if (t.off_d) cudaFree(t.off_d);
    }
    if (pl->walkbuf) cudaFree(pl->walkbuf);
    if (pl->mlem_exec) cudaGraphExecDestroy(pl->mlem_exec);
    if (pl->jobs_h) cudaFreeHost(pl->jobs_h);
    if (pl->jobs_d) cudaFree(pl->jobs_d);
    if (pl->off_d) cudaFree(pl->off_d);
    if (pl->counters_d) cudaFree(pl->counters_d);
    delete pl;
}

void op_free(xrdt_op *op)
{
    plan_free(op->plan);
    op->plan = nullptr;
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

// ---- plans ------------------------------------------------------------------

int64_t pairs_of(const xrdt_op *op) { return (int64_t)op->p.n_src * op->v.P.n_det; }
int chunks_of(const xrdt_op *op) { return (op->v.nv + 31) / 32; }

// Adjoint split for a warps-per-block count and a target tile count: one
// pairs-per-group for the whole batch, so that tiles carry similar work.
void plan_split(Plan *pl, int warps, int64_t tiles)
{
    const int n = (int)pl->ops.size();
    double work = 0.0;   // sum of chunk blocks x pairs
    for (int i = 0; i < n; i++) {
        const int cb = (chunks_of(pl->ops[i]) + warps - 1) / warps;
        work += (double)cb * (double)pairs_of(pl->ops[i]);
    }
    int64_t ppg = (int64_t)std::ceil(work / (double)std::max<int64_t>(tiles, 1));
    if (ppg < 1) ppg = 1;
    pl->off.assign(5 * (size_t)(n + 1), 0);
    size_t smem = 0;
    for (int i = 0; i < n; i++) {
        const xrdt_op *op = pl->ops[i];
        VoxJob &J = pl->jobs_h[i];
        const int64_t np = pairs_of(op);
        J.chunk_blocks = std::max(1, (chunks_of(op) + warps - 1) / warps);
        int64_t g = (np + ppg - 1) / ppg;
        if (g > op->groups_cap) g = op->groups_cap;
        if (g < 1) g = 1;
        J.groups = (int)g;
        J.ppg = (int)((np + g - 1) / g);
        int64_t *o = pl->off.data();
        const int N1 = n + 1;
        o[0 * N1 + i + 1] = o[0 * N1 + i] + np;
        o[1 * N1 + i + 1] = o[1 * N1 + i] + (op->v.nv > 0 ? (int64_t)J.chunk_blocks * J.groups : 0);
        o[2 * N1 + i + 1] = o[2 * N1 + i] + (int64_t)op->v.nv * op->p.nwt;
        o[3 * N1 + i + 1] = o[3 * N1 + i] + (int64_t)op->p.nx * op->p.ny * op->p.nwt;
        o[4 * N1 + i + 1] = o[4 * N1 + i] + np * J.E;
        smem = std::max(smem, vox_adj_smem(op->v.P, warps));
    }
    pl->adj_warps = warps;
    pl->adj_tiles = tiles;
    pl->adj_smem = smem;
    const int bps = vox_adj_blocks_per_sm(warps, smem);
    int64_t items = pl->off[1 * (size_t)(n + 1) + n];
    if (pl->streamed) {
        // each tile's segments split their pairs with the batch's pairs per
        // group, capped at the operator's partial-sum rows; the reduction
        // adds the rows any tile of the operator used
        pl->rows.assign(n, 1);
        items = 0;
        for (Plan::Tile &t : pl->tiles) {
            const int ns = (int)t.segs.size();
            t.off.assign(5 * (size_t)(ns + 1), 0);
            for (int k = 0; k < ns; k++) {
                const Plan::Seg &sg = t.segs[k];
                const xrdt_op *op = pl->ops[sg.op];
                VoxJob J = pl->jobs_h[sg.op];
                const int64_t len = sg.p1 - sg.p0;
                int64_t g = std::min<int64_t>((len + ppg - 1) / ppg, op->groups_cap);
                if (g < 1) g = 1;
                J.groups = (int)g;
                J.ppg = (int)((len + g - 1) / g);
                J.pair0 = sg.p0;
                J.pair1 = sg.p1;
                J.accumulate = 1;
                J.op.walk = sg.woff < 0 ? op->v.walk : pl->walkbuf + sg.woff;
                t.jobs_h[k] = J;
                pl->rows[sg.op] = std::max(pl->rows[sg.op], (int)g);
                t.off[0 * (ns + 1) + k + 1] = t.off[0 * (ns + 1) + k] + len;
                t.off[1 * (ns + 1) + k + 1] = t.off[1 * (ns + 1) + k] + (op->v.nv > 0 ? (int64_t)J.chunk_blocks * g : 0);
            }
            items = std::max(items, t.off[1 * (ns + 1) + ns]);
        }
        for (int i = 0; i < n; i++) pl->jobs_h[i].groups = pl->rows[i];
    }
    pl->adj_grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)pl->sms * bps, items));
}

int plan_upload(Plan *pl)
{
    xrdt_ctx *ctx = pl->ctx;
    const size_t n = pl->ops.size();
    CK(cudaMemcpyAsync(pl->jobs_d, pl->jobs_h, sizeof(VoxJob) * n, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(pl->off_d, pl->off.data(), sizeof(int64_t) * pl->off.size(), cudaMemcpyHostToDevice,
                       ctx->stream));
    for (Plan::Tile &t : pl->tiles) {
        // the tile's descriptors carry the per-call pointers of their problems
        for (size_t k = 0; k < t.segs.size(); k++) {
            const VoxJob &M = pl->jobs_h[t.segs[k].op];
            VoxJob &J = t.jobs_h[k];
            J.xd = M.xd; J.xc = M.xc; J.y = M.y; J.ymeas = M.ymeas; J.cbg = M.cbg; J.what = M.what;
            J.part = M.part; J.sens = M.sens; J.g = M.g; J.w = M.w; J.xfull = M.xfull; J.xout = M.xout;
        }
        CK(cudaMemcpyAsync(t.jobs_d, t.jobs_h, sizeof(VoxJob) * t.segs.size(), cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(t.off_d, t.off.data(), sizeof(int64_t) * t.off.size(), cudaMemcpyHostToDevice,
                           ctx->stream));
    }
    return XRDT_OK;
}

VoxBatch tile_batch(const Plan *pl, const Plan::Tile &t)
{
    VoxBatch B;
    B.jobs = t.jobs_d;
    B.off = t.off_d;
    B.counters = pl->counters_d;
    B.n = (int)t.segs.size();
    B.adj_warps = pl->adj_warps;
    return B;
}

int64_t tile_items(const Plan::Tile &t, int row) { return t.off[(size_t)row * (t.segs.size() + 1) + t.segs.size()]; }

// Walks the detector-side tables of a tile's segments into the shared buffer.
cudaError_t tile_walks(const Plan *pl, const Plan::Tile &t, cudaStream_t st, int64_t *launches)
{
    for (const Plan::Seg &sg : t.segs) {
        if (sg.woff < 0) continue;
        const xrdt_op *op = pl->ops[sg.op];
        cudaError_t e = launch_det_walk(op->v.P, op->src, nullptr, sg.p0, sg.p1 - sg.p0, op->v.vox_xy, op->v.nv,
                                        op->v.cells, pl->walkbuf + sg.woff, st, launches);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// Clears the partial-sum rows the tiles add to.
cudaError_t zero_rows(const Plan *pl, cudaStream_t st)
{
    for (size_t i = 0; i < pl->ops.size(); i++) {
        const xrdt_op *op = pl->ops[i];
        if (op->v.nv == 0) continue;
        cudaError_t e = cudaMemsetAsync(op->part, 0, sizeof(float2) * (size_t)pl->rows[i] * op->v.nv * op->p.nwt, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// The adjoint of every tile (after its walks) into the cleared partial rows;
// what[] must hold the per-energy weights of all pairs.
cudaError_t stream_adjoint(Plan *pl, cudaStream_t st, int64_t *launches)
{
    cudaError_t e = zero_rows(pl, st);
    for (const Plan::Tile &t : pl->tiles) {
        if (e == cudaSuccess) e = tile_walks(pl, t, st, launches);
        const int64_t items = tile_items(t, 1);
        if (e == cudaSuccess && items > 0)
            e = launch_vox_adjoint(tile_batch(pl, t), (int)std::min<int64_t>(pl->adj_grid, items), pl->adj_smem, st,
                                   launches);
    }
    return e;
}

// The forward of every tile (after its walks); MLEM: with the ratios and
// per-energy weights, then the tile's adjoint, so a tile's table is walked
// once per iteration.
cudaError_t stream_forward(Plan *pl, bool mlem, cudaStream_t st, int64_t *launches)
{
    cudaError_t e = mlem ? zero_rows(pl, st) : cudaSuccess;
    for (const Plan::Tile &t : pl->tiles) {
        if (e == cudaSuccess) e = tile_walks(pl, t, st, launches);
        const int64_t fi = tile_items(t, 0), ai = tile_items(t, 1);
        if (e == cudaSuccess && fi > 0)
            e = launch_vox_forward(tile_batch(pl, t), mlem, (int)std::min<int64_t>(pl->fwd_grid, fi), pl->fwd_smem,
                                   st, launches);
        if (mlem && e == cudaSuccess && ai > 0)
            e = launch_vox_adjoint(tile_batch(pl, t), (int)std::min<int64_t>(pl->adj_grid, ai), pl->adj_smem, st,
                                   launches);
    }
    return e;
}

VoxBatch plan_batch(const Plan *pl)
{
    VoxBatch B;
    B.jobs = pl->jobs_d;
    B.off = pl->off_d;
    B.counters = pl->counters_d;
    B.n = (int)pl->ops.size();
    B.adj_warps = pl->adj_warps;
    return B;
}

int64_t plan_total(const Plan *pl, int row) { return pl->off[(size_t)row * (pl->ops.size() + 1) + pl->ops.size()]; }

// Cuts the pairs of the operators without a table of their own into
// segments of whole pixels (every view) and packs them, in operator order,
// into tiles whose tables fit the walk buffer.  The buffer holds a quarter of
// the free device memory, at most 8 GiB, or XRDT_WALK_TILE_BYTES when that is
// set; one pixel column of the largest phantom is the least it holds.
// Operators that keep a table ride along in the first tile.
int plan_make_tiles(Plan *pl)
{
    xrdt_ctx *ctx = pl->ctx;
    int64_t budget = 0;
    const char *tb = getenv("XRDT_WALK_TILE_BYTES");
    if (tb && *tb) budget = atoll(tb);
    if (budget <= 0) {
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
            cudaGetLastError();
            fr = 0;
        }
        budget = std::min<int64_t>((int64_t)(fr / 4), (int64_t)8 << 30);
    }
    for (const xrdt_op *op : pl->ops)
        if (op->v.nv > 0 && !op->v.walk)
            budget = std::max<int64_t>(budget, (int64_t)sizeof(float2) * op->p.n_src * op->v.nv);
    pl->tile_budget = budget;
    const int64_t cap = budget / (int64_t)sizeof(float2);   // float2 rows of the buffer
    pl->tiles.clear();
    pl->tiles.emplace_back();
    int64_t used = 0, most = 0;
    for (int i = 0; i < (int)pl->ops.size(); i++) {
        const xrdt_op *op = pl->ops[i];
        const int64_t np = pairs_of(op), nv = op->v.nv;
        if (nv == 0) continue;
        if (op->v.walk) {
            pl->tiles.front().segs.push_back({i, 0, np, -1});
            continue;
        }
        const int64_t unit = op->p.n_src;   // whole pixels of every view
        const int64_t seg = std::max<int64_t>(unit, cap / nv / unit * unit);
        for (int64_t p0 = 0; p0 < np; p0 += seg) {
            const int64_t len = std::min(seg, np - p0);
            if (used > 0 && used + len * nv > cap) {
                pl->tiles.emplace_back();
                used = 0;
            }
            pl->tiles.back().segs.push_back({i, p0, p0 + len, used});
            used += len * nv;
            most = std::max(most, used);
        }
    }
    cudaError_t e = test_alloc_fails() ? cudaErrorMemoryAllocation
                                       : cudaMalloc((void **)&pl->walkbuf, sizeof(float2) * (size_t)std::max<int64_t>(most, 1));
    for (Plan::Tile &t : pl->tiles) {
        const size_t ns = std::max<size_t>(t.segs.size(), 1);
        if (e == cudaSuccess) e = cudaMallocHost((void **)&t.jobs_h, sizeof(VoxJob) * ns);
        if (e == cudaSuccess) e = cudaMalloc((void **)&t.jobs_d, sizeof(VoxJob) * ns);
        if (e == cudaSuccess) e = cudaMalloc((void **)&t.off_d, sizeof(int64_t) * 5 * (ns + 1));
        if (e == cudaSuccess) memset(t.jobs_h, 0, sizeof(VoxJob) * ns);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, XRDT_ERR_ALLOC, fmt("walk tiles: %s", cudaGetErrorString(e)));
    }
    return XRDT_OK;
}

int plan_create(xrdt_ctx *ctx, xrdt_op *const *ops, int n, Plan **out)
{
    Plan *pl = new Plan();
    pl->ctx = ctx;
    pl->ops.assign(ops, ops + n);
    cudaError_t e = test_alloc_fails() ? cudaErrorMemoryAllocation
                                       : cudaMallocHost((void **)&pl->jobs_h, sizeof(VoxJob) * n);
    if (e == cudaSuccess) e = cudaMalloc((void **)&pl->jobs_d, sizeof(VoxJob) * n);
    if (e == cudaSuccess) e = cudaMalloc((void **)&pl->off_d, sizeof(int64_t) * 5 * (n + 1));
    if (e == cudaSuccess) e = cudaMalloc((void **)&pl->counters_d, sizeof(unsigned long long) * 2);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&pl->sms, cudaDevAttrMultiProcessorCount, ctx->device);
    if (e != cudaSuccess) {
        cudaGetLastError();
        plan_free(pl);
        return fail(ctx, XRDT_ERR_ALLOC, fmt("batch set-up: %s", cudaGetErrorString(e)));
    }
    memset(pl->jobs_h, 0, sizeof(VoxJob) * n);
    size_t fsmem = 0;
    for (int i = 0; i < n; i++) {
        xrdt_op *op = ops[i];
        VoxJob &J = pl->jobs_h[i];
        J.op = op->v;
        J.c = make_f32_consts(op->v.P);
        J.E = op->v.P.e_hi - op->v.P.e_lo + 1;
        J.xd = op->xd;
        J.xc = op->xc;
        J.what = op->what;
        J.part = op->part;
        J.sens = op->sens;
        J.pair0 = 0;
        J.pair1 = pairs_of(op);
        J.accumulate = 0;
        fsmem = std::max(fsmem, vox_fwd_smem(op->v.P));
        if (op->v.nv > 0 && !op->v.walk) pl->streamed = true;
    }
    pl->fwd_smem = fsmem;
    if (pl->streamed) {
        int rc = plan_make_tiles(pl);
        if (rc) {
            plan_free(pl);
            return rc;
        }
    }
    // the widest adjoint block the shared memory allows
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
    int warps = 4;
    for (; warps > 1; warps /= 2) {
        size_t sm = 0;
        for (int i = 0; i < n; i++) sm = std::max(sm, vox_adj_smem(ops[i]->v.P, warps));
        if ((int64_t)(sm + vox_adj_static_smem()) <= optin) break;
    }
    plan_split(pl, warps, (int64_t)pl->sms * 4 * vox_adj_blocks_per_sm(warps, 0));
    const int64_t items = plan_total(pl, 0);
    pl->fwd_grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)pl->sms * vox_fwd_blocks_per_sm(fsmem), items));
    *out = pl;
    return XRDT_OK;
}

// Sensitivity Av^T 1 of every operator of the plan that has none yet.
int plan_sens(Plan *pl)
{
    xrdt_ctx *ctx = pl->ctx;
    bool all = true;
    for (xrdt_op *op : pl->ops) all = all && op->sens_ready;
    if (all) return XRDT_OK;
    int rc = plan_upload(pl);
    if (rc) return rc;
    const VoxBatch B = plan_batch(pl);
    cudaStream_t st = ctx->stream;
    // Av^T 1 in two parts: the weights of ones rounded to float, then what
    // that rounding dropped (k_vox_wtab), added in FP64
    for (int part = 0; part < 2; part++) {
        {
            ProfScope ps(ctx, XRDT_KERNEL_VOX_UPDATE);
            CK(launch_vox_wtab(B, plan_total(pl, 4), 1 + part, st, &ctx->launches));
        }
        if (pl->streamed) {
            ProfScope ps(ctx, XRDT_KERNEL_VOX_ADJOINT);
            CK(stream_adjoint(pl, st, &ctx->launches));
        } else {
            ProfScope ps(ctx, XRDT_KERNEL_VOX_ADJOINT);
            CK(launch_vox_adjoint(B, pl->adj_grid, pl->adj_smem, st, &ctx->launches));
        }
        {
            ProfScope ps(ctx, XRDT_KERNEL_VOX_UPDATE);
            CK(launch_vox_reduce(B, plan_total(pl, 2), part ? 4 : 0, st, &ctx->launches));
        }
    }
    for (xrdt_op *op : pl->ops) op->sens_ready = true;
    return XRDT_OK;
}

// ---- the autotuner's cache on disk ----------------------------------------
// One line per tuned batch: "<key> <warps> <tiles>".  The key names the GPU
// and every problem's sizes, so a cached choice is reused only for the same
// shapes on the same kind of GPU.  XRDT_TUNE_CACHE names the file ("" turns
// the cache off); by default it is $XDG_CACHE_HOME/xrdt/tune.txt or
// $HOME/.cache/xrdt/tune.txt.

std::string tune_cache_path()
{
    const char *e = getenv("XRDT_TUNE_CACHE");
    if (e) return std::string(e);
    const char *x = getenv("XDG_CACHE_HOME");
    const char *h = getenv("HOME");
    std::string dir = x && *x ? std::string(x) : (h && *h ? std::string(h) + "/.cache" : std::string());
    if (dir.empty()) return std::string();
    mkdir(dir.c_str(), 0755);
    dir += "/xrdt";
    mkdir(dir.c_str(), 0755);
    return dir + "/tune.txt";
}

std::string tune_key(const Plan *pl)
{
    cudaDeviceProp prop;
    std::string key;
    if (cudaGetDeviceProperties(&prop, pl->ctx->device) == cudaSuccess) {
        for (const char *c = prop.name; *c; c++) key += (*c == ' ') ? '_' : *c;
        key += fmt("-sm%d", prop.multiProcessorCount);
    } else {
        cudaGetLastError();
        key = "gpu";
    }
    for (const xrdt_op *op : pl->ops)
        key += fmt("|%dx%d,v%d,s%d,d%d,e%d,k%d", op->p.nx, op->p.ny, op->v.nv, op->p.n_src, op->v.P.n_det,
                   op->v.P.e_hi - op->v.P.e_lo + 1, op->p.nwt);
    if (pl->streamed) key += fmt("|tiles%lld", (long long)pl->tile_budget);
    return key;
}

bool tune_cache_get(const std::string &path, const std::string &key, int *warps, int64_t *tiles)
{
    if (path.empty()) return false;
    FILE *f = fopen(path.c_str(), "r");
    if (!f) return false;
    bool found = false;
    std::string line;
    char buf[4096];
    while (fgets(buf, sizeof buf, f)) {
        line = buf;
        const size_t sp = line.find(' ');
        if (sp == std::string::npos || line.compare(0, sp, key) != 0 || sp != key.size()) continue;
        int w = 0;
        long long t = 0;
        if (sscanf(line.c_str() + sp + 1, "%d %lld", &w, &t) == 2 && (w == 1 || w == 2 || w == 4) && t > 0) {
            *warps = w;
            *tiles = t;
            found = true;   // the last entry wins
        }
    }
    fclose(f);
    return found;
}

void tune_cache_put(const std::string &path, const std::string &key, int warps, int64_t tiles)
{
    if (path.empty()) return;
    FILE *f = fopen(path.c_str(), "a");
    if (!f) return;
    fprintf(f, "%s %d %lld\n", key.c_str(), warps, (long long)tiles);
    fclose(f);
}

// Autotuner of the adjoint split: times one adjoint launch per candidate
// (warps per block x tiles per SM slot) and keeps the fastest.  Reads the
// per-energy weights of all ones and writes only the partial sums.
int plan_tune(Plan *pl)
{
    xrdt_ctx *ctx = pl->ctx;
    if (pl->tuned) return XRDT_OK;
    cudaStream_t st = ctx->stream;
    int optin = 0;
    CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
    const std::string cache = tune_cache_path(), key = tune_key(pl);
    {
        int w = 0;
        int64_t t = 0;
        size_t sm = 0;
        if (tune_cache_get(cache, key, &w, &t)) {
            for (xrdt_op *op : pl->ops) sm = std::max(sm, vox_adj_smem(op->v.P, w));
            if ((int64_t)(sm + vox_adj_static_smem()) <= optin) {
                plan_split(pl, w, t);
                pl->tuned = true;
                return plan_upload(pl);
            }
        }
    }
    int rc = plan_upload(pl);
    if (rc) return rc;
    CK(launch_vox_wtab(plan_batch(pl), plan_total(pl, 4), 1, st, &ctx->launches));
    // streamed: the candidates are timed on the first tile, walked once here
    // (they add into partial rows that every real call clears first)
    if (pl->streamed) CK(tile_walks(pl, pl->tiles.front(), st, &ctx->launches));
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    float best = 1e30f;
    int best_w = pl->adj_warps;
    int64_t best_t = pl->adj_tiles;
    const int warps_c[3] = {1, 2, 4};
    const int per_slot[3] = {2, 4, 8};
    for (int wi = 0; wi < 3; wi++) {
        const int w = warps_c[wi];
        size_t sm = 0;
        for (xrdt_op *op : pl->ops) sm = std::max(sm, vox_adj_smem(op->v.P, w));
        if ((int64_t)(sm + vox_adj_static_smem()) > optin) continue;
        const int64_t slots = (int64_t)pl->sms * vox_adj_blocks_per_sm(w, sm);
        for (int ti = 0; ti < 3; ti++) {
            plan_split(pl, w, slots * per_slot[ti]);
            if ((rc = plan_upload(pl))) break;
            cudaError_t e = cudaEventRecord(a, st);
            if (e == cudaSuccess && pl->streamed) {
                const Plan::Tile &t0 = pl->tiles.front();
                const int64_t items = tile_items(t0, 1);
                if (items > 0)
                    e = launch_vox_adjoint(tile_batch(pl, t0), (int)std::min<int64_t>(pl->adj_grid, items),
                                           pl->adj_smem, st, &ctx->launches);
            } else if (e == cudaSuccess) {
                e = launch_vox_adjoint(plan_batch(pl), pl->adj_grid, pl->adj_smem, st, &ctx->launches);
            }
            if (e == cudaSuccess) e = cudaEventRecord(b, st);
            if (e == cudaSuccess) e = cudaEventSynchronize(b);
            float ms = 0.f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
            if (e != cudaSuccess) {
                cudaGetLastError();
                rc = fail(ctx, XRDT_ERR_CUDA, fmt("adjoint autotuning: %s", cudaGetErrorString(e)));
                break;
            }
            if (ms < best) {
                best = ms;
                best_w = w;
                best_t = slots * per_slot[ti];
            }
        }
        if (rc) break;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (rc) return rc;
    plan_split(pl, best_w, best_t);
    pl->tuned = true;
    tune_cache_put(cache, key, best_w, best_t);
    return plan_upload(pl);
}

int op_plan(xrdt_op *op, Plan **pl)
{
    if (!op->plan) {
        int rc = plan_create(op->ctx, &op, 1, &op->plan);
        if (rc) return rc;
    }
    *pl = op->plan;
    return XRDT_OK;
}

// y[i] = Av_i x[i] for every problem (device arrays, full-grid x; x == NULL:
// the compact xd = x dq of every problem is already in place).
int plan_forward(Plan *pl, const float *const *x, float *const *y)
{
    xrdt_ctx *ctx = pl->ctx;
    cudaStream_t st = ctx->stream;
    const int n = (int)pl->ops.size();
    for (int i = 0; i < n; i++) {
        pl->jobs_h[i].xfull = x ? x[i] : nullptr;
        pl->jobs_h[i].y = y[i];
    }
    int rc = plan_upload(pl);
    if (rc) return rc;
    const VoxBatch B = plan_batch(pl);
    if (x && plan_total(pl, 2) > 0) {
        ProfScope ps(ctx, XRDT_KERNEL_VOX_UPDATE);
        CK(launch_vox_gather(B, plan_total(pl, 2), false, st, &ctx->launches));
    }
    // a problem without voxels gets zeros: its pairs sum nothing
    ProfScope ps(ctx, XRDT_KERNEL_VOX_FORWARD);
    if (pl->streamed) {
        for (int i = 0; i < n; i++)
            if (pl->ops[i]->v.nv == 0) CK(cudaMemsetAsync(y[i], 0, sizeof(float) * (size_t)pl->ops[i]->rays, st));
        CK(stream_forward(pl, false, st, &ctx->launches));
    } else {
        CK(launch_vox_forward(B, false, pl->fwd_grid, pl->fwd_smem, st, &ctx->launches));
    }
    return XRDT_OK;
}

// g[i] = Av_i^T w[i] for every problem (device arrays, full-grid g; compact:
// g[i] in the compact voxel order [nv][NWT]).
int plan_adjoint(Plan *pl, const float *const *w, float *const *g, bool compact = false)
{
    xrdt_ctx *ctx = pl->ctx;
    cudaStream_t st = ctx->stream;
    const int n = (int)pl->ops.size();
    for (int i = 0; i < n; i++) {
        const xrdt_op *op = pl->ops[i];
        pl->jobs_h[i].w = w[i];
        pl->jobs_h[i].g = g[i];
        if (!compact) CK(cudaMemsetAsync(g[i], 0, sizeof(float) * (size_t)op->p.nx * op->p.ny * op->p.nwt, st));
    }
    if (plan_total(pl, 2) == 0) return XRDT_OK;
    int rc = plan_upload(pl);
    if (rc) return rc;
    const VoxBatch B = plan_batch(pl);
    {
        ProfScope ps(ctx, XRDT_KERNEL_VOX_UPDATE);
        CK(launch_vox_wtab(B, plan_total(pl, 4), 0, st, &ctx->launches));
    }
    {
        ProfScope ps(ctx, XRDT_KERNEL_VOX_ADJOINT);
        if (pl->streamed) CK(stream_adjoint(pl, st, &ctx->launches));
        else CK(launch_vox_adjoint(B, pl->adj_grid, pl->adj_smem, st, &ctx->launches));
    }
    ProfScope ps(ctx, XRDT_KERNEL_VOX_UPDATE);
    CK(launch_vox_reduce(B, plan_total(pl, 2), compact ? 3 : 2, st, &ctx->launches));
    return XRDT_OK;
}

// One MLEM pass of every problem without the update: the forward with the
// ratios y / (Av x + c) (xd in place, ymeas and cbg in the descriptors), the
// adjoint of the ratios, and their sums into g in the compact voxel order.
int plan_ratio_backprojection(Plan *pl)
{
    xrdt_ctx *ctx = pl->ctx;
    cudaStream_t st = ctx->stream;
    const VoxBatch B = plan_batch(pl);
    if (pl->streamed) {
        ProfScope ps(ctx, XRDT_KERNEL_VOX_FORWARD);
        CK(stream_forward(pl, true, st, &ctx->launches));
    } else {
        {
            ProfScope ps(ctx, XRDT_KERNEL_VOX_FORWARD);
            CK(launch_vox_forward(B, true, pl->fwd_grid, pl->fwd_smem, st, &ctx->launches));
        }
        ProfScope ps(ctx, XRDT_KERNEL_VOX_ADJOINT);
        CK(launch_vox_adjoint(B, pl->adj_grid, pl->adj_smem, st, &ctx->launches));
    }
    ProfScope ps(ctx, XRDT_KERNEL_VOX_UPDATE);
    CK(launch_vox_reduce(B, plan_total(pl, 2), 3, st, &ctx->launches));
    return XRDT_OK;
}

// iters MLEM updates of every problem; x[i] full grid, in and out (device).
int plan_mlem(Plan *pl, const float *const *y, const float *const *c, float *const *x, int iters)
{
    xrdt_ctx *ctx = pl->ctx;
    cudaStream_t st = ctx->stream;
    const int n = (int)pl->ops.size();
    if (iters == 0) return XRDT_OK;
    int rc;
    if (plan_total(pl, 2) > 0) {
        if ((rc = plan_tune(pl)) || (rc = plan_sens(pl))) return rc;
        for (int i = 0; i < n; i++) {
            pl->jobs_h[i].ymeas = y[i];
            pl->jobs_h[i].cbg = c[i];
            pl->jobs_h[i].xfull = x[i];
            pl->jobs_h[i].xout = x[i];
        }
        if ((rc = plan_upload(pl))) return rc;
        const VoxBatch B = plan_batch(pl);
        {
            ProfScope ps(ctx, XRDT_KERNEL_VOX_UPDATE);
            CK(launch_vox_gather(B, plan_total(pl, 2), true, st, &ctx->launches));
        }
        const int64_t cfg[3] = {pl->adj_warps, pl->adj_tiles, pl->fwd_grid};
        if (!pl->mlem_exec || memcmp(cfg, pl->mlem_cfg, sizeof cfg) != 0) {
            if (pl->mlem_exec) {
                cudaGraphExecDestroy(pl->mlem_exec);
                pl->mlem_exec = nullptr;
            }
            // the graph reads the job descriptors at run time: new arrays
            // only need a new upload, not a new capture
            cudaGraph_t graph;
            CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            int64_t dummy = 0;
            cudaError_t le;
            if (pl->streamed) {
                // per tile: walk, forward with the ratios, adjoint
                le = stream_forward(pl, true, st, &dummy);
            } else {
                le = launch_vox_forward(B, true, pl->fwd_grid, pl->fwd_smem, st, &dummy);
                if (le == cudaSuccess) le = launch_vox_adjoint(B, pl->adj_grid, pl->adj_smem, st, &dummy);
            }
            if (le == cudaSuccess) le = launch_vox_reduce(B, plan_total(pl, 2), 1, st, &dummy);
            pl->mlem_launches = dummy;
            cudaError_t ce = cudaStreamEndCapture(st, &graph);
            if (le != cudaSuccess) {
                if (ce == cudaSuccess) cudaGraphDestroy(graph);
                cudaGetLastError();
                return fail(ctx, XRDT_ERR_CUDA, fmt("MLEM capture: %s", cudaGetErrorString(le)));
            }
            CK(ce);
            cudaError_t ie = cudaGraphInstantiate(&pl->mlem_exec, graph, 0);
            cudaGraphDestroy(graph);
            CK(ie);
            memcpy(pl->mlem_cfg, cfg, sizeof cfg);
        }
        {
            ProfScope ps(ctx, XRDT_KERNEL_VOX_FORWARD);   // the whole iteration (three kernels)
            for (int it = 0; it < iters; it++) CK(cudaGraphLaunch(pl->mlem_exec, st));
        }
        ctx->launches += pl->mlem_launches * (int64_t)iters;
    }
    // empty voxels have no sensitivity: the update sets them to 0
    for (int i = 0; i < n; i++) {
        const xrdt_op *op = pl->ops[i];
        CK(cudaMemsetAsync(x[i], 0, sizeof(float) * (size_t)op->p.nx * op->p.ny * op->p.nwt, st));
    }
    if (plan_total(pl, 2) > 0) {
        ProfScope ps(ctx, XRDT_KERNEL_VOX_UPDATE);
        CK(launch_vox_scatter(plan_batch(pl), plan_total(pl, 2), st, &ctx->launches));
    }
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
    if ((rc = op_alloc_t(op, 4 * (size_t)(p->nx + 1) * (p->ny + 1), &B.cells)) ||
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

    // detector-side integrals of every (pair, voxel), walked once here when
    // the table fits in a quarter of the free device memory
    float2 *d_walk = nullptr;
    const char *wc = getenv("XRDT_WALK_CACHE");
    if (nv > 0 && !(wc && strcmp(wc, "0") == 0)) {
        const size_t bytes = sizeof(float2) * (size_t)npairs * nv;
        size_t fr = 0, tot = 0;
        if ((e = cudaMemGetInfo(&fr, &tot)) != cudaSuccess) {
            cudaGetLastError();
            fr = 0;
        }
        if (bytes <= fr / 4) {
            void *w;
            if ((rc = op_alloc(op, bytes, &w))) return bail(rc);
            d_walk = (float2 *)w;
            if ((e = launch_det_walk(P, d_src, nullptr, 0, npairs, B.vox_xy, nv, B.cells, d_walk, st,
                                     &ctx->launches)) != cudaSuccess) {
                cudaGetLastError();
                fail(ctx, XRDT_ERR_CUDA, fmt("detector-side integrals: %s", cudaGetErrorString(e)));
                return bail(XRDT_ERR_CUDA);
            }
            op->walk_bytes = (int64_t)bytes;
        }
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
    op->v.walk = d_walk;

    // work buffers
    int sms = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    if (e != cudaSuccess) {
        cudaGetLastError();
        fail(ctx, XRDT_ERR_CUDA, fmt("operator tables: %s", cudaGetErrorString(e)));
        return bail(XRDT_ERR_CUDA);
    }
    // partial-sum rows for up to the adjoint pair groups that fill the GPU
    // with the narrowest tiles this problem can get on its own
    {
        const int64_t cb = std::max(1, (nv + 63) / 64);
        op->groups_cap = (int)std::max<int64_t>(1, std::min<int64_t>(npairs, ((int64_t)sms * 64 + cb - 1) / cb));
    }
    const size_t nx_k = (size_t)std::max(nv, 1) * K;
    if ((rc = op_alloc_t(op, nx_k, &op->xc)) || (rc = op_alloc_t(op, nx_k, &op->xd)) ||
        (rc = op_alloc_t(op, (size_t)npairs * E, &op->what)) ||
        (rc = op_alloc_t(op, (size_t)op->groups_cap * nx_k, &op->part)) || (rc = op_alloc_t(op, nx_k, &op->sens)) ||
        (rc = op_alloc_t(op, (size_t)nvox * K, &op->xfull)) || (rc = op_alloc_t(op, (size_t)op->rays, &op->ray_a)) ||
        (rc = op_alloc_t(op, (size_t)op->rays, &op->ray_b)))
        return bail(rc);
    int optin = 0;
    e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
    if (e == cudaSuccess && ((int64_t)(vox_fwd_smem(P) + vox_fwd_static_smem()) > optin ||
                           (int64_t)(vox_adj_smem(P, 1) + vox_adj_static_smem()) > optin)) {
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

int64_t xrdt_op_walk_bytes(const xrdt_op *op) { return op ? op->walk_bytes : -1; }

int32_t xrdt_op_forward(xrdt_op *op, const float *x, float *y, uint32_t flags)
{
    int rc = begin(op);
    if (rc) return rc;
    xrdt_ctx *ctx = op->ctx;
    if (!x || !y) return fail(ctx, XRDT_ERR_NULL, "x and y are required");
    if (flags) return fail(ctx, XRDT_ERR_UNSUPPORTED, "unknown flag bits");
    cudaStream_t st = ctx->stream;
    const size_t nfull = (size_t)op->p.nx * op->p.ny * op->p.nwt;
    const bool hostY = !is_device_ptr(y);
    float *dy = hostY ? op->ray_a : y;
    const float *dx;
    Plan *pl;
    if ((rc = view_in(op, x, nfull, op->xfull, &dx)) || (rc = op_plan(op, &pl))) return rc;
    if ((rc = plan_forward(pl, &dx, &dy))) return rc;
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
    const size_t nfull = (size_t)op->p.nx * op->p.ny * op->p.nwt;
    const bool hostG = !is_device_ptr(g);
    float *dg = hostG ? op->xfull : g;
    const float *dw;
    Plan *pl;
    if ((rc = view_in(op, w, op->rays, op->ray_a, &dw)) || (rc = op_plan(op, &pl))) return rc;
    if ((rc = plan_adjoint(pl, &dw, &dg))) return rc;
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
    if (iters == 0) return XRDT_OK;
    cudaStream_t st = ctx->stream;
    const size_t nfull = (size_t)op->p.nx * op->p.ny * op->p.nwt;
    const bool hostX = !is_device_ptr(x);
    float *dx = hostX ? op->xfull : x;
    if (hostX) CK(cudaMemcpyAsync(dx, x, sizeof(float) * nfull, cudaMemcpyHostToDevice, st));
    const float *dy, *dc;
    Plan *pl;
    if ((rc = view_in(op, y, op->rays, op->ray_a, &dy)) || (rc = view_in(op, c, op->rays, op->ray_b, &dc)) ||
        (rc = op_plan(op, &pl)))
        return rc;
    if ((rc = plan_mlem(pl, &dy, &dc, &dx, iters))) return rc;
    if (hostX) CK(cudaMemcpyAsync(x, dx, sizeof(float) * nfull, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return XRDT_OK;
}

} // extern "C"

// ---- batches of operators ---------------------------------------------------

struct xrdt_batch {
    xrdt_ctx *ctx = nullptr;
    Plan *plan = nullptr;
};

namespace {

int batch_arrays(xrdt_batch *b, const void *const *a, const char *what)
{
    xrdt_ctx *ctx = b->ctx;
    if (!a) return fail(ctx, XRDT_ERR_NULL, fmt("the %s array is NULL", what));
    for (size_t i = 0; i < b->plan->ops.size(); i++) {
        if (!a[i]) return fail(ctx, XRDT_ERR_NULL, fmt("%s[%zu] is NULL", what, i));
        if (!is_device_ptr(a[i]))
            return fail(ctx, XRDT_ERR_UNSUPPORTED, fmt("%s[%zu] must be device memory", what, i));
    }
    return XRDT_OK;
}

int batch_begin(xrdt_batch *b)
{
    if (!b || !b->ctx || !b->plan) return XRDT_ERR_NULL;
    xrdt_ctx *ctx = b->ctx;
    ctx->err.clear();
    CK(cudaSetDevice(ctx->device));
    return XRDT_OK;
}

} // namespace

extern "C" {

int32_t xrdt_batch_create(xrdt_ctx *ctx, xrdt_op *const *ops, int32_t n, xrdt_batch **out)
{
    if (!ctx || !out) return XRDT_ERR_NULL;
    *out = nullptr;
    ctx->err.clear();
    if (!ops || n < 1) return fail(ctx, XRDT_ERR_DIMS, "a batch needs at least one operator");
    for (int i = 0; i < n; i++) {
        if (!ops[i]) return fail(ctx, XRDT_ERR_NULL, fmt("operator %d is NULL", i));
        if (ops[i]->ctx != ctx) return fail(ctx, XRDT_ERR_INPUT, fmt("operator %d belongs to another context", i));
        for (int j = 0; j < i; j++)
            if (ops[j] == ops[i]) return fail(ctx, XRDT_ERR_INPUT, fmt("operator %d appears twice", i));
    }
    CK(cudaSetDevice(ctx->device));
    xrdt_batch *b = new xrdt_batch();
    b->ctx = ctx;
    int rc = plan_create(ctx, ops, n, &b->plan);
    if (rc) {
        delete b;
        return rc;
    }
    *out = b;
    return XRDT_OK;
}

int32_t xrdt_batch_destroy(xrdt_batch *b)
{
    if (!b) return XRDT_ERR_NULL;
    if (b->ctx) {
        cudaSetDevice(b->ctx->device);
        cudaStreamSynchronize(b->ctx->stream);
    }
    plan_free(b->plan);
    delete b;
    return XRDT_OK;
}

int32_t xrdt_batch_forward(xrdt_batch *b, const float *const *x, float *const *y, uint32_t flags)
{
    int rc = batch_begin(b);
    if (rc) return rc;
    xrdt_ctx *ctx = b->ctx;
    if (flags) return fail(ctx, XRDT_ERR_UNSUPPORTED, "unknown flag bits");
    if ((rc = batch_arrays(b, (const void *const *)x, "x")) || (rc = batch_arrays(b, (const void *const *)y, "y")))
        return rc;
    if ((rc = plan_forward(b->plan, x, y))) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    return XRDT_OK;
}

int32_t xrdt_batch_adjoint(xrdt_batch *b, const float *const *w, float *const *g, uint32_t flags)
{
    int rc = batch_begin(b);
    if (rc) return rc;
    xrdt_ctx *ctx = b->ctx;
    if (flags) return fail(ctx, XRDT_ERR_UNSUPPORTED, "unknown flag bits");
    if ((rc = batch_arrays(b, (const void *const *)w, "w")) || (rc = batch_arrays(b, (const void *const *)g, "g")))
        return rc;
    if ((rc = plan_adjoint(b->plan, w, g))) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    return XRDT_OK;
}

int32_t xrdt_batch_mlem(xrdt_batch *b, const float *const *y, const float *const *c, float *const *x, int32_t iters,
                        uint32_t flags)
{
    int rc = batch_begin(b);
    if (rc) return rc;
    xrdt_ctx *ctx = b->ctx;
    if (flags) return fail(ctx, XRDT_ERR_UNSUPPORTED, "unknown flag bits");
    if (iters < 0) return fail(ctx, XRDT_ERR_DIMS, "iters must be >= 0");
    if ((rc = batch_arrays(b, (const void *const *)y, "y")) || (rc = batch_arrays(b, (const void *const *)c, "c")) ||
        (rc = batch_arrays(b, (const void *const *)x, "x")))
        return rc;
    if ((rc = plan_mlem(b->plan, y, c, x, iters))) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    return XRDT_OK;
}

int32_t xrdt_batch_tune(xrdt_batch *b, int32_t *adj_warps, int64_t *adj_tiles, int32_t *fwd_grid, int32_t *adj_grid)
{
    int rc = batch_begin(b);
    if (rc) return rc;
    xrdt_ctx *ctx = b->ctx;
    if ((rc = plan_tune(b->plan))) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    if (adj_warps) *adj_warps = b->plan->adj_warps;
    if (adj_tiles) *adj_tiles = plan_total(b->plan, 1);
    if (fwd_grid) *fwd_grid = b->plan->fwd_grid;
    if (adj_grid) *adj_grid = b->plan->adj_grid;
    return XRDT_OK;
}

} // extern "C"

// ---- the operator with a dense q basis -------------------------------------
// The unknowns of a voxel are J coefficients c[v, j] of a fixed basis
// B[j, k] over the NWT coarse q bins: x[v, k] = sum_j c[v, j] B[j, k].  The
// forward expands the coefficients on the tensor cores (tcgen05, 3xTF32,
// k_basis.cu) straight into x dq, the input of the per-voxel forward; the
// adjoint contracts the per-voxel back-projection with B^T on the tensor
// cores.  MLEM runs on the coefficients (main.m:162-176 with the operator
// A B^T), which keeps them non-negative for a non-negative basis.

struct xrdt_bop {
    xrdt_op *op = nullptr;
    int J = 0;
    std::vector<void *> allocs;
    float *Bdq = nullptr;    // [J][NWT]  B[j][k] dq_k: expands into x dq
    float *Bt = nullptr;     // [NWT][J]  B^T: contracts the back-projection
    float *coef = nullptr;   // [nv][J]
    float *gx = nullptr;     // [nv][NWT] back-projection of the coarse bins
    float *gc = nullptr;     // [nv][J]
    float *sc = nullptr;     // [nv][J] coefficient sensitivity B A^T 1
    float *full = nullptr;   // [NX*NY*J] staging of full-grid coefficient arrays
    unsigned *err = nullptr; // tensor-core wait flag
    bool sc_ready = false;
};

namespace {

void bop_free(xrdt_bop *b)
{
    for (void *p : b->allocs) cudaFree(p);
    b->allocs.clear();
}

int bop_alloc(xrdt_bop *b, size_t bytes, void **out)
{
    xrdt_ctx *ctx = b->op->ctx;
    void *p = nullptr;
    if (test_alloc_fails()) return fail(ctx, XRDT_ERR_ALLOC, fmt("cudaMalloc(%zu bytes): failure injected", bytes));
    cudaError_t e = cudaMalloc(&p, bytes ? bytes : 16);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, XRDT_ERR_ALLOC, fmt("cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e)));
    }
    b->allocs.push_back(p);
    *out = p;
    return XRDT_OK;
}

// coef [nv][J] -> x dq [nv][NWT] of the operator
int bop_expand(xrdt_bop *b)
{
    xrdt_op *op = b->op;
    xrdt_ctx *ctx = op->ctx;
    if (op->v.nv == 0) return XRDT_OK;
    ProfScope ps(ctx, XRDT_KERNEL_BASIS);
    CK(launch_basis_expand(b->coef, op->v.nv, b->J, b->Bdq, op->p.nwt, op->xd, b->err, ctx->stream, &ctx->launches));
    return XRDT_OK;
}

// gx [nv][NWT] -> gc [nv][J]
int bop_contract(xrdt_bop *b, const float *gx, float *gc)
{
    xrdt_op *op = b->op;
    xrdt_ctx *ctx = op->ctx;
    if (op->v.nv == 0) return XRDT_OK;
    ProfScope ps(ctx, XRDT_KERNEL_BASIS);
    CK(launch_basis_expand(gx, op->v.nv, op->p.nwt, b->Bt, b->J, gc, b->err, ctx->stream, &ctx->launches));
    return XRDT_OK;
}

// full-grid [NX*NY*J] device array -> coef
int bop_gather(xrdt_bop *b, const float *full)
{
    xrdt_op *op = b->op;
    xrdt_ctx *ctx = op->ctx;
    CK(launch_rows_gather(full, op->v.vox_xy, op->p.nx, op->v.nv, b->J, b->coef, ctx->stream, &ctx->launches));
    return XRDT_OK;
}

// compact [nv][J] -> full-grid [NX*NY*J] device array, zeros at empty voxels
int bop_scatter(xrdt_bop *b, const float *compact, float *full)
{
    xrdt_op *op = b->op;
    xrdt_ctx *ctx = op->ctx;
    CK(cudaMemsetAsync(full, 0, sizeof(float) * (size_t)op->p.nx * op->p.ny * b->J, ctx->stream));
    CK(launch_rows_scatter(compact, op->v.vox_xy, op->p.nx, op->v.nv, b->J, full, ctx->stream, &ctx->launches));
    return XRDT_OK;
}

// the tensor-core waits of the calls since the flag was cleared
int bop_check(xrdt_bop *b)
{
    xrdt_ctx *ctx = b->op->ctx;
    CK(cudaMemcpyAsync(ctx->h_counters + 2, b->err, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->h_counters[2]) return fail(ctx, XRDT_ERR_TIMEOUT, "the tensor-core accumulator never completed");
    return XRDT_OK;
}

int bop_begin(xrdt_bop *b)
{
    if (!b || !b->op) return XRDT_ERR_NULL;
    int rc = begin(b->op);
    if (rc) return rc;
    xrdt_ctx *ctx = b->op->ctx;
    CK(cudaMemsetAsync(b->err, 0, sizeof(unsigned), ctx->stream));
    return XRDT_OK;
}

} // namespace

extern "C" {

int32_t xrdt_bop_create(xrdt_op *op, const float *B, int32_t J, xrdt_bop **out)
{
    if (!op || !out) return XRDT_ERR_NULL;
    *out = nullptr;
    int rc = begin(op);
    if (rc) return rc;
    xrdt_ctx *ctx = op->ctx;
    if (!B) return fail(ctx, XRDT_ERR_NULL, "the basis is required");
    const int K = op->p.nwt;
    if (J < 16 || J > 64 || (J & 15) || K < 16 || K > 64 || (K & 15))
        return fail(ctx, XRDT_ERR_DIMS, "need J and NWT multiples of 16 in [16, 64]");
    std::vector<float> hB((size_t)J * K);
    CK(cudaMemcpy(hB.data(), B, sizeof(float) * hB.size(), cudaMemcpyDefault));
    for (float v : hB)
        if (!(v >= 0.f) || !std::isfinite(v)) return fail(ctx, XRDT_ERR_INPUT, "basis entries must be finite and >= 0");
    std::vector<float4> cq(K);
    CK(cudaMemcpy(cq.data(), op->v.coarse_q, sizeof(float4) * K, cudaMemcpyDeviceToHost));
    std::vector<float> hBdq((size_t)J * K), hBt((size_t)K * J);
    for (int j = 0; j < J; j++)
        for (int k = 0; k < K; k++) {
            hBdq[(size_t)j * K + k] = hB[(size_t)j * K + k] * cq[k].z;   // as the forward forms x dq
            hBt[(size_t)k * J + j] = hB[(size_t)j * K + k];
        }
    xrdt_bop *b = new xrdt_bop();
    b->op = op;
    b->J = J;
    const size_t nv = (size_t)std::max(op->v.nv, 1);
    void *p;
    auto alloc = [&](size_t bytes, void **dst) { return bop_alloc(b, bytes, dst); };
    if ((rc = alloc(sizeof(float) * hBdq.size(), &p)) == 0) b->Bdq = (float *)p;
    if (!rc && (rc = alloc(sizeof(float) * hBt.size(), &p)) == 0) b->Bt = (float *)p;
    if (!rc && (rc = alloc(sizeof(float) * nv * J, &p)) == 0) b->coef = (float *)p;
    if (!rc && (rc = alloc(sizeof(float) * nv * K, &p)) == 0) b->gx = (float *)p;
    if (!rc && (rc = alloc(sizeof(float) * nv * J, &p)) == 0) b->gc = (float *)p;
    if (!rc && (rc = alloc(sizeof(float) * nv * J, &p)) == 0) b->sc = (float *)p;
    if (!rc && (rc = alloc(sizeof(float) * (size_t)op->p.nx * op->p.ny * J, &p)) == 0) b->full = (float *)p;
    if (!rc && (rc = alloc(sizeof(unsigned), &p)) == 0) b->err = (unsigned *)p;
    cudaError_t e = cudaSuccess;
    if (!rc) e = cudaMemcpy(b->Bdq, hBdq.data(), sizeof(float) * hBdq.size(), cudaMemcpyHostToDevice);
    if (!rc && e == cudaSuccess) e = cudaMemcpy(b->Bt, hBt.data(), sizeof(float) * hBt.size(), cudaMemcpyHostToDevice);
    if (!rc && e != cudaSuccess) {
        cudaGetLastError();
        rc = fail(ctx, XRDT_ERR_CUDA, fmt("basis upload: %s", cudaGetErrorString(e)));
    }
    if (rc) {
        bop_free(b);
        delete b;
        return rc;
    }
    *out = b;
    return XRDT_OK;
}

int32_t xrdt_bop_destroy(xrdt_bop *b)
{
    if (!b) return XRDT_ERR_NULL;
    if (b->op && b->op->ctx) {
        cudaSetDevice(b->op->ctx->device);
        cudaStreamSynchronize(b->op->ctx->stream);
    }
    bop_free(b);
    delete b;
    return XRDT_OK;
}

int32_t xrdt_bop_forward(xrdt_bop *b, const float *c, float *y, uint32_t flags)
{
    int rc = bop_begin(b);
    if (rc) return rc;
    xrdt_op *op = b->op;
    xrdt_ctx *ctx = op->ctx;
    if (!c || !y) return fail(ctx, XRDT_ERR_NULL, "c and y are required");
    if (flags) return fail(ctx, XRDT_ERR_UNSUPPORTED, "unknown flag bits");
    cudaStream_t st = ctx->stream;
    const size_t nfull = (size_t)op->p.nx * op->p.ny * b->J;
    const float *dc;
    if ((rc = view_in(op, c, nfull, b->full, &dc))) return rc;
    const bool hostY = !is_device_ptr(y);
    float *dy = hostY ? op->ray_a : y;
    Plan *pl;
    if ((rc = op_plan(op, &pl)) || (rc = bop_gather(b, dc)) || (rc = bop_expand(b))) return rc;
    if ((rc = plan_forward(pl, nullptr, &dy))) return rc;
    if (hostY) CK(cudaMemcpyAsync(y, dy, sizeof(float) * op->rays, cudaMemcpyDeviceToHost, st));
    return bop_check(b);
}

int32_t xrdt_bop_adjoint(xrdt_bop *b, const float *w, float *g, uint32_t flags)
{
    int rc = bop_begin(b);
    if (rc) return rc;
    xrdt_op *op = b->op;
    xrdt_ctx *ctx = op->ctx;
    if (!w || !g) return fail(ctx, XRDT_ERR_NULL, "w and g are required");
    if (flags) return fail(ctx, XRDT_ERR_UNSUPPORTED, "unknown flag bits");
    cudaStream_t st = ctx->stream;
    const size_t nfull = (size_t)op->p.nx * op->p.ny * b->J;
    const float *dw;
    Plan *pl;
    if ((rc = view_in(op, w, op->rays, op->ray_a, &dw)) || (rc = op_plan(op, &pl))) return rc;
    float *gx = b->gx;
    if ((rc = plan_adjoint(pl, &dw, &gx, true)) || (rc = bop_contract(b, b->gx, b->gc))) return rc;
    const bool hostG = !is_device_ptr(g);
    float *dg = hostG ? b->full : g;
    if ((rc = bop_scatter(b, b->gc, dg))) return rc;
    if (hostG) CK(cudaMemcpyAsync(g, dg, sizeof(float) * nfull, cudaMemcpyDeviceToHost, st));
    return bop_check(b);
}

int32_t xrdt_bop_mlem(xrdt_bop *b, const float *y, const float *c, float *x, int32_t iters, uint32_t flags)
{
    int rc = bop_begin(b);
    if (rc) return rc;
    xrdt_op *op = b->op;
    xrdt_ctx *ctx = op->ctx;
    if (!y || !c || !x) return fail(ctx, XRDT_ERR_NULL, "y, c and x are required");
    if (iters < 0) return fail(ctx, XRDT_ERR_DIMS, "iters must be >= 0");
    if (flags) return fail(ctx, XRDT_ERR_UNSUPPORTED, "unknown flag bits");
    cudaStream_t st = ctx->stream;
    const size_t nfull = (size_t)op->p.nx * op->p.ny * b->J;
    const int64_t ncoef = (int64_t)op->v.nv * b->J;
    const float *dy, *dc, *dx0;
    Plan *pl;
    if ((rc = view_in(op, y, op->rays, op->ray_a, &dy)) || (rc = view_in(op, c, op->rays, op->ray_b, &dc)) ||
        (rc = view_in(op, x, nfull, b->full, &dx0)) || (rc = op_plan(op, &pl)))
        return rc;
    if ((rc = bop_gather(b, dx0))) return rc;
    if (op->v.nv > 0 && iters > 0) {
        if ((rc = plan_tune(pl)) || (rc = plan_sens(pl))) return rc;
        if (!b->sc_ready) {
            // the coefficient sensitivity B (A^T 1), from the operator's FP64 one
            CK(launch_to_float(op->sens, (int64_t)op->v.nv * op->p.nwt, b->gx, st, &ctx->launches));
            if ((rc = bop_contract(b, b->gx, b->sc))) return rc;
            b->sc_ready = true;
        }
        pl->jobs_h[0].ymeas = dy;
        pl->jobs_h[0].cbg = dc;
        pl->jobs_h[0].g = b->gx;
        if ((rc = plan_upload(pl))) return rc;
        for (int it = 0; it < iters; it++) {
            if ((rc = bop_expand(b)) || (rc = plan_ratio_backprojection(pl)) || (rc = bop_contract(b, b->gx, b->gc)))
                return rc;
            ProfScope ps(ctx, XRDT_KERNEL_VOX_UPDATE);
            CK(launch_bop_update(b->coef, b->gc, b->sc, ncoef, st, &ctx->launches));
        }
    }
    const bool hostX = !is_device_ptr(x);
    float *dxo = hostX ? b->full : x;
    if (iters > 0) {
        if ((rc = bop_scatter(b, b->coef, dxo))) return rc;
    } else if (hostX) {
        CK(cudaMemcpyAsync(dxo, dx0, sizeof(float) * nfull, cudaMemcpyDeviceToDevice, st));
    }
    if (hostX) CK(cudaMemcpyAsync(x, dxo, sizeof(float) * nfull, cudaMemcpyDeviceToHost, st));
    return bop_check(b);
}

} // extern "C"
