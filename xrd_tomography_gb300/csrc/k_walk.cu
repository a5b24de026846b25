// k_walk.cu -- detector-side line integrals of a tile of (source, pixel)
// pairs: tab[item * nv + v] = attenuator(Rdet, Rvox) of
// integrate_diffraction.cu:259 (attenuator.cu:9-109), for every non-empty
// voxel v.
//
// The forward projector needs one such walk per (pair, voxel).  Walked inside
// the projector they share its registers and occupancy with the energy loop;
// here a separate kernel walks them and the projector reads the results as
// one coalesced float2 per voxel.
//
// Sampled one point per lane, the walk is bound by L1 wavefronts: a
// warp-wide 16-byte load costs at least four, and every sample needs a
// 32-byte cell.  Here each lane walks a whole ray cell by cell (walk_cells,
// walk.cuh), one cell load per run of 3-4 samples.  A warp takes 32 rays
// that end on 32 neighbouring pixels of one view and leave from the same
// voxel, so its lanes take about the same number of steps and stay within a
// few voxels of each other, side by side across the rays.  The warp reads
// the copy of the cell map (row- or column-major) whose rows run across its
// rays, so that neighbouring lanes mostly share cache lines.  Per voxel each
// lane sets up its own ray (FP32 with the exact FP64 fallback) and stores its
// float2; the stores of consecutive voxels of a row merge in L2.
#include "scatter.cuh"

namespace xrdt {

namespace {

constexpr int kWalkThreads = 128;
constexpr int kWalkWarps = kWalkThreads / 32;
constexpr int kRays = 32;          // rays per group: neighbouring pixels of one view
constexpr int kVoxPerStrip = 64;   // voxels per warp item

// Ray r of group g.  Linear pairs (pairs == NULL): the tile holds the pixels
// d0 .. d0+nd-1 of every view, row (det - d0) * SRC + src; group g is view
// g % SRC and pixels d0 + 32 (g / SRC) + r.  A list: entries 32g + r.
__device__ __forceinline__ bool group_ray(const DevProblem &P, const int2 *pairs, long long n_items, int nd,
                                          long long g, int r, int *src, int *det, long long *row)
{
    if (pairs) {
        const long long e = g * kRays + r;
        if (e >= n_items) return false;
        const int2 pr = pairs[e];
        *src = pr.x;
        *det = pr.y;
        *row = e;
        return true;
    }
    const int s = (int)(g % P.n_src);
    const int dl = (int)(g / P.n_src) * kRays + r;
    if (dl >= nd) return false;
    *src = s;
    *det = dl;   // relative to d0
    *row = (long long)dl * P.n_src + s;
    return true;
}

// 8 blocks (32 warps) per SM: the walk waits on L1 latency, and at 64
// registers (8 bytes spilled around the FP64 fallback call) it ran 1016 ms on
// the 256x256 workload against 1089 ms at 6 blocks and 80 registers.
__global__ void __launch_bounds__(kWalkThreads, 8)
k_det_walk(DevProblem P, F32Consts c, const SrcGeom *__restrict__ sg, const int2 *__restrict__ pairs,
           long long n_items, int d0, int nd, long long n_groups, const int *__restrict__ vox_xy, int nv,
           const float4 *__restrict__ cells, float2 *__restrict__ tab)
{
    const int lane = threadIdx.x & 31;
    const int64_t ncell = (int64_t)(P.nx + 1) * (P.ny + 1);
    const unsigned ncell_m1 = (unsigned)(ncell - 1);
    const float4 *cells_t = cells + 2 * ncell;   // column-major copy
    const int nstrips = (nv + kVoxPerStrip - 1) / kVoxPerStrip;
    const long long nwork = n_groups * nstrips;
    const long long wstride = (long long)gridDim.x * kWalkWarps;
    for (long long wk = (long long)blockIdx.x * kWalkWarps + (threadIdx.x >> 5); wk < nwork; wk += wstride) {
        const long long g = wk / nstrips;
        const int strip = (int)(wk - g * nstrips);
        int src = 0, det = 0;
        long long row = -1;
        const bool valid = group_ray(P, pairs, n_items, nd, g, lane, &src, &det, &row);
        double ex = 0.0, ey = 0.0;
        if (valid) {
            if (!pairs) det += d0;
            const SrcGeom gs = sg[src];
            double ez;
            det_position(P, gs.sphi, gs.cphi, det, &ex, &ey, &ez);
        }
        const float exf = (float)ex, eyf = (float)ey;
        // the endpoint as float pairs, once per ray group (conversions from
        // double issue on the FP64 pipe)
        const ff exff = ff_from_double(ex), eyff = ff_from_double(ey);
        float2 *out = tab + (valid ? row : 0) * nv;
        const int v1 = min(nv, (strip + 1) * kVoxPerStrip);
        for (int v = strip * kVoxPerStrip; v < v1; v++) {
            const int xy = vox_xy[v];
            const float vx = ((float)(xy & 0xffff) + 0.5f) * c.vox;
            const float vy = ((float)(xy >> 16) + 0.5f) * c.vox;
            WalkSetup ws;
            ws.Lx = ws.Ly = 0.f;
            ws.n = 0;
            ws.dlt = ws.ux = ws.uy = ff{0.f, 0.f};
            if (valid) {
                // decided in FP32 (guard bands) or FP64; the anchor of an FP32
                // decision comes from the endpoint as a float pair
                if (walk_setup_f32(P, c, exf, eyf, vx, vy, &ws))
                    walk_anchor_ff(c, exff, eyff, vx, vy, &ws);
                else
                    walk_setup_f64(P, ex, ey, (double)vx, (double)vy, &ws);
            }
            // rays mostly along x lie side by side along y: column-major copy
            const unsigned along_x = __ballot_sync(0xffffffffu, valid && fabsf(ws.Lx) > fabsf(ws.Ly));
            const unsigned any = __ballot_sync(0xffffffffu, valid);
            const bool colmajor = 2 * __popc(along_x) > __popc(any);
            const float2 A = colmajor ? walk_cells(cells_t, P.ny + 1, 1, ncell_m1, ws, vx, vy, c.DQ)
                                      : walk_cells(cells, 1, P.nx + 1, ncell_m1, ws, vx, vy, c.DQ);
            if (valid) out[v] = A;
        }
    }
}

} // namespace

cudaError_t launch_det_walk(const DevProblem &P, const SrcGeom *sg, const int2 *pairs, long long p0,
                            long long n_items, const int *vox_xy, int nv, const float4 *cells, float2 *tab,
                            cudaStream_t s, int64_t *launches)
{
    if (n_items <= 0 || nv <= 0) return cudaSuccess;
    int d0 = 0, nd = 0;
    long long n_groups;
    if (pairs) {
        n_groups = (n_items + kRays - 1) / kRays;
    } else {
        // whole pixels of every view
        if (p0 % P.n_src != 0 || n_items % P.n_src != 0) return cudaErrorInvalidValue;
        d0 = (int)(p0 / P.n_src);
        nd = (int)(n_items / P.n_src);
        n_groups = (long long)P.n_src * ((nd + kRays - 1) / kRays);
    }
    const long long nwork = n_groups * ((nv + kVoxPerStrip - 1) / kVoxPerStrip);
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    long long blocks = (nwork + kWalkWarps - 1) / kWalkWarps;
    if (blocks > (long long)sms * 64) blocks = (long long)sms * 64;
    k_det_walk<<<(unsigned)blocks, kWalkThreads, 0, s>>>(P, make_f32_consts(P), sg, pairs, n_items, d0, nd, n_groups,
                                                          vox_xy, nv, cells, tab);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

} // namespace xrdt
