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
// The walk is bound by L1 wavefronts (one per distinct 128-byte line that a
// warp-wide load touches), so the lanes of a load are kept close together in
// the plane.  A warp takes a group of 8 rays that end on 8 neighbouring
// pixels of one view and a strip of voxels.  For each voxel the 8 rays leave
// from the same point and stay within a few voxels of each other, so lane
// (r, j) = (lane / 4, lane % 4) takes samples j, j+4, j+8, ... of ray r and
// each warp-wide load covers about one voxel of path of 8 adjacent rays --
// a few cells -- instead of 8 voxels of one ray.
//
// Per chunk of 32 voxels: lane = voxel sets up the walks of the 8 rays (FP32
// with the exact FP64 fallback, walk.cuh) into shared memory; then the warp
// walks voxel by voxel, sums the 4 lanes of each ray, and finally stores the
// 8 rays' results of the chunk as 8 coalesced rows.
#include "scatter.cuh"

namespace xrdt {

namespace {

constexpr int kWalkThreads = 128;
constexpr int kWalkWarps = kWalkThreads / 32;
constexpr int kRays = 8;            // rays per group: neighbouring pixels of one view
constexpr int kChunksPerStrip = 4;  // chunks of 32 voxels per warp item
constexpr int kPad = 33;            // row pitch of the per-ray tables (no bank conflicts)

struct WarpTables {
    float rx[kRays][kPad], ry[kRays][kPad], Lx[kRays][kPad], Ly[kRays][kPad];
    int n[kRays][kPad];
    float2 res[kRays][kPad];
    double ex[kRays], ey[kRays];
    long long row[kRays];   // output row of each ray, -1 for none
};

// Ray r of group g.  Linear pairs (pairs == NULL): the tile holds the pixels
// d0 .. d0+nd-1 of every view, row (det - d0) * SRC + src; group g is view
// g % SRC and pixels d0 + 8 (g / SRC) + r.  A list: entries 8g + r.
__device__ __forceinline__ bool group_ray(const DevProblem &P, const int2 *pairs, long long n_items, int d0, int nd,
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
    *det = d0 + dl;
    *row = (long long)dl * P.n_src + s;
    return true;
}

__global__ void __launch_bounds__(kWalkThreads)
k_det_walk(DevProblem P, F32Consts c, const SrcGeom *__restrict__ sg, const int2 *__restrict__ pairs,
           long long n_items, int d0, int nd, long long n_groups, const int *__restrict__ vox_xy, int nv,
           const float4 *__restrict__ cells, float2 *__restrict__ tab)
{
    __shared__ WarpTables wt_all[kWalkWarps];
    WarpTables &W = wt_all[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int r = lane >> 2, j = lane & 3;
    const unsigned ncell_m1 = (unsigned)((P.nx + 1) * (P.ny + 1) - 1);
    const int nchunks = (nv + 31) >> 5;
    const int nstrips = (nchunks + kChunksPerStrip - 1) / kChunksPerStrip;
    const long long nwork = n_groups * nstrips;
    const long long wstride = (long long)gridDim.x * kWalkWarps;
    for (long long wk = (long long)blockIdx.x * kWalkWarps + (threadIdx.x >> 5); wk < nwork; wk += wstride) {
        const long long g = wk / nstrips;
        const int strip = (int)(wk - g * nstrips);
        __syncwarp();
        if (lane < kRays) {
            int src, det;
            long long row;
            if (group_ray(P, pairs, n_items, d0, nd, g, lane, &src, &det, &row)) {
                const SrcGeom gs = sg[src];
                double Rdx, Rdy, Rdz;
                det_position(P, gs.sphi, gs.cphi, det, &Rdx, &Rdy, &Rdz);
                W.ex[lane] = Rdx;
                W.ey[lane] = Rdy;
                W.row[lane] = row;
            } else {
                W.row[lane] = -1;
            }
        }
        __syncwarp();
        const int c1 = min(nchunks, (strip + 1) * kChunksPerStrip);
        for (int chunk = strip * kChunksPerStrip; chunk < c1; chunk++) {
            const int nin = min(32, nv - chunk * 32);
            // set-up: lane = voxel, all rays of the group
            {
                const int v = min(chunk * 32 + lane, nv - 1);
                const int xy = vox_xy[v];
                const float vx = ((float)(xy & 0xffff) + 0.5f) * c.vox;
                const float vy = ((float)(xy >> 16) + 0.5f) * c.vox;
                for (int q = 0; q < kRays; q++) {
                    WalkSetup ws;
                    if (W.row[q] < 0) {
                        ws.rx = ws.ry = ws.Lx = ws.Ly = 0.f;
                        ws.n = 0;
                    } else {
                        const double ex = W.ex[q], ey = W.ey[q];
                        if (!walk_setup_f32(P, c, (float)ex, (float)ey, vx, vy, &ws))
                            walk_setup_f64(P, ex, ey, (double)vx, (double)vy, &ws);
                    }
                    W.rx[q][lane] = ws.rx;
                    W.ry[q][lane] = ws.ry;
                    W.Lx[q][lane] = ws.Lx;
                    W.Ly[q][lane] = ws.Ly;
                    W.n[q][lane] = ws.n;
                }
            }
            __syncwarp();
            // walks: lane (r, j) takes samples j, j+4, ... of ray r
            for (int i = 0; i < nin; i++) {
                const float2 L2 = make_float2(W.Lx[r][i], W.Ly[r][i]);
                const float2 R2 = make_float2(W.rx[r][i], W.ry[r][i]);
                const int n = W.n[r][i];
                float2 sa = make_float2(0.f, 0.f), sb = make_float2(0.f, 0.f);
                float kf = (float)j;
                int k = j;
                for (; k + 4 < n; k += 8, kf += 8.f) {
                    const float kg = kf + 4.f;
                    const float2 a = cell_sample(cells, P.nx, ncell_m1, __ffma2_rn(L2, make_float2(kf, kf), R2));
                    const float2 b = cell_sample(cells, P.nx, ncell_m1, __ffma2_rn(L2, make_float2(kg, kg), R2));
                    sa = __fadd2_rn(sa, a);
                    sb = __fadd2_rn(sb, b);
                }
                if (k < n)
                    sa = __fadd2_rn(sa, cell_sample(cells, P.nx, ncell_m1, __ffma2_rn(L2, make_float2(kf, kf), R2)));
                float2 s = __fadd2_rn(sa, sb);
                s.x += __shfl_xor_sync(0xffffffffu, s.x, 1);
                s.y += __shfl_xor_sync(0xffffffffu, s.y, 1);
                s.x += __shfl_xor_sync(0xffffffffu, s.x, 2);
                s.y += __shfl_xor_sync(0xffffffffu, s.y, 2);
                if (j == 0) W.res[r][i] = make_float2(s.x * c.DQ, s.y * c.DQ);
            }
            __syncwarp();
            for (int q = 0; q < kRays; q++) {
                const long long row = W.row[q];
                if (row >= 0 && lane < nin) tab[row * nv + chunk * 32 + lane] = W.res[q][lane];
            }
            __syncwarp();
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
    const int nchunks = (nv + 31) / 32;
    const long long nwork = n_groups * ((nchunks + kChunksPerStrip - 1) / kChunksPerStrip);
    long long blocks = (nwork + kWalkWarps - 1) / kWalkWarps;
    if (blocks > 152LL * 64) blocks = 152LL * 64;
    k_det_walk<<<(unsigned)blocks, kWalkThreads, 0, s>>>(P, make_f32_consts(P), sg, pairs, n_items, d0, nd, n_groups,
                                                          vox_xy, nv, cells, tab);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

} // namespace xrdt
