// k_prep.cu -- per-call staging for the factored forward projector.
//
//  * k_build_cells: the (a1,a2) map as bilinear cells.  Replaces Copy2Vector
//    (Copy2Vector.cu:9-23) and the cudaArray/texture set-up of
//    Forward_XRD.cu:209-237: cell (ci,cj) holds the bilinear coefficients of
//    the four texels (ci-1..ci, cj-1..cj) of a zero-bordered map, about the
//    cell centre, as two float4, so one sample is two 16-byte loads and three
//    packed FMAs with no border tests.  The map is stored twice: row-major
//    (ci + cj (NX+1)) and behind it column-major (cj + ci (NY+1)), so that a
//    warp whose rays lie side by side along y reads neighbouring cells from
//    one cache line as well as one whose rays lie side by side along x.  Also
//    quantises the Compton table to u8 (integrate_diffraction.cu:66-74).
//  * k_compact_voxels: non-empty voxels in the reference's loop order
//    (nx outer, ny inner; integrate_diffraction.cu:173-178) and the material
//    id check (ids above n_mat would index past Ifine in the reference).
//  * k_voxel_compton: the (a1,a2) sample of the Compton table lookup per voxel
//    (integrate_diffraction.cu:181-189), honouring the stale-coordinate quirk.
//  * k_src_atten: the source-side line integral per (source, voxel), which
//    the reference recomputes in every block (integrate_diffraction.cu:260).
#include "xrdt_device.cuh"
#include "walk.cuh"

namespace xrdt {

namespace {

__global__ void k_build_cells(int nx, int ny, const float *__restrict__ a1, const float *__restrict__ a2,
                              float4 *__restrict__ cells, const float *__restrict__ S2,
                              unsigned char *__restrict__ s2u8, int ns2, const float *__restrict__ S1,
                              unsigned char *__restrict__ s1u8)
{
    const int64_t ncell = (int64_t)(nx + 1) * (ny + 1);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncell; c += stride) {
        const int ci = (int)(c % (nx + 1)), cj = (int)(c / (nx + 1));
        float v[2][2][2];
#pragma unroll
        for (int dj = 0; dj < 2; dj++)
#pragma unroll
            for (int di = 0; di < 2; di++) {
                const int i = ci - 1 + di, j = cj - 1 + dj;
                const bool in = (i >= 0 && i < nx && j >= 0 && j < ny);
                const int64_t idx = in ? (int64_t)i + (int64_t)j * nx : 0;
                v[dj][di][0] = in ? a1[idx] : 0.f;
                v[dj][di][1] = in ? a2[idx] : 0.f;
            }
        // bilinear coefficients per component q about the cell centre:
        // f(u,v) = c00 + c10 u + c01 v + c11 u v for u, v in [-1/2, 1/2]
        float c00[2], c10[2], c01[2], c11[2];
        for (int q = 0; q < 2; q++) {
            const double f00 = v[0][0][q], f10 = v[0][1][q], f01 = v[1][0][q], f11 = v[1][1][q];
            c00[q] = (float)(0.25 * ((f00 + f10) + (f01 + f11)));
            c10[q] = (float)(0.5 * ((f10 - f00) + (f11 - f01)));
            c01[q] = (float)(0.5 * ((f01 - f00) + (f11 - f10)));
            c11[q] = (float)((f11 - f01) - (f10 - f00));
        }
        const float4 lo = make_float4(c00[0], c00[1], c10[0], c10[1]);
        const float4 hi = make_float4(c01[0], c01[1], c11[0], c11[1]);
        const int64_t ct = ncell + (int64_t)cj + (int64_t)ci * (ny + 1);
        cells[2 * c] = lo;
        cells[2 * c + 1] = hi;
        cells[2 * ct] = lo;
        cells[2 * ct + 1] = hi;
    }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ns2; i += stride) {
        const int q = floor_to_int((double)S2[i]);
        s2u8[i] = (unsigned char)(q < 0 ? 0 : (q > 255 ? 255 : q));
        if (S1) {
            const int q1 = floor_to_int((double)S1[i]);
            s1u8[i] = (unsigned char)(q1 < 0 ? 0 : (q1 > 255 ? 255 : q1));
        }
    }
}

// One block of 1024 threads: stream compaction in loop order.
__global__ void __launch_bounds__(1024)
k_compact_voxels(int nx, int ny, int n_mat, const int32_t *__restrict__ seg, int *__restrict__ vox_xy,
                 int *__restrict__ vox_mat, int *__restrict__ counters)
{
    __shared__ int warp_cnt[32];
    __shared__ int base_s;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) base_s = 0;
    __syncthreads();
    int bad = 0;
    const int64_t total = (int64_t)nx * ny;
    for (int64_t L0 = 0; L0 < total; L0 += blockDim.x) {
        const int64_t L = L0 + threadIdx.x;
        int x = 0, y = 0, s = 0;
        if (L < total) {
            x = (int)(L / ny);
            y = (int)(L % ny);
            s = seg[(int64_t)x + (int64_t)y * nx];
            bad |= (s > n_mat);
        }
        const bool keep = (L < total) && (s > 0) && (s <= n_mat);
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (lane == 0) warp_cnt[wid] = __popc(m);
        __syncthreads();
        int off = 0, tot = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
            if (w < wid) off += warp_cnt[w];
            tot += warp_cnt[w];
        }
        const int base = base_s;
        if (keep) {
            const int pos = base + off + __popc(m & ((1u << lane) - 1u));
            vox_xy[pos] = x | (y << 16);
            vox_mat[pos] = s - 1;
        }
        __syncthreads();
        if (threadIdx.x == 0) base_s = base + tot;
        __syncthreads();
    }
    bad = __syncthreads_or(bad);
    if (threadIdx.x == 0) {
        counters[0] = base_s;
        counters[1] = bad;
    }
}

__global__ void k_voxel_compton(DevProblem P, const float *__restrict__ a1, const float *__restrict__ a2,
                                const int *__restrict__ vox_xy, const int *__restrict__ counters,
                                int *__restrict__ vox_na, float *__restrict__ vox_a2, float *__restrict__ vox_ta)
{
    const int nv = counters[0];
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
        double sx = 0.0, sy = 0.0;  // stale coordinates start at (0,0)
        int use = P.quirk_stale ? v - 1 : v;
        if (use >= 0) {
            const int xy = vox_xy[use];
            sx = ((double)(xy & 0xffff) + 0.5) * P.vox;
            sy = ((double)(xy >> 16) + 0.5) * P.vox;
        }
        double a1now, a2now;
        bilinear_f64(a1, a2, P.nx, P.ny, sx, sy, &a1now, &a2now);
        const double l2a = log2(fabs(a1now / a2now));
        int na = floor_to_int((l2a - P.a_min) / P.da_tab);
        vox_na[v] = na < 0 ? 0 : (na >= P.na ? P.na - 1 : na);
        vox_a2[v] = (float)a2now;
        if (vox_ta) vox_ta[v] = (float)((l2a - P.a_min) / P.da_grid);   // clamped where it is used
    }
}

// One lane per (source, voxel): attenuator(Rsrc, Rvox) of
// integrate_diffraction.cu:260, set up in FP64 and walked cell by cell from
// the voxel (walk_cells).  A warp takes 32 neighbouring voxels of one source.
__global__ void k_src_atten(DevProblem P, const SrcGeom *__restrict__ sg, const int *__restrict__ vox_xy,
                            int nv, const float4 *__restrict__ cells, float2 *__restrict__ out)
{
    const int64_t nwork = (int64_t)P.n_src * nv;
    const unsigned ncell_m1 = (unsigned)((P.nx + 1) * (P.ny + 1) - 1);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < nwork; w += stride) {
        const int src = (int)(w / nv), v = (int)(w % nv);
        const int xy = vox_xy[v];
        const double vx = ((double)(xy & 0xffff) + 0.5) * P.vox;
        const double vy = ((double)(xy >> 16) + 0.5) * P.vox;
        WalkSetup ws;
        walk_setup(P, sg[src].Rsrc_x, sg[src].Rsrc_y, vx, vy, &ws);
        out[(int64_t)src * nv + v] = walk_cells(cells, 1, P.nx + 1, ncell_m1, ws, (float)vx, (float)vy, (float)P.DQ);
    }
}

} // namespace

cudaError_t launch_prep_map(const DevProblem &P, const float *a1, const float *a2, const float *S2,
                            PrepBuffers &B, cudaStream_t s, int64_t *launches, const float *S1)
{
    const int64_t ncell = (int64_t)(P.nx + 1) * (P.ny + 1);
    int blocks = (int)((ncell + 255) / 256);
    if (blocks > 4096) blocks = 4096;
    k_build_cells<<<blocks, 256, 0, s>>>(P.nx, P.ny, a1, a2, B.cells, S2, B.s2u8, S2 ? P.nq * P.na : 0,
                                         B.s1u8 ? S1 : nullptr, B.s1u8);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

cudaError_t launch_prep_voxels(const DevProblem &P, const int32_t *seg, const float *a1,
                               const float *a2, PrepBuffers &B, cudaStream_t s, int64_t *launches)
{
    k_compact_voxels<<<1, 1024, 0, s>>>(P.nx, P.ny, P.n_mat, seg, B.vox_xy, B.vox_mat, B.counters);
    const int64_t nvox = (int64_t)P.nx * P.ny;
    int blocks = (int)((nvox + 255) / 256);
    if (blocks > 2048) blocks = 2048;
    k_voxel_compton<<<blocks, 256, 0, s>>>(P, a1, a2, B.vox_xy, B.counters, B.vox_na, B.vox_a2, B.vox_ta);
    if (launches) (*launches) += 2;
    return cudaGetLastError();
}

cudaError_t launch_compact_voxels(const DevProblem &P, const int32_t *seg, PrepBuffers &B, cudaStream_t s,
                                  int64_t *launches)
{
    k_compact_voxels<<<1, 1024, 0, s>>>(P.nx, P.ny, P.n_mat, seg, B.vox_xy, B.vox_mat, B.counters);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

int current_sm_count()
{
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();   // a failed query leaves no error behind for the next launch check
        return 152;
    }
    if (cached[dev] > 0) return cached[dev];
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) {
        cudaGetLastError();
        return 152;
    }
    cached[dev] = sms;
    return sms;
}

cudaError_t launch_src_atten(const DevProblem &P, const SrcGeom *d_src, int nv, PrepBuffers &B,
                             cudaStream_t s, int64_t *launches)
{
    if (nv == 0) return cudaSuccess;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int64_t items = (int64_t)P.n_src * nv;
    int64_t blocks = (items + 127) / 128;
    if (blocks > (int64_t)sms * 16) blocks = (int64_t)sms * 16;
    k_src_atten<<<(int)blocks, 128, 0, s>>>(P, d_src, B.vox_xy, nv, B.cells, B.atten_src);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

} // namespace xrdt
