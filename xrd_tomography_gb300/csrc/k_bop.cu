// k_bop.cu -- element-wise kernels of the per-voxel operator with a dense q
// basis (xrdt_bop, op.cu): moving rows of R values per non-empty voxel
// between the full-grid layout [NX*NY][R] and the compact voxel order
// [nv][R], and the MLEM update in coefficient space (main.m:162-176).
#include "xrdt_device.cuh"

namespace xrdt {

namespace {

__global__ void k_rows_gather(const float *__restrict__ full, const int *__restrict__ vox_xy, int nx, int64_t nv,
                              int R, float *__restrict__ compact)
{
    const int64_t n = nv * R;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = t / R;
        const int r = (int)(t - v * R);
        const int xy = vox_xy[v];
        compact[t] = full[((int64_t)(xy & 0xffff) + (int64_t)(xy >> 16) * nx) * R + r];
    }
}

__global__ void k_rows_scatter(const float *__restrict__ compact, const int *__restrict__ vox_xy, int nx, int64_t nv,
                               int R, float *__restrict__ full)
{
    const int64_t n = nv * R;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = t / R;
        const int r = (int)(t - v * R);
        const int xy = vox_xy[v];
        full[((int64_t)(xy & 0xffff) + (int64_t)(xy >> 16) * nx) * R + r] = compact[t];
    }
}

// c <- c * g / (s + 1e-7); non-finite -> 0; negative -> 0
__global__ void k_bop_update(float *__restrict__ c, const float *__restrict__ g, const float *__restrict__ s,
                             int64_t n)
{
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        float v = (float)((double)c[t] * (double)g[t] / ((double)s[t] + 1e-7));
        if (!isfinite(v)) v = 0.f;
        if (v < 0.f) v = 0.f;
        c[t] = v;
    }
}

__global__ void k_to_float(const double *__restrict__ a, int64_t n, float *__restrict__ b)
{
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
        b[t] = (float)a[t];
}

int grid_of(int64_t n)
{
    int64_t b = (n + 255) / 256;
    return (int)(b < 1 ? 1 : (b > 65535 ? 65535 : b));
}

} // namespace

cudaError_t launch_rows_gather(const float *full, const int *vox_xy, int nx, int64_t nv, int R, float *compact,
                               cudaStream_t s, int64_t *launches)
{
    if (nv <= 0) return cudaSuccess;
    k_rows_gather<<<grid_of(nv * R), 256, 0, s>>>(full, vox_xy, nx, nv, R, compact);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

cudaError_t launch_rows_scatter(const float *compact, const int *vox_xy, int nx, int64_t nv, int R, float *full,
                                cudaStream_t s, int64_t *launches)
{
    if (nv <= 0) return cudaSuccess;
    k_rows_scatter<<<grid_of(nv * R), 256, 0, s>>>(compact, vox_xy, nx, nv, R, full);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

cudaError_t launch_bop_update(float *c, const float *g, const float *s, int64_t n, cudaStream_t st,
                              int64_t *launches)
{
    if (n <= 0) return cudaSuccess;
    k_bop_update<<<grid_of(n), 256, 0, st>>>(c, g, s, n);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

cudaError_t launch_to_float(const double *a, int64_t n, float *b, cudaStream_t s, int64_t *launches)
{
    if (n <= 0) return cudaSuccess;
    k_to_float<<<grid_of(n), 256, 0, s>>>(a, n, b);
    if (launches) (*launches)++;
    return cudaGetLastError();
}

} // namespace xrdt
