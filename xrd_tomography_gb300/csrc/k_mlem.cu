// k_mlem.cu -- MLEM with an explicit model matrix (main.m:154-176).
//
//   x <- x .* (A' * (y ./ (A*x + c + 1e-20))) ./ (sum(A,1)' + 1e-7)
//   x(~isfinite(x)) = 0;  x(x < 0) = 0
//
// A is the model matrix of Forward_XRD in its own layout: row r (a ray,
// src + det*SRC + nrg*SRC*DET) is the K = NWT*MAT contiguous floats
// Amatrix[:, :, ray] (main.m:140 reshapes it to [K, rays] and transposes).
//
// One iteration reads A once: a warp takes a ray, forms t = A(r,:).x with a
// shuffle reduction, the ratio y_r / (t + c_r + 1e-20), and adds ratio*A(r,:)
// into its register accumulators -- the same row, still in registers.  The
// pass is HBM-bound (2 flops per 4 bytes).  Each block writes its column
// sums to a partial row; the update kernel adds the partial rows in FP64,
// divides by the sensitivity sum(A,1) (also FP64) and applies the fix-ups.
#include "xrdt_device.cuh"

namespace xrdt {

namespace {

constexpr int kMlemThreads = 512;
constexpr int kMlemWarps = kMlemThreads / 32;

// KC = number of 128-column chunks (K <= 128*KC); lane l holds columns
// 4l..4l+3 of every chunk.
template <int KC, bool ONES>
__global__ void __launch_bounds__(kMlemThreads)
k_mlem_pass(const float *__restrict__ A, long long rays, int K, const float *__restrict__ y,
            const float *__restrict__ c, const float *__restrict__ x, float *__restrict__ partial)
{
    __shared__ float4 red[kMlemWarps][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int K4 = K >> 2;
    float4 xv[KC], g[KC];
#pragma unroll
    for (int i = 0; i < KC; i++) {
        const int q = lane + 32 * i;
        xv[i] = (!ONES && q < K4) ? reinterpret_cast<const float4 *>(x)[q] : make_float4(0.f, 0.f, 0.f, 0.f);
        g[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    // U rows per warp iteration keep U*KC 16-byte loads per lane in flight
    constexpr int U = KC <= 2 ? 4 : (KC <= 4 ? 2 : 1);
    const long long gw = (long long)blockIdx.x * kMlemWarps + wid;
    const long long nw = (long long)gridDim.x * kMlemWarps;
    for (long long r0 = gw; r0 < rays; r0 += U * nw) {
        float4 a[U][KC];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const long long r = r0 + u * nw;
            const float4 *row = reinterpret_cast<const float4 *>(A + (r < rays ? r : 0) * (long long)K);
#pragma unroll
            for (int i = 0; i < KC; i++) {
                const int q = lane + 32 * i;
                a[u][i] = (q < K4 && r < rays) ? __ldcs(row + q) : make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const long long r = r0 + u * nw;
            float ratio = r < rays ? 1.f : 0.f;
            if (!ONES) {
                float t = 0.f;
#pragma unroll
                for (int i = 0; i < KC; i++)
                    t = fmaf(a[u][i].x, xv[i].x,
                             fmaf(a[u][i].y, xv[i].y, fmaf(a[u][i].z, xv[i].z, fmaf(a[u][i].w, xv[i].w, t))));
                t = warp_sum(t);
                ratio = r < rays ? __ldg(y + r) / (t + __ldg(c + r) + 1e-20f) : 0.f;
            }
#pragma unroll
            for (int i = 0; i < KC; i++) {
                g[i].x = fmaf(ratio, a[u][i].x, g[i].x);
                g[i].y = fmaf(ratio, a[u][i].y, g[i].y);
                g[i].z = fmaf(ratio, a[u][i].z, g[i].z);
                g[i].w = fmaf(ratio, a[u][i].w, g[i].w);
            }
        }
    }
    // block sum of the warps' accumulators, one 128-column chunk at a time
#pragma unroll
    for (int i = 0; i < KC; i++) {
        red[wid][lane] = g[i];
        __syncthreads();
        if (threadIdx.x < 32) {
            float4 s = red[0][lane];
            for (int w = 1; w < kMlemWarps; w++) {
                const float4 v = red[w][lane];
                s.x += v.x;
                s.y += v.y;
                s.z += v.z;
                s.w += v.w;
            }
            const int q = lane + 32 * i;
            if (q < K4) reinterpret_cast<float4 *>(partial + (size_t)blockIdx.x * K)[q] = s;
        }
        __syncthreads();
    }
}

// Column sums of the partial rows in FP64, one warp per column (the lanes
// split the partial rows, so the loads overlap): the sensitivity (mode 0) or
// the back-projected ratio followed by the multiplicative update (mode 1).
__global__ void k_mlem_update(const float *__restrict__ partial, int nparts, int K, double *__restrict__ sens,
                              float *__restrict__ x, int mode)
{
    const int lane = threadIdx.x & 31;
    const int k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (k >= K) return;
    double s = 0.0;
    for (int p = lane; p < nparts; p += 32) s += (double)partial[(size_t)p * K + k];
    s = warp_sum(s);
    if (lane != 0) return;
    if (mode == 0) {
        sens[k] = s;
    } else {
        float v = (float)((double)x[k] * s / (sens[k] + 1e-7));
        if (!isfinite(v)) v = 0.f;   // main.m:163
        if (v < 0.f) v = 0.f;        // main.m:176
        x[k] = v;
    }
}

template <bool ONES>
cudaError_t launch_pass_kc(int kc, int blocks, const float *A, long long rays, int K, const float *y,
                           const float *c, const float *x, float *partial, cudaStream_t s)
{
    switch (kc) {
#define XRDT_KC(n)                                                                                   \
    case n:                                                                                          \
        k_mlem_pass<n, ONES><<<blocks, kMlemThreads, 0, s>>>(A, rays, K, y, c, x, partial);         \
        break;
        XRDT_KC(1) XRDT_KC(2) XRDT_KC(3) XRDT_KC(4) XRDT_KC(5) XRDT_KC(6) XRDT_KC(7) XRDT_KC(8)
#undef XRDT_KC
    default:
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

} // namespace

// Persistent grid: as many blocks as fit on the GPU at once.
int mlem_pass_blocks(int sm_count, int K)
{
    const int kc = (K + 127) / 128;
    int per_sm = 1;
    switch (kc) {
#define XRDT_OCC(n)                                                                                         \
    case n:                                                                                                 \
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mlem_pass<n, false>, kMlemThreads, 0);  \
        break;
        XRDT_OCC(1) XRDT_OCC(2) XRDT_OCC(3) XRDT_OCC(4) XRDT_OCC(5) XRDT_OCC(6) XRDT_OCC(7) XRDT_OCC(8)
#undef XRDT_OCC
    default:
        break;
    }
    if (per_sm < 1) per_sm = 1;
    return sm_count * per_sm;
}

cudaError_t launch_mlem_sensitivity(const float *A, long long rays, int K, float *partial, int nparts,
                                    double *sens, cudaStream_t s, int64_t *launches)
{
    const int kc = (K + 127) / 128;
    cudaError_t e = launch_pass_kc<true>(kc, nparts, A, rays, K, nullptr, nullptr, nullptr, partial, s);
    if (e != cudaSuccess) return e;
    k_mlem_update<<<(K + 7) / 8, 256, 0, s>>>(partial, nparts, K, sens, nullptr, 0);
    if (launches) (*launches) += 2;
    return cudaGetLastError();
}

cudaError_t launch_mlem_iteration(const float *A, long long rays, int K, const float *y, const float *c,
                                  float *x, float *partial, int nparts, const double *sens, cudaStream_t s,
                                  int64_t *launches)
{
    const int kc = (K + 127) / 128;
    cudaError_t e = launch_pass_kc<false>(kc, nparts, A, rays, K, y, c, x, partial, s);
    if (e != cudaSuccess) return e;
    k_mlem_update<<<(K + 7) / 8, 256, 0, s>>>(partial, nparts, K, const_cast<double *>(sens), x, 1);
    if (launches) (*launches) += 2;
    return cudaGetLastError();
}

} // namespace xrdt
