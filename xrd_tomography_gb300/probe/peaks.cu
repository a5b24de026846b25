// peaks.cu -- throughput probes for the roofline denominators that the
// driver's peak file does not carry: FP32 FMA, the SFU exp2, FP64 FMA.
//
// Each probe runs a kernel of independent dependency chains (8 per thread,
// enough to cover the pipeline latency) on every SM and returns operations
// per second measured with CUDA events.  Built into libxrdt_probe.so, which
// only the benchmark loads.
#include <cuda_runtime.h>
#include <stdint.h>

namespace {

constexpr int kChains = 8;

__global__ void k_fma32(float *out, int iters, float a, float b)
{
    float x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = threadIdx.x * 1e-3f + c;
    for (int i = 0; i < iters; i++)
#pragma unroll
        for (int c = 0; c < kChains; c++) x[c] = fmaf(x[c], a, b);
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += x[c];
    if (s == 1.2345f) out[threadIdx.x] = s;
}

__global__ void k_ex2(float *out, int iters, float a)
{
    float x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = -(threadIdx.x & 7) * 1e-3f - c * 1e-2f;
    for (int i = 0; i < iters; i++)
#pragma unroll
        for (int c = 0; c < kChains; c++) {
            float y;
            asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x[c]));
            x[c] = y * a - 1.0f;   // stays in (-1, 0]
        }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += x[c];
    if (s == 1.2345f) out[threadIdx.x] = s;
}

__global__ void k_fma64(double *out, int iters, double a, double b)
{
    double x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = threadIdx.x * 1e-3 + c;
    for (int i = 0; i < iters; i++)
#pragma unroll
        for (int c = 0; c < kChains; c++) x[c] = fma(x[c], a, b);
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += x[c];
    if (s == 1.2345) out[threadIdx.x] = s;
}

template <class F>
double timed(F launch, double ops)
{
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    launch();  // warm-up
    cudaEventRecord(a);
    launch();
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (cudaGetLastError() != cudaSuccess || ms <= 0.f) return -1.0;
    return ops / (ms * 1e-3);
}

} // namespace

extern "C" {

// kind: 0 = FP32 FMA (flop/s, 2 per FMA), 1 = exp2 on the SFU (op/s),
// 2 = FP64 FMA (flop/s).  Returns -1 on error.
double xrdt_probe_peak(int kind)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    void *buf = nullptr;
    if (cudaMalloc(&buf, 1 << 16) != cudaSuccess) return -1.0;
    const int threads = 512, blocks = sms * 4;
    double r = -1.0;
    if (kind == 0) {
        const int iters = 1 << 14;
        r = timed([&] { k_fma32<<<blocks, threads>>>((float *)buf, iters, 0.999f, 1e-3f); },
                  2.0 * kChains * (double)iters * threads * blocks);
    } else if (kind == 1) {
        const int iters = 1 << 12;
        r = timed([&] { k_ex2<<<blocks, threads>>>((float *)buf, iters, 0.5f); },
                  (double)kChains * iters * threads * blocks);
    } else if (kind == 2) {
        const int iters = 1 << 9;
        r = timed([&] { k_fma64<<<blocks, threads>>>((double *)buf, iters, 0.999, 1e-3); },
                  2.0 * kChains * (double)iters * threads * blocks);
    }
    cudaFree(buf);
    return r;
}

} // extern "C"
