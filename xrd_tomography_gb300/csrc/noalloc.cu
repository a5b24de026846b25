// noalloc.cu -- MLEM with an explicit model matrix that allocates nothing.
//
// Some callers of this library cannot allocate device memory: code running
// inside a host framework that owns the whole device pool and forbids
// cudaMalloc in callbacks, real-time loops that must not risk an allocation
// failure or the synchronisation cudaMalloc/cudaFree imply, and embedders
// that only hand over pre-allocated buffers.  xrdt_mlem_matrix_noalloc serves
// them: it does what xrdt_mlem_matrix does, but its scratch -- the per-block
// partial column sums of the MLEM pass and the FP64 sensitivity -- lives in
// the fixed arrays below, which every GPU that loads the library holds until
// the process exits (2 MiB + 8 KiB per device).
//
// Device code could name the arrays directly; the host needs their device
// addresses, which cudaGetSymbolAddress returns per device.  The first call
// on a device looks them up (with that device current) and caches them, so
// that first call should come before any stream capture.  Every call shares
// the arrays: a call overwrites all the scratch it reads, but calls that
// overlap on the GPU (on different streams, or from different host threads
// without ordering) race on them.
#include <mutex>

#include "xrdt_device.cuh"

namespace {

constexpr int kMaxK = 1024;                          // columns the MLEM kernels take
constexpr size_t kScratchFloats = (size_t)1 << 19;   // 2 MiB of partial column sums
constexpr int kMaxDevices = 64;

static __device__ __align__(256) float g_mlem_partial[kScratchFloats];
static __device__ __align__(256) double g_mlem_sens[kMaxK];

struct SymbolAddrs {
    bool ready = false;
    float *partial = nullptr;
    double *sens = nullptr;
};

std::mutex g_mutex;
SymbolAddrs g_addrs[kMaxDevices];

// Addresses of the scratch arrays on the current device (looked up once).
int scratch_addresses(int device, float **partial, double **sens)
{
    if (device < 0 || device >= kMaxDevices) return XRDT_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_mutex);
    SymbolAddrs &a = g_addrs[device];
    if (!a.ready) {
        void *p = nullptr, *s = nullptr;
        if (cudaGetSymbolAddress(&p, g_mlem_partial) != cudaSuccess ||
            cudaGetSymbolAddress(&s, g_mlem_sens) != cudaSuccess) {
            cudaGetLastError();
            return XRDT_ERR_CUDA;
        }
        a.partial = (float *)p;
        a.sens = (double *)s;
        a.ready = true;
    }
    *partial = a.partial;
    *sens = a.sens;
    return XRDT_OK;
}

// Device memory of `device` (or managed memory): a buffer of another GPU
// would be read through peer access, and the scratch belongs to the current
// device only.
bool on_device(const void *p, int device)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeDevice && a.device == device;
}

} // namespace

extern "C" int32_t xrdt_mlem_matrix_noalloc(const float *A, int64_t rays, int32_t K, const float *y,
                                            const float *c, float *x, int32_t iters, void *stream)
{
    if (!A || !y || !c || !x) return XRDT_ERR_NULL;
    if (rays < 1 || K < 4 || K > kMaxK || (K & 3) || iters < 0) return XRDT_ERR_DIMS;
    int device = 0, sms = 0;
    if (cudaGetDevice(&device) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
        cudaGetLastError();
        return XRDT_ERR_CUDA;
    }
    if (!on_device(A, device) || !on_device(y, device) || !on_device(c, device) || !on_device(x, device))
        return XRDT_ERR_UNSUPPORTED;
    // the MLEM pass reads rows of A and x as 16-byte vectors
    if (((uintptr_t)A | (uintptr_t)x) & 15) return XRDT_ERR_UNSUPPORTED;
    float *partial;
    double *sens;
    int rc = scratch_addresses(device, &partial, &sens);
    if (rc) return rc;
    // as many partial rows as the pass wants, up to what the scratch holds
    int nparts = xrdt::mlem_pass_blocks(sms, K);
    const int cap = (int)(kScratchFloats / (size_t)K);
    if (nparts > cap) nparts = cap;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = xrdt::launch_mlem_sensitivity(A, rays, K, partial, nparts, sens, st, nullptr);
    for (int it = 0; it < iters && e == cudaSuccess; it++)
        e = xrdt::launch_mlem_iteration(A, rays, K, y, c, x, partial, nparts, sens, st, nullptr);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return XRDT_ERR_CUDA;
    }
    return XRDT_OK;
}
