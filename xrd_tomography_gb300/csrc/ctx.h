// ctx.h -- the library context (xrdt_ctx) shared by the C ABI's source files.
#pragma once

#include <cstdlib>
#include <string>
#include <vector>

#include "xrdt_device.cuh"

struct xrdt_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string err;
    int64_t launches = 0;
    // grow-only device buffers, one per slot
    std::vector<void *> buf;
    std::vector<size_t> cap;
    int *h_counters = nullptr;  // pinned
    // profiling: events bracketing launches, folded into totals on query
    bool profiling = false;
    struct Pending {
        int kernel;
        cudaEvent_t a, b;
    };
    std::vector<Pending> pending;
    int64_t prof_launches[XRDT_KERNEL_COUNT] = {};
    double prof_ms[XRDT_KERNEL_COUNT] = {};
    unsigned long long *d_work = nullptr;  // exp2 evaluations of the forward kernel
    // MLEM iteration captured as a graph, keyed by its arguments
    cudaGraphExec_t mlem_exec = nullptr;
    const void *mlem_key[6] = {};
    long long mlem_rays = 0;
    int mlem_K = 0;
};

namespace xrdt {

// Failure injection on the host: while the environment variable
// XRDT_TEST_FAIL_ALLOC is "1", every device allocation the library makes
// reports failure, as on a device that is full, so that callers can check
// that XRDT_ERR_ALLOC comes back and that the context stays usable.
inline bool test_alloc_fails()
{
    const char *e = getenv("XRDT_TEST_FAIL_ALLOC");
    return e && e[0] == '1';
}

// Brackets one kernel group with events when profiling is on.
struct ProfScope {
    xrdt_ctx *ctx;
    int kernel;
    cudaEvent_t a = nullptr, b = nullptr;
    ProfScope(xrdt_ctx *c, int k) : ctx(c), kernel(k)
    {
        if (!ctx->profiling) return;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, ctx->stream);
    }
    ~ProfScope()
    {
        if (!a) return;
        cudaEventRecord(b, ctx->stream);
        ctx->pending.push_back({kernel, a, b});
    }
};

inline bool is_device_ptr(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

} // namespace xrdt
