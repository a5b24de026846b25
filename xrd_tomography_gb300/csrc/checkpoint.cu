// checkpoint.cu -- MLEM checkpoints: the estimate and the iteration count in
// a file, so that a long reconstruction can stop and continue.
//
// File layout (this library's byte order): "XRDTMLEM", u32 version 1, u32 0,
// i64 element count, i64 iteration, the float estimate, then a 64-bit FNV-1a
// checksum of everything before it.  A write goes to "<path>.tmp" and is
// renamed over path once complete, so an interrupted write leaves the
// previous checkpoint intact.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "xrdt.h"

namespace {

const char kMagic[8] = {'X', 'R', 'D', 'T', 'M', 'L', 'E', 'M'};

uint64_t fnv1a(uint64_t h, const void *p, size_t n)
{
    const unsigned char *b = static_cast<const unsigned char *>(p);
    for (size_t i = 0; i < n; i++) {
        h ^= b[i];
        h *= 1099511628211ull;
    }
    return h;
}

struct Header {
    char magic[8];
    uint32_t version, reserved;
    int64_t n, iteration;
};

bool on_device(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

} // namespace

extern "C" int32_t xrdt_mlem_checkpoint_write(const char *path, const float *x, int64_t n, int64_t iteration)
{
    if (!path || !x) return XRDT_ERR_NULL;
    if (n < 1 || iteration < 0) return XRDT_ERR_DIMS;
    std::vector<float> host;
    const float *src = x;
    if (on_device(x)) {
        host.resize((size_t)n);
        if (cudaMemcpy(host.data(), x, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost) != cudaSuccess) {
            cudaGetLastError();
            return XRDT_ERR_CUDA;
        }
        src = host.data();
    }
    Header h;
    memcpy(h.magic, kMagic, 8);
    h.version = 1;
    h.reserved = 0;
    h.n = n;
    h.iteration = iteration;
    uint64_t sum = fnv1a(1469598103934665603ull, &h, sizeof h);
    sum = fnv1a(sum, src, sizeof(float) * (size_t)n);
    const std::string tmp = std::string(path) + ".tmp";
    FILE *f = fopen(tmp.c_str(), "wb");
    if (!f) return XRDT_ERR_IO;
    bool ok = fwrite(&h, sizeof h, 1, f) == 1 && fwrite(src, sizeof(float), (size_t)n, f) == (size_t)n &&
              fwrite(&sum, sizeof sum, 1, f) == 1;
    ok = (fclose(f) == 0) && ok;
    if (!ok || rename(tmp.c_str(), path) != 0) {
        remove(tmp.c_str());
        return XRDT_ERR_IO;
    }
    return XRDT_OK;
}

extern "C" int32_t xrdt_mlem_checkpoint_read(const char *path, float *x, int64_t n, int64_t *iteration)
{
    if (!path || !x || !iteration) return XRDT_ERR_NULL;
    if (n < 1) return XRDT_ERR_DIMS;
    FILE *f = fopen(path, "rb");
    if (!f) return XRDT_ERR_IO;
    Header h;
    std::vector<float> data;
    uint64_t stored = 0;
    bool ok = fread(&h, sizeof h, 1, f) == 1 && memcmp(h.magic, kMagic, 8) == 0 && h.version == 1 && h.n == n &&
              h.iteration >= 0;
    if (ok) {
        data.resize((size_t)n);
        ok = fread(data.data(), sizeof(float), (size_t)n, f) == (size_t)n && fread(&stored, sizeof stored, 1, f) == 1;
    }
    char extra;
    ok = ok && fread(&extra, 1, 1, f) == 0;   // nothing after the checksum
    fclose(f);
    if (!ok) return XRDT_ERR_INPUT;
    uint64_t sum = fnv1a(1469598103934665603ull, &h, sizeof h);
    sum = fnv1a(sum, data.data(), sizeof(float) * (size_t)n);
    if (sum != stored) return XRDT_ERR_INPUT;
    if (on_device(x)) {
        if (cudaMemcpy(x, data.data(), sizeof(float) * (size_t)n, cudaMemcpyHostToDevice) != cudaSuccess) {
            cudaGetLastError();
            return XRDT_ERR_CUDA;
        }
    } else {
        memcpy(x, data.data(), sizeof(float) * (size_t)n);
    }
    *iteration = h.iteration;
    return XRDT_OK;
}
