// Library-wide C ABI entry points: version, per-thread last error, device
// capabilities the host side needs.
#include <algorithm>
#include <string>

#include "skg_common.cuh"

namespace skg {
namespace {
thread_local std::string g_last_error;
}
void set_last_error(const std::string &msg) { g_last_error = msg; }
}  // namespace skg

extern "C" int skg_version(void) { return 100; }

extern "C" const char *skg_last_error(void) { return skg::g_last_error.c_str(); }

extern "C" int skg_device_pageable_access(int32_t *out) {
    return skg::guarded([&] {
        skg::require(out != nullptr, "output pointer is NULL");
        int dev = 0, v = 0;
        SKG_CUDA(cudaGetDevice(&dev));
        SKG_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev));
        *out = v;
    });
}

namespace skg {
namespace {
__global__ void k_stage(const double *__restrict__ src, double *__restrict__ dst, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}
}  // namespace

const double *device_resident(const double *p, int64_t n, DevBuf<double> &stage, cudaStream_t s) {
    if (!p || n <= 0) return p;
    cudaPointerAttributes attr{};
    SKG_CUDA(cudaPointerGetAttributes(&attr, p));
    if (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged) return p;
    stage = DevBuf<double>((size_t)n, s);
    const int64_t blocks = std::min<int64_t>((n + 255) / 256, 4 * kSmCount);
    k_stage<<<(unsigned)blocks, 256, 0, s>>>(p, stage.get(), n);
    SKG_LAUNCH_CHECK("stage");
    return stage.get();
}

}  // namespace skg
