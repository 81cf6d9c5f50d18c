// Library-wide C ABI entry points: version, per-thread last error, device
// capabilities the host side needs.
#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

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

// ---------------------------------------------------------------- FP64 rate
// Measured FP64 FMA throughput of this device: every thread of a full grid
// runs eight independent FMA chains; the time of one launch (CUDA events on
// the stream) gives FMAs per second.  The FP64 roof against which the FP64
// assembly passes are reported.
namespace skg {
namespace {
constexpr int kRateBlocksPerSm = 4, kRateThreads = 256, kRateIters = 1024;

__global__ void __launch_bounds__(kRateThreads) k_fp64_rate(double *out, int iters, double a, double b) {
    double x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = threadIdx.x + k;
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += x[k];
    out[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace
}  // namespace skg

extern "C" int skg_fp64_fma_rate(double *h_gfma, void *stream) {
    return skg::guarded([&] {
        using namespace skg;
        require(h_gfma != nullptr, "output pointer is NULL");
        cudaStream_t s = as_stream(stream);
        int dev = 0, sms = 0;
        SKG_CUDA(cudaGetDevice(&dev));
        SKG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        const int blocks = sms * kRateBlocksPerSm;
        DevBuf<double> out((size_t)blocks * kRateThreads, s);
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        float ms = 0.f;
        try {
            SKG_CUDA(cudaEventCreate(&e0));
            SKG_CUDA(cudaEventCreate(&e1));
            k_fp64_rate<<<blocks, kRateThreads, 0, s>>>(out.get(), 64, 1.0000001, 1e-9);  // warm-up
            SKG_LAUNCH_CHECK("fp64_rate");
            SKG_CUDA(cudaEventRecord(e0, s));
            k_fp64_rate<<<blocks, kRateThreads, 0, s>>>(out.get(), kRateIters, 1.0000001, 1e-9);
            SKG_LAUNCH_CHECK("fp64_rate");
            SKG_CUDA(cudaEventRecord(e1, s));
            SKG_CUDA(cudaEventSynchronize(e1));
            SKG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        } catch (...) {
            if (e0) cudaEventDestroy(e0);
            if (e1) cudaEventDestroy(e1);
            throw;
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        const double fmas = 8.0 * kRateIters * (double)blocks * kRateThreads;
        *h_gfma = fmas / ((double)ms * 1e-3) / 1e9;
    });
}

namespace skg {

const double *device_table(const double *h, size_t n, cudaStream_t s) {
    static std::mutex mu;
    static std::map<std::pair<int, std::vector<double>>, double *> cache;
    int dev = 0;
    SKG_CUDA(cudaGetDevice(&dev));
    std::pair<int, std::vector<double>> key(dev, std::vector<double>(h, h + n));
    std::lock_guard<std::mutex> lock(mu);
    const auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    SKG_CUDA(cudaStreamIsCapturing(s, &cap));
    require(cap == cudaStreamCaptureStatusNone,
            "assembly tables are built on the first call: run the assembly once before capturing it");
    double *d = nullptr;
    SKG_CUDA(cudaMalloc((void **)&d, std::max<size_t>(n, 1) * sizeof(double)));
    if (n) SKG_CUDA(cudaMemcpy(d, h, n * sizeof(double), cudaMemcpyHostToDevice));
    cache.emplace(std::move(key), d);
    return d;
}

}  // namespace skg
