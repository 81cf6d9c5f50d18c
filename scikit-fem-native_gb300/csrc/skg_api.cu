// Library-wide C ABI entry points: version, per-thread last error, device
// capabilities the host side needs.
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
