// Shared host/device infrastructure of the GB300 assembly backend:
// status handling (no exception crosses the C ABI), stream-ordered device
// buffers, launch helpers and small device utilities.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "skfem_gb300.h"

namespace skg {

// GB300: 152 SMs (two dies of 76); grid-stride kernels size their grids by it.
constexpr int kSmCount = 152;

// ---------------------------------------------------------------- errors

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string &msg);

[[noreturn]] inline void fail(int code, const std::string &msg) { throw Error(code, msg); }

inline void check_cuda(cudaError_t e, const char *what) {
    if (e != cudaSuccess) {
        if (e == cudaErrorMemoryAllocation) {
            cudaGetLastError();
            fail(SKG_ENOMEM, std::string(what) + ": out of device memory");
        }
        fail(SKG_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
    }
}

#define SKG_CUDA(call) ::skg::check_cuda((call), #call)
#define SKG_LAUNCH_CHECK(name) ::skg::check_cuda(cudaGetLastError(), name)

inline void require(bool ok, const std::string &msg, int code = SKG_EINVAL) {
    if (!ok) fail(code, msg);
}

// Runs `body` and converts any failure into a status code + message.
template <class F>
int guarded(F &&body) {
    try {
        body();
        set_last_error("");
        return SKG_OK;
    } catch (const Error &e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::bad_alloc &) {
        set_last_error("host allocation failed");
        return SKG_ENOMEM;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return SKG_ECUDA;
    } catch (...) {
        set_last_error("unknown failure");
        return SKG_ECUDA;
    }
}

// ---------------------------------------------------------------- buffers

// Stream-ordered scratch comes from the device's default memory pool.  Its
// release threshold is raised once per device so that memory freed at the
// end of one assembly stays reserved for the next (the default threshold
// returns it to the CUDA driver at every synchronisation, and re-mapping
// gigabytes of scratch per call costs milliseconds).  The pool belongs to
// this process and ends with it.
inline void retain_pool_memory() {
    static bool done[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64 || done[dev]) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t threshold = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
    }
    done[dev] = true;
}

// Device buffer.  Temporaries are stream-ordered (cudaMallocAsync /
// cudaFreeAsync on the call's stream); buffers owned by handles, which may
// outlive the stream that created them, use plain cudaMalloc / cudaFree.
template <class T>
struct DevBuf {
    T *ptr = nullptr;
    size_t n = 0;
    cudaStream_t stream = nullptr;
    bool async = false;
    DevBuf() = default;
    DevBuf(size_t count, cudaStream_t s) : n(count), stream(s), async(true) {
        if (count) {
            retain_pool_memory();
            SKG_CUDA(cudaMallocAsync((void **)&ptr, count * sizeof(T), s));
        }
    }
    static DevBuf owned(size_t count) {
        DevBuf b;
        b.n = count;
        if (count) SKG_CUDA(cudaMalloc((void **)&b.ptr, count * sizeof(T)));
        return b;
    }
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : ptr(o.ptr), n(o.n), stream(o.stream), async(o.async) {
        o.ptr = nullptr; o.n = 0;
    }
    DevBuf &operator=(DevBuf &&o) noexcept {
        release();
        ptr = o.ptr; n = o.n; stream = o.stream; async = o.async;
        o.ptr = nullptr; o.n = 0;
        return *this;
    }
    ~DevBuf() { release(); }
    void release() {
        if (ptr) {
            if (async) cudaFreeAsync(ptr, stream);
            else cudaFree(ptr);
        }
        ptr = nullptr;
        n = 0;
    }
    T *get() const { return ptr; }
};

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// p (n doubles) in device memory: p itself.  In host memory the device can
// read (page-locked, or pageable on a device with pageable access): a device
// copy in `stage`, made by a coalesced read on the stream, so that kernels
// gathering from it at random do not cross the host link per access.
const double *device_resident(const double *p, int64_t n, DevBuf<double> &stage, cudaStream_t s);

// Device copy of a small host table (quadrature / basis tables of a few KB),
// made on first use per content and device and kept for the process, so
// that repeated assemblies need no host-to-device copy; in particular an
// assembly captured into a CUDA graph after one warm-up call replays without
// reading host memory.  Fails if the first use happens while s is capturing.
const double *device_table(const double *h, size_t n, cudaStream_t s);

inline unsigned grid_for(int64_t n, int block) {
    int64_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > 0x7fffffffLL) g = 0x7fffffffLL;
    return (unsigned)g;
}

// Exclusive scan of n int32 counts into out[0..n] (out[n] = total) on the
// stream; returns nothing (total read by the caller if needed).  Counts and
// totals must stay below 2^31.
void exclusive_scan_i32(const int32_t *d_in, int32_t *d_out, int64_t n, cudaStream_t s);

// ---------------------------------------------------------------- device

__device__ __forceinline__ int lower_bound_i32(const int32_t *b, int n, int32_t key) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (b[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

}  // namespace skg

namespace skg {
// The row groups one row-pass launch handles, per class (see skg_pattern).
struct GroupSet {
    int n_small = 0;
    const int2 *small = nullptr;
    int n_large = 0;
    const int2 *large = nullptr;
};

constexpr int kGroupSlotsSmall = 768;
constexpr int kGroupSlotsLarge = 2048;
// Row chunks of the host-output paths (values copied to host memory chunk by
// chunk while later chunks are computed).
constexpr int kHostChunks = 16;
constexpr int64_t kHostChunkMinNnz = int64_t(1) << 22;  // 32 MiB of values
}  // namespace skg

// Pattern handle (defined here so every translation unit sees the layout).
struct skg_pattern {
    int64_t n_elements = 0, n_rows = 0, n_cols = 0, nnz = 0;
    int32_t row_local = 0, col_local = 0;
    skg::DevBuf<int32_t> row_dofs;  // (E, row_local) copy
    skg::DevBuf<int32_t> col_dofs;  // (E, col_local) copy
    skg::DevBuf<int32_t> indptr;    // (n_rows+1)
    skg::DevBuf<int32_t> indices;   // (nnz)
    skg::DevBuf<int32_t> inc_ptr;   // (n_rows+1) incidences per row
    skg::DevBuf<int32_t> inc;       // (E*row_local) e*row_local + i, ascending per row
    // Longest row (columns); 0 when no incidence records were built.
    int32_t max_row_len = 0;
    // Row groups for the thread-per-row kernels: up to 32 consecutive rows
    // whose slots fit a warp's shared-memory budget, split into a class of
    // short groups (<= kGroupSlotsSmall slots) and long groups.  Each entry is
    // (first row, end row).
    int32_t n_groups_small = 0, n_groups_large = 0;
    skg::DevBuf<int2> groups_small, groups_large;
    // Host-output row chunks: up to kHostChunks row ranges of about equal
    // slot counts whose boundaries are group starts.  Chunk c covers rows
    // [hc_row[c], hc_row[c+1]) = slots [hc_slot[c], hc_slot[c+1]); its rows
    // reference elements below hc_ready[c] only.  The same groups as above,
    // ordered by chunk (then by first element), are hc_small / hc_large, and
    // chunk c's groups of a class start at hc_small_off[c] / hc_large_off[c].
    std::vector<int32_t> hc_row, hc_slot, hc_small_off, hc_large_off;
    std::vector<int64_t> hc_ready;
    skg::DevBuf<int2> hc_small, hc_large;
    // Incidence records (col_local <= 12 and every row shorter than 256):
    // one int4 per incidence in `inc` order, x = e*row_local + i and the
    // bytes of y, z, w = column offset within the row of each local column.
    skg::DevBuf<int4> rec;
};


