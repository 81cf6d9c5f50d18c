// CSR sparsity pattern on the device.
//
// Same result as the reference's per-row "collect, sort, unique" pattern
// (cpp/src/assembly/bilinear_form_assembler.cpp:111-116 and the identical
// rule in cross_bilinear_assembler.cpp and edge_topology.cpp:86-154), built
// GPU-first:
//   1. row incidence lists: for every row r the (element, local row) pairs
//      whose row dof is r, as e*row_local+i, sorted ascending.  These lists
//      are kept: every assembly on the pattern sums a slot's contributions
//      in this order, which makes the result run-to-run deterministic;
//   2. per row, one warp gathers the candidate columns of its incidences into
//      shared memory, sorts them with a bitonic network and counts / writes
//      the unique ones (rows with more candidates than fit in shared memory
//      use a slower repeated-minimum extraction over global memory).
#include <climits>
#include <algorithm>
#include <vector>

#include <mutex>

#include "skg_common.cuh"
#include "skg_rows.cuh"

namespace skg {

namespace {

constexpr int kScanBlock = 1024;

__global__ void k_scan_block(const int32_t *in, int32_t *out, int32_t *block_sums, int64_t n) {
    __shared__ int32_t s[kScanBlock];
    const int64_t i = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
    const int32_t v = i < n ? in[i] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < kScanBlock; off <<= 1) {
        int32_t t = threadIdx.x >= off ? s[threadIdx.x - off] : 0;
        __syncthreads();
        s[threadIdx.x] += t;
        __syncthreads();
    }
    if (i < n) out[i] = s[threadIdx.x] - v;  // exclusive
    if (threadIdx.x == kScanBlock - 1 && block_sums) block_sums[blockIdx.x] = s[threadIdx.x];
}

__global__ void k_scan_add(int32_t *out, const int32_t *offsets, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
    if (i < n) out[i] += offsets[blockIdx.x];
}

__global__ void k_set_total(const int32_t *in, int32_t *out, int64_t n) {
    // out[n] = out[n-1] + in[n-1]
    if (threadIdx.x == 0 && blockIdx.x == 0) out[n] = n ? out[n - 1] + in[n - 1] : 0;
}

void scan_rec(const int32_t *in, int32_t *out, int64_t n, cudaStream_t s) {
    const int64_t nb = (n + kScanBlock - 1) / kScanBlock;
    if (nb <= 1) {
        k_scan_block<<<1, kScanBlock, 0, s>>>(in, out, nullptr, n);
        SKG_LAUNCH_CHECK("scan");
        return;
    }
    DevBuf<int32_t> sums(nb, s), offs(nb, s);
    k_scan_block<<<(unsigned)nb, kScanBlock, 0, s>>>(in, out, sums.get(), n);
    SKG_LAUNCH_CHECK("scan");
    scan_rec(sums.get(), offs.get(), nb, s);
    k_scan_add<<<(unsigned)nb, kScanBlock, 0, s>>>(out, offs.get(), n);
    SKG_LAUNCH_CHECK("scan_add");
}

}  // namespace

void exclusive_scan_i32(const int32_t *d_in, int32_t *d_out, int64_t n, cudaStream_t s) {
    if (n > 0) scan_rec(d_in, d_out, n, s);
    k_set_total<<<1, 32, 0, s>>>(d_in, d_out, n);
    SKG_LAUNCH_CHECK("scan_total");
}

namespace {

__global__ void k_check_range(const int32_t *v, int64_t n, int64_t hi, int32_t *err) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t x = v[i];
        if (x < 0 || x >= hi) atomicMin(err, (int32_t)(i < (int64_t)INT_MAX - 1 ? i : (int64_t)INT_MAX - 1));
    }
}

__global__ void k_count_rows(const int32_t *row_dofs, int64_t total, int32_t *cnt) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&cnt[row_dofs[i]], 1);
}

__global__ void k_fill_incidence(const int32_t *row_dofs, int64_t total, const int32_t *inc_ptr,
                                 int32_t *cursor, int32_t *inc) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t r = row_dofs[i];
        const int32_t pos = inc_ptr[r] + atomicAdd(&cursor[r], 1);
        inc[pos] = (int32_t)i;
    }
}

// Thread per row: insertion sort of the (short) incidence list.
__global__ void k_sort_incidence(const int32_t *inc_ptr, int32_t *inc, int64_t n_rows) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rows) return;
    const int32_t b = inc_ptr[r], e = inc_ptr[r + 1];
    for (int32_t k = b + 1; k < e; ++k) {
        const int32_t x = inc[k];
        int32_t j = k - 1;
        while (j >= b && inc[j] > x) {
            inc[j + 1] = inc[j];
            --j;
        }
        inc[j + 1] = x;
    }
}

constexpr int kWarpsPerBlock = 4;
constexpr int kCap = 1024;  // candidates per warp held in shared memory

// Warp per row.  mode 0: write the unique-column count to counts[r];
// mode 1: write the unique columns to indices[indptr[r]...].
__global__ void k_row_columns(const int32_t *inc_ptr, const int32_t *inc, const int32_t *col_dofs,
                              int32_t row_local, int32_t col_local, int64_t n_rows, int mode,
                              int32_t *counts, const int32_t *indptr, int32_t *indices) {
    __shared__ int32_t smem[kWarpsPerBlock * kCap];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t r = (int64_t)blockIdx.x * kWarpsPerBlock + warp;
    if (r >= n_rows) return;
    const int32_t ib = inc_ptr[r];
    const int32_t ninc = inc_ptr[r + 1] - ib;
    const int64_t n = (int64_t)ninc * col_local;
    int32_t *buf = smem + warp * kCap;
    if (n <= kCap) {
        int P = 1;
        while (P < n) P <<= 1;
        for (int k = lane; k < P; k += 32) {
            int32_t v = INT_MAX;
            if (k < n) {
                const int32_t item = inc[ib + k / col_local];
                const int32_t e = item / row_local;
                v = col_dofs[(int64_t)e * col_local + k % col_local];
            }
            buf[k] = v;
        }
        __syncwarp();
        for (int size = 2; size <= P; size <<= 1) {
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                for (int t = lane; t < P / 2; t += 32) {
                    const int lo = 2 * t - (t & (stride - 1));
                    const int hi = lo + stride;
                    const bool up = (lo & size) == 0;
                    const int32_t a = buf[lo], c = buf[hi];
                    if ((a > c) == up) { buf[lo] = c; buf[hi] = a; }
                }
                __syncwarp();
            }
        }
        int32_t written = 0;
        const int32_t base = mode == 1 ? indptr[r] : 0;
        for (int k0 = 0; k0 < n; k0 += 32) {
            const int k = k0 + lane;
            const bool first = k < n && (k == 0 || buf[k] != buf[k - 1]);
            const unsigned m = __ballot_sync(0xffffffffu, first);
            if (mode == 1 && first) indices[base + written + __popc(m & ((1u << lane) - 1u))] = buf[k];
            written += __popc(m);
        }
        if (mode == 0 && lane == 0) counts[r] = written;
        return;
    }
    // Large row: extract the distinct columns in increasing order.
    int32_t last = INT_MIN, written = 0;
    const int32_t base = mode == 1 ? indptr[r] : 0;
    for (;;) {
        int32_t best = INT_MAX;
        for (int64_t k = lane; k < n; k += 32) {
            const int32_t item = inc[ib + k / col_local];
            const int32_t e = item / row_local;
            const int32_t v = col_dofs[(int64_t)e * col_local + k % col_local];
            if (v > last && v < best) best = v;
        }
        for (int off = 16; off > 0; off >>= 1) best = min(best, __shfl_xor_sync(0xffffffffu, best, off));
        if (best == INT_MAX) break;
        if (mode == 1 && lane == 0) indices[base + written] = best;
        ++written;
        last = best;
    }
    if (mode == 0 && lane == 0) counts[r] = written;
}

// Thread per row: column offsets of every incidence's local columns.
__global__ void k_records(int64_t n_rows, const int32_t *__restrict__ indptr, const int32_t *__restrict__ indices,
                          const int32_t *__restrict__ inc_ptr, const int32_t *__restrict__ inc,
                          const int32_t *__restrict__ col_dofs, int32_t row_local, int32_t col_local,
                          int4 *__restrict__ rec) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rows) return;
    const int32_t rb = indptr[r], rn = indptr[r + 1] - rb;
    const int32_t *cols = indices + rb;
    for (int32_t it = inc_ptr[r]; it < inc_ptr[r + 1]; ++it) {
        const int32_t item = inc[it];
        const int64_t e = item / row_local;
        unsigned w[3] = {0u, 0u, 0u};
        for (int k = 0; k < col_local; ++k) {
            const int pos = lower_bound_i32(cols, rn, col_dofs[e * col_local + k]);
            w[k >> 2] |= (unsigned)(pos & 0xff) << (8 * (k & 3));
        }
        rec[it] = make_int4(item, (int)w[0], (int)w[1], (int)w[2]);
    }
}

}  // namespace

// First and last element referenced by each row (incidences are in ascending
// element order; rows without incidences: INT_MAX and -1).
__global__ void k_element_span(int64_t n_rows, const int32_t *__restrict__ inc_ptr, const int32_t *__restrict__ inc,
                               int32_t row_local, int2 *__restrict__ span) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rows) return;
    const int32_t i0 = inc_ptr[r], i1 = inc_ptr[r + 1];
    span[r] = i0 < i1 ? make_int2(inc[i0] / row_local, inc[i1 - 1] / row_local) : make_int2(INT_MAX, -1);
}

// Incidence records for the warp-per-row assembly kernels; skipped when the
// pattern is unsuitable (elements wider than 12 columns or rows of 256+
// columns), in which case assemblies use the per-row global-memory gather.
void build_records(skg_pattern *p, cudaStream_t s) {
    if (p->col_local > 12 || p->n_rows == 0) return;
    std::vector<int32_t> ip(p->n_rows + 1);
    SKG_CUDA(cudaMemcpyAsync(ip.data(), p->indptr.get(), ip.size() * 4, cudaMemcpyDeviceToHost, s));
    SKG_CUDA(cudaStreamSynchronize(s));
    int32_t longest = 0;
    for (int64_t r = 0; r < p->n_rows; ++r) longest = std::max(longest, ip[r + 1] - ip[r]);
    if (longest > 255) return;
    const int64_t n_inc = p->n_elements * p->row_local;
    p->rec = DevBuf<int4>::owned(n_inc);
    k_records<<<grid_for(p->n_rows, 128), 128, 0, s>>>(p->n_rows, p->indptr.get(), p->indices.get(),
                                                       p->inc_ptr.get(), p->inc.get(), p->col_dofs.get(),
                                                       p->row_local, p->col_local, p->rec.get());
    SKG_LAUNCH_CHECK("records");
    // Row groups.  A group first takes up to 32 consecutive rows within
    // kGroupSlotsSmall slots (one thread per row); when fewer than 24 rows
    // fit (long rows), it is re-formed as up to 16 rows within
    // kGroupSlotsLarge / 2 slots, served by two threads per row with one
    // accumulator copy each.
    std::vector<int2> small, large, all;  // `all`: every group, in row order
    int64_t r = 0;
    while (r < p->n_rows) {
        const int64_t r0 = r;
        int64_t r1 = r0;
        while (r1 < p->n_rows && r1 - r0 < 32 && ip[r1 + 1] - ip[r0] <= kGroupSlotsSmall) ++r1;
        if (r1 - r0 >= 24 || r1 == p->n_rows) {
            if (r1 == r0) r1 = r0 + 1;
            small.push_back(make_int2((int)r0, (int)r1));
        } else {
            r1 = r0;
            while (r1 < p->n_rows && r1 - r0 < 16 && ip[r1 + 1] - ip[r0] <= kGroupSlotsLarge / 2) ++r1;
            if (r1 == r0) r1 = r0 + 1;  // single row above the budget (cannot happen below 256 columns)
            large.push_back(make_int2((int)r0, (int)r1));
        }
        all.push_back(make_int2((int)r0, (int)r1));
        r = r1;
    }
    std::vector<int2> span(p->n_rows);
    {
        DevBuf<int2> d_span(p->n_rows, s);
        k_element_span<<<grid_for(p->n_rows, 256), 256, 0, s>>>(p->n_rows, p->inc_ptr.get(), p->inc.get(),
                                                              p->row_local, d_span.get());
        SKG_LAUNCH_CHECK("element_span");
        SKG_CUDA(cudaMemcpyAsync(span.data(), d_span.get(), span.size() * 8, cudaMemcpyDeviceToHost, s));
        SKG_CUDA(cudaStreamSynchronize(s));
    }
    // Order the groups by the first element they reference, so that groups
    // running at the same time touch a compact band of elements (their
    // per-element data stays in L2).  Each group still owns a contiguous
    // slot range, so the output writes stay coalesced.
    auto first_element = [&](const int2 &g) {
        int32_t m = INT_MAX;
        for (int32_t q = g.x; q < g.y; ++q) m = std::min(m, span[q].x);
        return m;
    };
    auto sort_by = [](std::vector<int2> &vec, const std::vector<int64_t> &key) {
        std::vector<size_t> order(vec.size());
        for (size_t i = 0; i < order.size(); ++i) order[i] = i;
        std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return key[a] < key[b]; });
        std::vector<int2> out(vec.size());
        for (size_t i = 0; i < order.size(); ++i) out[i] = vec[order[i]];
        vec.swap(out);
    };
    for (auto *vec : {&small, &large}) {
        std::vector<int64_t> key(vec->size());
        for (size_t i = 0; i < vec->size(); ++i) key[i] = first_element((*vec)[i]);
        sort_by(*vec, key);
    }
    // Host-output chunks: boundaries at group starts near equal slot counts.
    const int64_t nnz = ip[p->n_rows];
    p->hc_row.assign(1, 0);
    for (int k = 1; k < kHostChunks; ++k) {
        const int64_t target = nnz * k / kHostChunks;
        const auto it = std::lower_bound(all.begin(), all.end(), target,
                                         [&](const int2 &g, int64_t t) { return (int64_t)ip[g.x] < t; });
        if (it != all.end() && it->x > p->hc_row.back()) p->hc_row.push_back(it->x);
    }
    p->hc_row.push_back((int32_t)p->n_rows);
    const int n_chunks = (int)p->hc_row.size() - 1;
    p->hc_slot.resize(n_chunks + 1);
    for (int c = 0; c <= n_chunks; ++c) p->hc_slot[c] = ip[p->hc_row[c]];
    p->hc_ready.assign(n_chunks, 0);
    auto chunk_of = [&](int32_t row) {
        return (int)(std::upper_bound(p->hc_row.begin(), p->hc_row.end(), row) - p->hc_row.begin()) - 1;
    };
    for (int c = 0; c < n_chunks; ++c)
        for (int32_t q = p->hc_row[c]; q < p->hc_row[c + 1]; ++q)
            p->hc_ready[c] = std::max(p->hc_ready[c], (int64_t)span[q].y + 1);
    std::vector<int2> hc_small = small, hc_large = large;
    for (auto *vec : {&hc_small, &hc_large}) {
        std::vector<int64_t> key(vec->size());
        for (size_t i = 0; i < vec->size(); ++i) key[i] = chunk_of((*vec)[i].x);
        sort_by(*vec, key);  // stable: first-element order within a chunk
    }
    auto offsets = [&](const std::vector<int2> &vec, std::vector<int32_t> &off) {
        off.assign(n_chunks + 1, 0);
        for (const int2 &g : vec) ++off[chunk_of(g.x) + 1];
        for (int c = 0; c < n_chunks; ++c) off[c + 1] += off[c];
    };
    offsets(hc_small, p->hc_small_off);
    offsets(hc_large, p->hc_large_off);
    auto upload = [&](const std::vector<int2> &vec, DevBuf<int2> &dst) {
        dst = DevBuf<int2>::owned(vec.size());
        if (!vec.empty())
            SKG_CUDA(cudaMemcpyAsync(dst.get(), vec.data(), vec.size() * 8, cudaMemcpyHostToDevice, s));
    };
    p->n_groups_small = (int32_t)small.size();
    p->n_groups_large = (int32_t)large.size();
    upload(small, p->groups_small);
    upload(large, p->groups_large);
    upload(hc_small, p->hc_small);
    upload(hc_large, p->hc_large);
    SKG_CUDA(cudaStreamSynchronize(s));
    p->max_row_len = longest;
}

}  // namespace skg

using namespace skg;

extern "C" int skg_pattern_create(const int32_t *d_row_dofs, const int32_t *d_col_dofs,
                                  int64_t n_elements, int32_t row_local, int32_t col_local,
                                  int64_t n_rows, int64_t n_cols, void *stream, skg_pattern **out) {
    return guarded([&] {
        require(out != nullptr, "output handle pointer is NULL");
        *out = nullptr;
        // CSR columns when column DOFs are given (for an empty mesh, whose arrays
        // may be NULL, when the column width is)
        const bool with_csr = d_col_dofs != nullptr || (n_elements == 0 && col_local > 0);
        if (!with_csr) col_local = 0;
        require(n_elements >= 0 && row_local > 0 && (col_local > 0 || !with_csr), "invalid pattern sizes");
        require(n_rows >= 0 && n_cols >= 0, "invalid matrix shape");
        require(n_elements == 0 || d_row_dofs, "dof arrays are NULL");
        const int64_t tr = n_elements * row_local, tc = n_elements * col_local;
        require(tr < INT_MAX && tc < INT_MAX && n_rows < INT_MAX && n_cols < INT_MAX,
                "pattern too large for 32-bit element indexing");
        require(n_elements * row_local * (int64_t)col_local < (int64_t)INT_MAX * 8,
                "pattern too large");
        cudaStream_t s = as_stream(stream);
        auto *p = new skg_pattern();
        try {
            p->n_elements = n_elements; p->row_local = row_local; p->col_local = col_local;
            p->n_rows = n_rows; p->n_cols = n_cols;
            p->row_dofs = DevBuf<int32_t>::owned(tr);
            p->col_dofs = DevBuf<int32_t>::owned(tc);
            if (tr) SKG_CUDA(cudaMemcpyAsync(p->row_dofs.get(), d_row_dofs, tr * 4, cudaMemcpyDeviceToDevice, s));
            if (tc) SKG_CUDA(cudaMemcpyAsync(p->col_dofs.get(), d_col_dofs, tc * 4, cudaMemcpyDeviceToDevice, s));
            // range checks (the reference raises "element DOF index is out of bounds")
            DevBuf<int32_t> err(2, s);
            const int32_t init[2] = {INT_MAX, INT_MAX};
            SKG_CUDA(cudaMemcpyAsync(err.get(), init, sizeof(init), cudaMemcpyHostToDevice, s));
            if (tr) k_check_range<<<grid_for(tr, 256), 256, 0, s>>>(p->row_dofs.get(), tr, n_rows, err.get());
            if (tc) k_check_range<<<grid_for(tc, 256), 256, 0, s>>>(p->col_dofs.get(), tc, n_cols, err.get() + 1);
            SKG_LAUNCH_CHECK("check_range");
            int32_t herr[2];
            SKG_CUDA(cudaMemcpyAsync(herr, err.get(), sizeof(herr), cudaMemcpyDeviceToHost, s));
            SKG_CUDA(cudaStreamSynchronize(s));
            require(herr[0] == INT_MAX && herr[1] == INT_MAX, "element DOF index is out of bounds", SKG_ERANGE);

            DevBuf<int32_t> cnt(n_rows + 1, s), cursor(n_rows + 1, s);
            SKG_CUDA(cudaMemsetAsync(cnt.get(), 0, (n_rows + 1) * 4, s));
            SKG_CUDA(cudaMemsetAsync(cursor.get(), 0, (n_rows + 1) * 4, s));
            if (tr) k_count_rows<<<grid_for(tr, 256), 256, 0, s>>>(p->row_dofs.get(), tr, cnt.get());
            SKG_LAUNCH_CHECK("count_rows");
            p->inc_ptr = DevBuf<int32_t>::owned(n_rows + 1);
            exclusive_scan_i32(cnt.get(), p->inc_ptr.get(), n_rows, s);
            p->inc = DevBuf<int32_t>::owned(tr);
            if (tr) k_fill_incidence<<<grid_for(tr, 256), 256, 0, s>>>(p->row_dofs.get(), tr, p->inc_ptr.get(), cursor.get(), p->inc.get());
            SKG_LAUNCH_CHECK("fill_incidence");
            if (n_rows) k_sort_incidence<<<grid_for(n_rows, 128), 128, 0, s>>>(p->inc_ptr.get(), p->inc.get(), n_rows);
            SKG_LAUNCH_CHECK("sort_incidence");
            if (!with_csr) {
                p->indptr = DevBuf<int32_t>::owned(n_rows + 1);
                SKG_CUDA(cudaMemsetAsync(p->indptr.get(), 0, (n_rows + 1) * 4, s));
                SKG_CUDA(cudaStreamSynchronize(s));
                *out = p;
                return;
            }
            const unsigned gw = grid_for(n_rows, kWarpsPerBlock);
            if (n_rows)
                k_row_columns<<<gw, 32 * kWarpsPerBlock, 0, s>>>(p->inc_ptr.get(), p->inc.get(), p->col_dofs.get(),
                                                                 row_local, col_local, n_rows, 0, cnt.get(), nullptr, nullptr);
            SKG_LAUNCH_CHECK("row_columns_count");
            p->indptr = DevBuf<int32_t>::owned(n_rows + 1);
            exclusive_scan_i32(cnt.get(), p->indptr.get(), n_rows, s);
            int32_t nnz = 0;
            SKG_CUDA(cudaMemcpyAsync(&nnz, p->indptr.get() + n_rows, 4, cudaMemcpyDeviceToHost, s));
            SKG_CUDA(cudaStreamSynchronize(s));
            require(nnz >= 0, "pattern too large for 32-bit CSR offsets");
            p->nnz = nnz;
            p->indices = DevBuf<int32_t>::owned(nnz);
            if (n_rows)
                k_row_columns<<<gw, 32 * kWarpsPerBlock, 0, s>>>(p->inc_ptr.get(), p->inc.get(), p->col_dofs.get(),
                                                                 row_local, col_local, n_rows, 1, nullptr, p->indptr.get(),
                                                                 p->indices.get());
            SKG_LAUNCH_CHECK("row_columns_write");
            SKG_CUDA(cudaStreamSynchronize(s));
            build_records(p, s);
        } catch (...) {
            delete p;
            throw;
        }
        *out = p;
    });
}

extern "C" int skg_pattern_destroy(skg_pattern *pattern) {
    return guarded([&] { delete pattern; });
}

extern "C" int skg_pattern_info(const skg_pattern *p, int64_t *nnz, int64_t *n_rows, int64_t *n_cols) {
    return guarded([&] {
        require(p != nullptr, "pattern is NULL");
        if (nnz) *nnz = p->nnz;
        if (n_rows) *n_rows = p->n_rows;
        if (n_cols) *n_cols = p->n_cols;
    });
}

namespace skg {
namespace {
__global__ void k_widen(const int32_t *in, int64_t *out, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = in[i];
}
}  // namespace
}  // namespace skg

extern "C" int skg_pattern_export(const skg_pattern *p, int64_t *d_indptr, int32_t *d_indices, void *stream) {
    return guarded([&] {
        require(p != nullptr, "pattern is NULL");
        cudaStream_t s = as_stream(stream);
        if (d_indptr) {
            k_widen<<<grid_for(p->n_rows + 1, 256), 256, 0, s>>>(p->indptr.get(), d_indptr, p->n_rows + 1);
            SKG_LAUNCH_CHECK("export_indptr");
        }
        if (d_indices && p->nnz)
            SKG_CUDA(cudaMemcpyAsync(d_indices, p->indices.get(), p->nnz * 4, cudaMemcpyDeviceToDevice, s));
    });
}

extern "C" int skg_pattern_row_groups(const skg_pattern *p, int32_t *max_row_len) {
    return guarded([&] {
        require(p != nullptr && max_row_len != nullptr, "pattern or output is NULL");
        *max_row_len = p->max_row_len;
    });
}

namespace skg {

// Non-blocking side streams per device (copy, rows, minor class).  The row
// streams have the highest priority: their blocks are scheduled ahead of the
// element pass running beside them, so each chunk's values are ready for its
// copy as early as possible.
cudaStream_t side_stream(Side which) {
    static std::mutex mu;
    static cudaStream_t streams[64][3] = {};
    int dev = 0;
    SKG_CUDA(cudaGetDevice(&dev));
    require(dev >= 0 && dev < 64, "device index out of range");
    const int k = (int)which;
    std::lock_guard<std::mutex> lock(mu);
    if (!streams[dev][k]) {
        int least = 0, greatest = 0;
        SKG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        const int priority = which == Side::copy ? least : greatest;
        SKG_CUDA(cudaStreamCreateWithPriority(&streams[dev][k], cudaStreamNonBlocking, priority));
    }
    return streams[dev][k];
}
}  // namespace skg
