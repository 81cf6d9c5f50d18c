// Row pass over precomputed element matrices: the CSR values of a pattern
// with row groups are the fixed-order sums of the element matrices' rows.
//
// One warp per row group (<= 32 / P consecutive CSR rows whose slots, times
// P accumulator copies, fit SLOTS in shared memory); thread part p of row r
// walks the row's incidence records p, p + P, ... (ascending element order),
// loads row a of K_e (N doubles, the next record's row one step ahead) and
// adds it into its accumulator copy at the record's column offsets; the
// warp sums the copies in copy order and writes the group's slot range with
// coalesced stores.  No atomics: bitwise reproducible.
#pragma once

#include "skg_common.cuh"

namespace skg {

constexpr int kRowWarps = 4;  // warps per CTA in the row passes

template <int N, int SLOTS, int P>
__global__ void __launch_bounds__(kRowWarps * 32) k_rows_ke(int n_groups, const int2 *__restrict__ groups,
                                                           const int32_t *__restrict__ indptr,
                                                           const int32_t *__restrict__ inc_ptr,
                                                           const int4 *__restrict__ rec, const double *__restrict__ Ke,
                                                           double *__restrict__ values, RowRange rr) {
    static_assert(N % 2 == 0 && N <= 12, "rows are loaded as 16-byte pairs, at most 12 columns");
    extern __shared__ __align__(16) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gi = blockIdx.x * kRowWarps + warp;
    if (gi >= n_groups) return;
    double *acc = reinterpret_cast<double *>(smem + (size_t)warp * SLOTS * 8);
    const int2 grp = groups[gi];
    if (grp.x < rr.lo || grp.x >= rr.hi) return;  // row range of this launch
    const int32_t s0 = indptr[grp.x];
    const int nslots = indptr[grp.y] - s0;
    for (int j = lane; j < P * nslots; j += 32) acc[j] = 0.0;
    __syncwarp();
    const int ridx = lane / P, part = lane - (lane / P) * P;
    const int32_t r = grp.x + ridx;
    if (ridx < 32 / P && r < grp.y) {
        const int base = indptr[r] - s0 + part * nslots;
        const int32_t it1 = inc_ptr[r + 1];
        int32_t it = inc_ptr[r] + part;
        if (it < it1) {
            int4 rc = rec[it];
            double2 cur[N / 2];
            {
                const double2 *src = reinterpret_cast<const double2 *>(Ke + (int64_t)rc.x * N);
#pragma unroll
                for (int q = 0; q < N / 2; ++q) cur[q] = __ldg(src + q);
            }
            for (; it < it1; it += P) {
                const bool has_next = it + P < it1;
                int4 rcn = make_int4(0, 0, 0, 0);
                double2 nxt[N / 2];
                if (has_next) {
                    rcn = rec[it + P];
                    const double2 *src = reinterpret_cast<const double2 *>(Ke + (int64_t)rcn.x * N);
#pragma unroll
                    for (int q = 0; q < N / 2; ++q) nxt[q] = __ldg(src + q);
                }
                const unsigned ow[3] = {(unsigned)rc.y, (unsigned)rc.z, (unsigned)rc.w};
                int off[N];
#pragma unroll
                for (int bb = 0; bb < N; ++bb) off[bb] = base + (int)((ow[bb >> 2] >> (8 * (bb & 3))) & 0xffu);
                double a[N];
#pragma unroll
                for (int bb = 0; bb < N; ++bb) a[bb] = acc[off[bb]];
#pragma unroll
                for (int q = 0; q < N / 2; ++q) {
                    acc[off[2 * q]] = a[2 * q] + cur[q].x;
                    acc[off[2 * q + 1]] = a[2 * q + 1] + cur[q].y;
                }
                if (has_next) {
                    rc = rcn;
#pragma unroll
                    for (int q = 0; q < N / 2; ++q) cur[q] = nxt[q];
                }
            }
        }
    }
    __syncwarp();
    for (int j = lane; j < nslots; j += 32) {
        double v = acc[j];
#pragma unroll
        for (int c = 1; c < P; ++c) v += acc[c * nslots + j];
        values[s0 + j] = v;
    }
}

template <int N, int SLOTS, int P>
inline void launch_ke_class(int n_groups, const int2 *groups, const skg_pattern *pat, const double *Ke,
                            double *values, cudaStream_t s, RowRange rr = RowRange()) {
    if (n_groups == 0) return;
    const size_t smem = (size_t)kRowWarps * SLOTS * 8;
    if (smem > 48 * 1024)
        SKG_CUDA(cudaFuncSetAttribute(k_rows_ke<N, SLOTS, P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    const unsigned grid = (unsigned)((n_groups + kRowWarps - 1) / kRowWarps);
    k_rows_ke<N, SLOTS, P><<<grid, kRowWarps * 32, smem, s>>>(n_groups, groups, pat->indptr.get(),
                                                              pat->inc_ptr.get(), pat->rec.get(), Ke, values, rr);
    SKG_LAUNCH_CHECK("rows_ke");
}

// Sums element matrices Ke (E, N, N) into the CSR values of a pattern with
// row groups (pat->max_row_len > 0, square N x N element blocks).
template <int N>
inline void add_element_rows(const skg_pattern *pat, const double *Ke, double *values, cudaStream_t s,
                             RowRange rr = RowRange()) {
    launch_ke_class<N, kGroupSlotsSmall, 1>(pat->n_groups_small, pat->groups_small.get(), pat, Ke, values, s, rr);
    launch_ke_class<N, kGroupSlotsLarge, 2>(pat->n_groups_large, pat->groups_large.get(), pat, Ke, values, s, rr);
}

// Runs a row pass fn(RowRange) over all rows, or, with a host output,
// in row chunks of about equal slot counts: after each chunk's kernels the
// chunk's value range is copied to the page-locked h_values on a second
// stream while the next chunk runs.  A group that starts in one chunk and
// ends in the next is written by the first chunk's launch, before the copy of
// the second chunk's range, so every copied range is complete.  The caller's
// stream waits for the copies at the end.
void host_output_chunks(const skg_pattern *pat, int n_chunks, std::vector<int32_t> &rows, cudaStream_t s);
cudaStream_t copy_stream();

template <class F>
void run_row_pass(const skg_pattern *pat, double *d_values, double *h_values, cudaStream_t s, F &&fn) {
    if (!h_values) {
        fn(RowRange());
        return;
    }
    std::vector<int32_t> rows;
    host_output_chunks(pat, 8, rows, s);
    cudaStream_t cs = copy_stream();
    const std::vector<int32_t> &hp = pat->h_indptr;
    std::vector<cudaEvent_t> evs;
    for (size_t k = 0; k + 1 < rows.size(); ++k) {
        const int32_t r0 = rows[k], r1 = rows[k + 1];
        fn(RowRange{r0, r1});
        cudaEvent_t ev;
        SKG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        evs.push_back(ev);
        SKG_CUDA(cudaEventRecord(ev, s));
        SKG_CUDA(cudaStreamWaitEvent(cs, ev, 0));
        const size_t n = (size_t)(hp[r1] - hp[r0]);
        if (n)
            SKG_CUDA(cudaMemcpyAsync(h_values + hp[r0], d_values + hp[r0], n * sizeof(double), cudaMemcpyDeviceToHost,
                                     cs));
    }
    cudaEvent_t done;
    SKG_CUDA(cudaEventCreateWithFlags(&done, cudaEventDisableTiming));
    evs.push_back(done);
    SKG_CUDA(cudaEventRecord(done, cs));
    SKG_CUDA(cudaStreamWaitEvent(s, done, 0));
    for (cudaEvent_t ev : evs) cudaEventDestroy(ev);  // released once complete
}

}  // namespace skg
