// Row pass over precomputed element matrices: the CSR values of a pattern
// with row groups are the fixed-order sums of the element matrices' rows.
//
// One warp per row group (<= 32 / P consecutive CSR rows whose slots, times
// P accumulator copies, fit SLOTS in shared memory); thread part p of row r
// walks the row's incidence records p, p + P, ... (ascending element order),
// loads row a of K_e (N doubles, the next record's row one step ahead, the
// records themselves two steps ahead) and adds it into its accumulator copy
// at the record's column offsets (the first incidence stores instead: an
// element's columns are distinct slots, so no slot is touched twice); the
// warp sums the copies in copy order and writes the group's slot range with
// coalesced stores.  No atomics: bitwise reproducible.  Optionally the same
// walk sums a per-incidence vector re (E * row_local, e.g. element residual
// entries) into residual[row], the P parts combined in part order.
#pragma once

#include <algorithm>
#include <vector>

#include "skg_common.cuh"

namespace skg {

constexpr int kRowWarps = 4;  // warps per CTA in the row passes

// One warp's share of the row pass: row group grp (rows [grp.x, grp.y)),
// accumulators in `acc` (SLOTS doubles of shared memory).  Each part's first
// incidence stores its row into the accumulators (the other slots start at
// zero), later incidences add.  See k_rows_ke.
template <int N, int SLOTS, int P>
__device__ __forceinline__ void rows_ke_warp(int2 grp, const int32_t *__restrict__ indptr,
                                             const int32_t *__restrict__ inc_ptr, const int4 *__restrict__ rec,
                                             const double *__restrict__ Ke, double *__restrict__ values,
                                             const double *__restrict__ re, double *__restrict__ residual,
                                             double *acc) {
    static_assert(N % 2 == 0 && N <= 12, "rows are loaded as 16-byte pairs, at most 12 columns");
    static_assert(P == 1 || P == 2, "one or two accumulator copies");
    const int lane = threadIdx.x & 31;
    const int32_t s0 = indptr[grp.x];
    const int nslots = indptr[grp.y] - s0;
    for (int j = lane; j < P * nslots; j += 32) acc[j] = 0.0;
    __syncwarp();
    const int ridx = lane / P, part = lane - (lane / P) * P;
    const int32_t r = grp.x + ridx;
    const bool live = ridx < 32 / P && r < grp.y;
    double rsum = 0.0;
    if (live) {
        const int base = indptr[r] - s0 + part * nslots;
        const int32_t it1 = inc_ptr[r + 1];
        int32_t it = inc_ptr[r] + part;
        if (it < it1) {
            // records run two incidences ahead of the rows they address, rows one
            int4 rc = rec[it];
            int4 rcn = it + P < it1 ? rec[it + P] : make_int4(0, 0, 0, 0);
            double2 cur[N / 2];
            {
                const double2 *src = reinterpret_cast<const double2 *>(Ke + (int64_t)rc.x * N);
#pragma unroll
                for (int q = 0; q < N / 2; ++q) cur[q] = __ldg(src + q);
            }
            bool first = true;
            for (; it < it1; it += P) {
                const bool has_next = it + P < it1;
                double2 nxt[N / 2];
                if (has_next) {
                    const double2 *src = reinterpret_cast<const double2 *>(Ke + (int64_t)rcn.x * N);
#pragma unroll
                    for (int q = 0; q < N / 2; ++q) nxt[q] = __ldg(src + q);
                }
                const int4 rcnn = it + 2 * P < it1 ? rec[it + 2 * P] : make_int4(0, 0, 0, 0);
                if (re) rsum += __ldg(re + rc.x);
                const unsigned ow[3] = {(unsigned)rc.y, (unsigned)rc.z, (unsigned)rc.w};
                int off[N];
#pragma unroll
                for (int bb = 0; bb < N; ++bb) off[bb] = base + (int)((ow[bb >> 2] >> (8 * (bb & 3))) & 0xffu);
                if (first) {
                    // an element's columns are distinct slots: no add needed
#pragma unroll
                    for (int q = 0; q < N / 2; ++q) {
                        acc[off[2 * q]] = cur[q].x;
                        acc[off[2 * q + 1]] = cur[q].y;
                    }
                    first = false;
                } else {
                    double a[N];
#pragma unroll
                    for (int bb = 0; bb < N; ++bb) a[bb] = acc[off[bb]];
#pragma unroll
                    for (int q = 0; q < N / 2; ++q) {
                        acc[off[2 * q]] = a[2 * q] + cur[q].x;
                        acc[off[2 * q + 1]] = a[2 * q + 1] + cur[q].y;
                    }
                }
                if (has_next) {
                    rc = rcn;
                    rcn = rcnn;
#pragma unroll
                    for (int q = 0; q < N / 2; ++q) cur[q] = nxt[q];
                }
            }
        }
    }
    if (re) {  // uniform across the warp: every lane takes part in the shuffle
        if constexpr (P == 2) rsum += __shfl_down_sync(0xffffffffu, rsum, 1);
        if (live && part == 0) residual[r] = rsum;
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
__global__ void __launch_bounds__(kRowWarps * 32) k_rows_ke(int n_groups, const int2 *__restrict__ groups,
                                                           const int32_t *__restrict__ indptr,
                                                           const int32_t *__restrict__ inc_ptr,
                                                           const int4 *__restrict__ rec, const double *__restrict__ Ke,
                                                           double *__restrict__ values, const double *__restrict__ re,
                                                           double *__restrict__ residual) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int warp = threadIdx.x >> 5;
    const int gi = blockIdx.x * kRowWarps + warp;
    if (gi >= n_groups) return;
    double *acc = reinterpret_cast<double *>(smem + (size_t)warp * SLOTS * 8);
    rows_ke_warp<N, SLOTS, P>(groups[gi], indptr, inc_ptr, rec, Ke, values, re, residual, acc);
}

template <int N, int SLOTS, int P>
inline void launch_ke_class(int n_groups, const int2 *groups, const skg_pattern *pat, const double *Ke,
                            double *values, cudaStream_t s, const double *re = nullptr,
                            double *residual = nullptr) {
    if (n_groups == 0) return;
    const size_t smem = (size_t)kRowWarps * SLOTS * 8;
    if (smem > 48 * 1024)
        SKG_CUDA(cudaFuncSetAttribute(k_rows_ke<N, SLOTS, P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    const unsigned grid = (unsigned)((n_groups + kRowWarps - 1) / kRowWarps);
    k_rows_ke<N, SLOTS, P><<<grid, kRowWarps * 32, smem, s>>>(n_groups, groups, pat->indptr.get(),
                                                              pat->inc_ptr.get(), pat->rec.get(), Ke, values, re,
                                                              residual);
    SKG_LAUNCH_CHECK("rows_ke");
}

inline GroupSet all_groups(const skg_pattern *pat) {
    return GroupSet{pat->n_groups_small, pat->groups_small.get(), pat->n_groups_large, pat->groups_large.get()};
}

// Groups of host-output chunk c.
inline GroupSet chunk_groups(const skg_pattern *pat, int c) {
    const int s0 = pat->hc_small_off[c], l0 = pat->hc_large_off[c];
    return GroupSet{pat->hc_small_off[c + 1] - s0, pat->hc_small.get() + s0, pat->hc_large_off[c + 1] - l0,
                    pat->hc_large.get() + l0};
}

// Sums element matrices Ke (E, N, N) into the CSR values of a pattern with
// row groups (pat->max_row_len > 0, square N x N element blocks).
template <int N>
inline void add_element_rows(const skg_pattern *pat, const double *Ke, double *values, cudaStream_t s,
                             const GroupSet &gs, const double *re = nullptr, double *residual = nullptr) {
    launch_ke_class<N, kGroupSlotsSmall, 1>(gs.n_small, gs.small, pat, Ke, values, s, re, residual);
    launch_ke_class<N, kGroupSlotsLarge, 2>(gs.n_large, gs.large, pat, Ke, values, s, re, residual);
}

// Per-device non-blocking side streams of the assembly passes.
enum class Side { copy = 0, rows = 1, minor = 2 };
cudaStream_t side_stream(Side which);

// Events of one assembly call, released at the end (an event destroyed
// while its work is pending is released once that work completes).
struct EventSet {
    std::vector<cudaEvent_t> evs;
    cudaEvent_t record(cudaStream_t s) {
        cudaEvent_t ev;
        SKG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        evs.push_back(ev);
        SKG_CUDA(cudaEventRecord(ev, s));
        return ev;
    }
    void order(cudaStream_t from, cudaStream_t to) {  // `to` waits for the work queued on `from`
        SKG_CUDA(cudaStreamWaitEvent(to, record(from), 0));
    }
    ~EventSet() {
        for (cudaEvent_t ev : evs) cudaEventDestroy(ev);
    }
};

// Row pass of a group set on stream st.  When both classes are present the
// class with fewer groups runs on the minor side stream at the same time: a
// class of a few groups is bound by the latency of one group's incidence
// walk and would otherwise leave the GPU idle behind the other class.
template <class FR>
void rows_on(const GroupSet &gs, cudaStream_t st, EventSet &ev, FR &&rows) {
    if (gs.n_small == 0 || gs.n_large == 0) {
        rows(gs, st);
        return;
    }
    const GroupSet small{gs.n_small, gs.small, 0, nullptr}, large{0, nullptr, gs.n_large, gs.large};
    const bool small_major = gs.n_small >= gs.n_large;
    cudaStream_t xs = side_stream(Side::minor);
    ev.order(st, xs);
    rows(small_major ? large : small, xs);
    rows(small_major ? small : large, st);
    ev.order(xs, st);
}

// All groups (both classes at once, see rows_on).
template <int N>
inline void add_element_rows(const skg_pattern *pat, const double *Ke, double *values, cudaStream_t s) {
    EventSet ev;
    rows_on(all_groups(pat), s, ev,
            [&](const GroupSet &gs, cudaStream_t st) { add_element_rows<N>(pat, Ke, values, st, gs); });
}

// Element pass and row pass of a pattern with row groups; elem(e0, e1)
// launches the element pass over elements [e0, e1) on s, rows(groups, st)
// the row pass of a group set on stream st.  The values optionally go to
// the page-locked host array h_values as well.
//
// Device output, or a host output of fewer than kHostChunkMinNnz values
// (where the chunks' launches and events would cost more than the overlap
// gains): elem(0, ne), the row pass of all groups on s, then one copy.
// Host output: the row chunks are taken in the order in which their elements
// are complete (hc_ready).  The element pass runs on s in steps of at least
// ne / kHostChunks elements, so launches stay large; each chunk's row pass
// runs on the rows side stream once the element steps it needs are done,
// overlapping the following element steps, and its slot range is then copied
// to h_values on the copy stream.  Every group lies inside one chunk, so each
// copied range is complete.  d_rowvec / h_rowvec (optional): a per-row vector
// the row pass also writes (a residual), copied with each chunk's rows.  At
// the end s waits for the copies, which waited for every row pass.
template <class FE, class FR>
void run_passes(const skg_pattern *pat, int64_t ne, double *d_values, double *h_values, cudaStream_t s, FE &&elem,
                FR &&rows, const double *d_rowvec = nullptr, double *h_rowvec = nullptr) {
    EventSet ev;
    if (!h_values || pat->nnz < kHostChunkMinNnz) {
        if (ne) elem((int64_t)0, ne);
        rows_on(all_groups(pat), s, ev, rows);
        if (h_values && pat->nnz)
            SKG_CUDA(cudaMemcpyAsync(h_values, d_values, (size_t)pat->nnz * sizeof(double), cudaMemcpyDeviceToHost, s));
        if (h_values && d_rowvec && h_rowvec && pat->n_rows)
            SKG_CUDA(cudaMemcpyAsync(h_rowvec, d_rowvec, (size_t)pat->n_rows * sizeof(double), cudaMemcpyDeviceToHost,
                                     s));
        return;
    }
    const int n_chunks = (int)pat->hc_ready.size();
    std::vector<int> order(n_chunks);
    for (int c = 0; c < n_chunks; ++c) order[c] = c;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return pat->hc_ready[a] < pat->hc_ready[b]; });
    const int64_t step = std::max<int64_t>(1, ne / kHostChunks);
    cudaStream_t rs = side_stream(Side::rows), cs = side_stream(Side::copy);
    try {
        ev.order(s, rs);  // inputs written earlier on s
        int64_t done = 0;
        for (int c : order) {
            const int64_t need = std::min(ne, pat->hc_ready[c]);
            if (need > done) {
                const int64_t to = std::min(ne, std::max(need, done + step));
                elem(done, to);
                done = to;
                ev.order(s, rs);
            }
            rows_on(chunk_groups(pat, c), rs, ev, rows);
            ev.order(rs, cs);
            const int64_t s0 = pat->hc_slot[c], n = pat->hc_slot[c + 1] - s0;
            if (n)
                SKG_CUDA(cudaMemcpyAsync(h_values + s0, d_values + s0, (size_t)n * sizeof(double),
                                         cudaMemcpyDeviceToHost, cs));
            const int64_t r0 = pat->hc_row[c], nr = pat->hc_row[c + 1] - r0;
            if (d_rowvec && h_rowvec && nr)
                SKG_CUDA(cudaMemcpyAsync(h_rowvec + r0, d_rowvec + r0, (size_t)nr * sizeof(double),
                                         cudaMemcpyDeviceToHost, cs));
        }
        if (done < ne) elem(done, ne);  // elements no row references
        ev.order(rs, cs);
        ev.order(cs, s);
    } catch (...) {
        // scratch freed on s after this call must outlive the queued work
        cudaEvent_t e;
        for (cudaStream_t st : {rs, cs, side_stream(Side::minor)})
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess) {
                cudaEventRecord(e, st);
                cudaStreamWaitEvent(s, e, 0);
                cudaEventDestroy(e);
            }
        throw;
    }
}

// Row pass alone (element data already computed), as run_passes.
template <class FR>
void run_row_pass(const skg_pattern *pat, double *d_values, double *h_values, cudaStream_t s, FR &&rows) {
    run_passes(pat, 0, d_values, h_values, s, [](int64_t, int64_t) {}, rows);
}

}  // namespace skg
