// Neo-Hookean residual and tangent on vector P1 tetrahedra.
//
// The reference keeps the law as scikit-fem forms
// (benchmarks/skfem_neo_hookean.py:8-52):
//   P = mu (F - F^-T) + lambda ln J F^-T,
//   A_iJkL = mu d_ik d_JL + (mu - lambda ln J) F^-T_iL F^-T_kJ + lambda F^-T_iJ F^-T_kL,
// assembled with NativeLinearForm (residual, linear_form_assembler.cpp:41-154)
// and NativeCrossBilinearForm.assemble_tensor (tangent,
// cross_bilinear_assembler.cpp:207-247).  For P1, F = I + grad u is constant
// on an element, so with g_a = grad lambda_a, h_a = F^-T g_a and the element
// measure V = |det J| * (sum of the rule's weights):
//   r_(a,c)          = V sum_j P_cj g_a,j
//   K_(a,i),(b,k)    = V [ mu d_ik (g_a . g_b) + (mu - lambda ln J) h_b,i h_a,k
//                          + lambda h_a,i h_b,k ]
// (the contraction of A with g_a and g_b written out).
//
// Fused path (patterns with row groups): one thread per element writes a
// 36-double record (g, h = F^-T g, V P and three scaled moduli); the row pass
// below evaluates each CSR row's 12 entries per incident element from the
// records and sums them in shared-memory slots in element order, together
// with the row's residual entry.  Nothing of size 144 per element is stored.
// Without row groups, one thread per element writes the 144 tangent and 12
// residual entries, summed by the fixed-order gathers.  Either way the results
// are bitwise reproducible (no atomics).
//
// The surrogate entry point replaces the law by a small MLP on the
// invariants (see skg_mlp.cu) with a per-element fallback to this law.
#include "skg_common.cuh"
#include "skg_df64.cuh"
#include "skg_nh.cuh"
#include "skg_nh_rows.cuh"

namespace skg {

void gather_element_matrices(const skg_pattern *pat, const double *Ke, double *values, cudaStream_t s);

namespace {

constexpr int kNhKeBlock = 128;
constexpr int kNhKeRound = 36;  // the three tangent rows of one vertex per staging round

// Element tangent (E, 12, 12; row (a,i), column (b,k)) and residual (E, 12)
// of the plain law for elements [e_begin, e_end), thread per element.  With
// h_a = F^-T g_a, p_a = (mu - lambda ln J) V h_a, q_a = lambda V h_a and
// G_ab = mu V g_a . g_b every entry is p_a,k h_b,i + q_a,i h_b,k (+ G_ab when
// i = k): two FP64 operations.  The matrix is symmetric (block (b,a) is block
// (a,b) transposed), so only the upper blocks and the upper halves of the
// diagonal blocks are evaluated; upper blocks are kept in registers until the
// rows of their lower twins are written.  The three rows of one vertex at a
// time go through a shared-memory stage, so that the block writes whole
// contiguous row triples.  Ke or re may be NULL (that output is skipped).
__global__ void __launch_bounds__(kNhKeBlock) k_nh_ke(int64_t ne, int64_t e_begin, int64_t e_end,
                                                     const double *__restrict__ p, int64_t npts,
                                                     const int32_t *__restrict__ t, const int32_t *__restrict__ dofs,
                                                     const double *__restrict__ u, double mu, double lmbda,
                                                     double wsum, double *__restrict__ Ke, double *__restrict__ re) {
    __shared__ double stage[kNhKeBlock * (kNhKeRound + 1)];
    const int64_t e0 = e_begin + (int64_t)blockIdx.x * kNhKeBlock;
    const int64_t e = e0 + threadIdx.x;
    double h[4][3], pp[4][3], qq[4][3], G[4][4], r[12];
    if (e < e_end) {
        NhGeom g;
        nh_geometry(p, npts, t, ne, e, wsum, g);
        double Gu[9];
        displacement_gradient(g, dofs + e * 12, u, Gu);
        NhLaw law;
        nh_plain_law(Gu, mu, lmbda, law);
        const double c2V = (mu - lmbda * law.lnJ) * g.V, lamV = lmbda * g.V, muV = mu * g.V;
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                h[a][i] = law.FiT[i * 3] * g.g[a][0] + law.FiT[i * 3 + 1] * g.g[a][1] + law.FiT[i * 3 + 2] * g.g[a][2];
                pp[a][i] = c2V * h[a][i];
                qq[a][i] = lamV * h[a][i];
                r[a * 3 + i] =
                    g.V * (law.P[i * 3] * g.g[a][0] + law.P[i * 3 + 1] * g.g[a][1] + law.P[i * 3 + 2] * g.g[a][2]);
            }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = a; b < 4; ++b) {
                G[a][b] = muV * (g.g[a][0] * g.g[b][0] + g.g[a][1] * g.g[b][1] + g.g[a][2] * g.g[b][2]);
                G[b][a] = G[a][b];
            }
    } else {
#pragma unroll
        for (int a = 0; a < 4; ++a) {
#pragma unroll
            for (int i = 0; i < 3; ++i) h[a][i] = pp[a][i] = qq[a][i] = r[a * 3 + i] = 0.0;
#pragma unroll
            for (int b = 0; b < 4; ++b) G[a][b] = 0.0;
        }
    }
    const int nvalid = (int)(e_end - e0 < kNhKeBlock ? e_end - e0 : kNhKeBlock);
    double *st = stage + threadIdx.x * (kNhKeRound + 1);
    double up[4][4][9];  // upper blocks (a < b), entry i * 3 + k; only those indices are used
#pragma unroll
    for (int rnd = 0; rnd < (Ke ? 4 : 0); ++rnd) {
        const int a = rnd;
        double dg[9];
#pragma unroll
        for (int b = 0; b < 4; ++b)
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    double v;
                    if (b > a) {
                        v = pp[a][k] * h[b][i] + qq[a][i] * h[b][k];
                        if (i == k) v += G[a][b];
                        up[a][b][i * 3 + k] = v;
                    } else if (b == a) {
                        if (k >= i) {
                            v = pp[a][k] * h[a][i] + qq[a][i] * h[a][k];
                            if (i == k) v += G[a][a];
                            dg[i * 3 + k] = v;
                        } else {
                            v = dg[k * 3 + i];
                        }
                    } else {
                        v = up[b][a][k * 3 + i];
                    }
                    st[i * 12 + b * 3 + k] = v;
                }
        __syncthreads();
        for (int x = threadIdx.x; x < nvalid * kNhKeRound; x += kNhKeBlock) {
            const int el = x / kNhKeRound, q = x - el * kNhKeRound;
            Ke[(e0 + el) * 144 + rnd * kNhKeRound + q] = stage[el * (kNhKeRound + 1) + q];
        }
        __syncthreads();
    }
    if (re) {
#pragma unroll
        for (int q = 0; q < 12; ++q) st[q] = r[q];
        __syncthreads();
        for (int x = threadIdx.x; x < nvalid * 12; x += kNhKeBlock) {
            const int el = x / 12, q = x - el * 12;
            re[(e0 + el) * 12 + q] = stage[el * (kNhKeRound + 1) + q];
        }
    }
}

// ------------------------------------------------------------------ row pass

constexpr int kNhWarps = 4;

// Row a_l = 3a + i of element e (plain record) -> val[12] and the residual term.
__device__ __forceinline__ void nh_plain_row(const double *__restrict__ R, int a, int i, double val[12],
                                             double &rr) {
    double ga[3], ha[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        ga[j] = R[a * 3 + j];
        ha[j] = R[12 + a * 3 + j];
    }
    const double muV = R[33], c2V = R[34], lamV = R[35];
    double alpha[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) alpha[k] = c2V * ha[k];
    const double beta = lamV * ha[i];
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        double gb[3], hb[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            gb[j] = R[b * 3 + j];
            hb[j] = R[12 + b * 3 + j];
        }
        const double gam = muV * (ga[0] * gb[0] + ga[1] * gb[1] + ga[2] * gb[2]);
        double hbi = hb[0];
        if (i == 1) hbi = hb[1];
        if (i == 2) hbi = hb[2];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            double v = alpha[k] * hbi + beta * hb[k];
            if (k == i) v += gam;
            val[b * 3 + k] = v;
        }
    }
    const double *PV = R + 24 + 3 * i;
    rr = PV[0] * ga[0] + PV[1] * ga[1] + PV[2] * ga[2];
}

// Row of element e from the surrogate record (FP32): precomputed tangent row
// and residual entry.
__device__ __forceinline__ void nh_surrogate_row(const float *__restrict__ R, int a, int i, float val[12],
                                                 float &rr) {
    const int l = a * 3 + i;
    const float4 *src = reinterpret_cast<const float4 *>(R + 12 * l);
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const float4 v = __ldg(src + q);
        val[4 * q] = v.x; val[4 * q + 1] = v.y; val[4 * q + 2] = v.z; val[4 * q + 3] = v.w;
    }
    rr = __ldg(R + 144 + l);
}

__device__ __forceinline__ df64 df_split(double v) {
    const float h = (float)v;
    return df64{h, (float)(v - (double)h)};
}

// Surrogate row pass with fallbacks: row groups as in the affine row pass
// (one warp per group of CSR rows, P threads per row walking its incidences
// in element order, per-copy slot sums in shared memory, summed in copy order
// and written coalesced); the FP32 surrogate rows and, for the elements
// flagged as fallback, the FP64 plain rows from their records, summed in
// double-float slots (a call in which every element falls back gives the
// plain law's values to ~1e-14).
//
// With `fallbacks` (the call's count of elements sent to the plain law) the
// kernel runs only when that count is nonzero, k_nh_rows_f32 otherwise; its
// warps then take groups grid-stride, so that the launch that finds nothing
// to do is a small grid.
template <int SLOTS, int P>
__global__ void __launch_bounds__(kNhWarps * 32) k_nh_rows(
    int n_groups, const int2 *__restrict__ groups, const int32_t *__restrict__ indptr,
    const int32_t *__restrict__ inc_ptr, const int4 *__restrict__ rec_inc, const double *__restrict__ recd,
    const float *__restrict__ recf, const unsigned char *__restrict__ flags,
    const unsigned long long *__restrict__ fallbacks, double *__restrict__ residual, double *__restrict__ values) {
    if (fallbacks && *fallbacks == 0) return;
    extern __shared__ __align__(16) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    df64 *accf = reinterpret_cast<df64 *>(smem + (size_t)warp * SLOTS * 8);
    for (int gi = blockIdx.x * kNhWarps + warp; gi < n_groups; gi += gridDim.x * kNhWarps) {
        const int2 grp = groups[gi];
        const int32_t s0 = indptr[grp.x];
        const int nslots = indptr[grp.y] - s0;
        for (int j = lane; j < P * nslots; j += 32) accf[j] = df64{0.f, 0.f};
        __syncwarp();
        const int ridx = lane / P, part = lane - (lane / P) * P;
        const int32_t r = grp.x + ridx;
        const bool live = ridx < 32 / P && r < grp.y;
        df64 rf{0.f, 0.f};
        if (live) {
            const int base = indptr[r] - s0 + part * nslots;
            const int32_t it1 = inc_ptr[r + 1];
            int32_t it = inc_ptr[r] + part;
            int4 rcn = it < it1 ? rec_inc[it] : make_int4(0, 0, 0, 0);  // records one incidence ahead
            for (; it < it1; it += P) {
                const int4 rc = rcn;
                if (it + P < it1) rcn = rec_inc[it + P];
                const int32_t e = rc.x / 12;
                const int l = rc.x - e * 12;
                const int a = l / 3, i = l - 3 * (l / 3);
                const unsigned ow[3] = {(unsigned)rc.y, (unsigned)rc.z, (unsigned)rc.w};
                int off[12];
#pragma unroll
                for (int bb = 0; bb < 12; ++bb) off[bb] = base + (int)((ow[bb >> 2] >> (8 * (bb & 3))) & 0xffu);
                if (flags[e]) {
                    double val[12], rr;
                    nh_plain_row(recd + (int64_t)e * kNhRecD, a, i, val, rr);
                    df64 acc[12];
#pragma unroll
                    for (int bb = 0; bb < 12; ++bb) acc[bb] = accf[off[bb]];
#pragma unroll
                    for (int bb = 0; bb < 12; ++bb) accf[off[bb]] = df_add(acc[bb], df_split(val[bb]));
                    rf = df_add(rf, df_split(rr));
                } else {
                    float val[12], rr;
                    nh_surrogate_row(recf + (int64_t)e * kNhRecF, a, i, val, rr);
                    df64 acc[12];
#pragma unroll
                    for (int bb = 0; bb < 12; ++bb) acc[bb] = accf[off[bb]];
#pragma unroll
                    for (int bb = 0; bb < 12; ++bb) {
                        const df64 sm = two_sum(acc[bb].hi, val[bb]);
                        accf[off[bb]] = df64{sm.hi, acc[bb].lo + sm.lo};
                    }
                    const df64 sm = two_sum(rf.hi, rr);
                    rf = df64{sm.hi, rf.lo + sm.lo};
                }
            }
        }
        // residual: combine the P parts of each row (lane order), part 0 writes
        if constexpr (P == 2) {
            const float h = __shfl_down_sync(0xffffffffu, rf.hi, 1), lo = __shfl_down_sync(0xffffffffu, rf.lo, 1);
            rf = df_add(fast_two_sum(rf.hi, rf.lo), fast_two_sum(h, lo));
        }
        if (live && part == 0 && residual) residual[r] = df_to_double(fast_two_sum(rf.hi, rf.lo), 0);
        __syncwarp();
        if (values) {
            for (int j = lane; j < nslots; j += 32) {
                // copies summed in double-float, converted by integer arithmetic (no FP64 pipe)
                df64 v = fast_two_sum(accf[j].hi, accf[j].lo);
#pragma unroll
                for (int c = 1; c < P; ++c) v = df_add(v, fast_two_sum(accf[c * nslots + j].hi, accf[c * nslots + j].lo));
                values[s0 + j] = df_to_double(v, 0);
            }
        }
        __syncwarp();  // the slots are zeroed again for the next group
    }
}

// Exact float -> double by integer arithmetic (FP32 subnormals through the
// conversion instruction: they do not occur in practice).
__device__ __forceinline__ double float_to_double_exact(float v) {
    const unsigned b = __float_as_uint(v);
    if ((b & 0x7f800000u) == 0 && (b & 0x7fffffu) != 0) return (double)v;
    return __longlong_as_double((long long)float_to_double_bits(v, 0));
}

// Surrogate row pass of a call in which no element fell back to the plain
// law (`*fallbacks` == 0; otherwise k_nh_rows runs instead): every incidence
// adds a precomputed FP32 tangent row, summed in FP32 slots (the network's
// own error, ~1e-5, is far above FP32 rounding), half the shared memory of
// double-float slots and so twice the resident warps; the residual entries in
// double-float registers.  Records run two incidences ahead of the rows they
// address, rows one (as k_rows_ke); each thread part's first incidence stores
// its row.  One warp per row group.
template <int SLOTS, int P>
__global__ void __launch_bounds__(kNhWarps * 32) k_nh_rows_f32(
    int n_groups, const int2 *__restrict__ groups, const int32_t *__restrict__ indptr,
    const int32_t *__restrict__ inc_ptr, const int4 *__restrict__ rec_inc, const float *__restrict__ recf,
    const unsigned long long *__restrict__ fallbacks, double *__restrict__ residual, double *__restrict__ values) {
    if (*fallbacks != 0) return;
    extern __shared__ __align__(16) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gi = blockIdx.x * kNhWarps + warp;
    if (gi >= n_groups) return;
    float *acc = reinterpret_cast<float *>(smem + (size_t)warp * SLOTS * 4);
    const int2 grp = groups[gi];
    const int32_t s0 = indptr[grp.x];
    const int nslots = indptr[grp.y] - s0;
    for (int j = lane; j < P * nslots; j += 32) acc[j] = 0.f;
    __syncwarp();
    const int ridx = lane / P, part = lane - (lane / P) * P;
    const int32_t r = grp.x + ridx;
    const bool live = ridx < 32 / P && r < grp.y;
    df64 rf{0.f, 0.f};
    // row l = 3a + i of element e: 12 FP32 tangent entries and the residual entry
    const auto load_row = [&](int32_t item, float v[12], float &rr) {
        const int32_t e = item / 12;
        const int l = item - e * 12;
        const float *R = recf + (int64_t)e * kNhRecF;
        const float4 *src = reinterpret_cast<const float4 *>(R + 12 * l);
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const float4 w = __ldg(src + q);
            v[4 * q] = w.x; v[4 * q + 1] = w.y; v[4 * q + 2] = w.z; v[4 * q + 3] = w.w;
        }
        rr = __ldg(R + 144 + l);
    };
    if (live) {
        const int base = indptr[r] - s0 + part * nslots;
        const int32_t it1 = inc_ptr[r + 1];
        int32_t it = inc_ptr[r] + part;
        if (it < it1) {
            int4 rc = rec_inc[it];
            int4 rcn = it + P < it1 ? rec_inc[it + P] : make_int4(0, 0, 0, 0);
            float cur[12], crr;
            load_row(rc.x, cur, crr);
            bool first = true;
            for (; it < it1; it += P) {
                const bool has_next = it + P < it1;
                float nxt[12], nrr = 0.f;
                if (has_next) load_row(rcn.x, nxt, nrr);
                const int4 rcnn = it + 2 * P < it1 ? rec_inc[it + 2 * P] : make_int4(0, 0, 0, 0);
                const unsigned ow[3] = {(unsigned)rc.y, (unsigned)rc.z, (unsigned)rc.w};
                int off[12];
#pragma unroll
                for (int bb = 0; bb < 12; ++bb) off[bb] = base + (int)((ow[bb >> 2] >> (8 * (bb & 3))) & 0xffu);
                if (first) {
                    // an element's columns are distinct slots: no add needed
#pragma unroll
                    for (int bb = 0; bb < 12; ++bb) acc[off[bb]] = cur[bb];
                    first = false;
                } else {
                    float a[12];
#pragma unroll
                    for (int bb = 0; bb < 12; ++bb) a[bb] = acc[off[bb]];
#pragma unroll
                    for (int bb = 0; bb < 12; ++bb) acc[off[bb]] = a[bb] + cur[bb];
                }
                const df64 sm = two_sum(rf.hi, crr);
                rf = df64{sm.hi, rf.lo + sm.lo};
                if (has_next) {
                    rc = rcn;
                    rcn = rcnn;
#pragma unroll
                    for (int bb = 0; bb < 12; ++bb) cur[bb] = nxt[bb];
                    crr = nrr;
                }
            }
        }
    }
    // residual: combine the P parts of each row (lane order), part 0 writes
    if constexpr (P == 2) {
        const float h = __shfl_down_sync(0xffffffffu, rf.hi, 1), lo = __shfl_down_sync(0xffffffffu, rf.lo, 1);
        rf = df_add(fast_two_sum(rf.hi, rf.lo), fast_two_sum(h, lo));
    }
    if (live && part == 0 && residual) residual[r] = df_to_double(fast_two_sum(rf.hi, rf.lo), 0);
    __syncwarp();
    if (values) {
        for (int j = lane; j < nslots; j += 32) {
            float v = acc[j];
#pragma unroll
            for (int c = 1; c < P; ++c) v += acc[c * nslots + j];
            values[s0 + j] = float_to_double_exact(v);
        }
    }
}

template <int SLOTS, int P>
void launch_nh_rows_f32(int n_groups, const int2 *groups, const skg_pattern *pat, const float *recf,
                        const unsigned long long *fallbacks, double *residual, double *values, cudaStream_t s) {
    if (n_groups == 0) return;
    const size_t smem = (size_t)kNhWarps * SLOTS * 4;
    if (smem > 48 * 1024)
        SKG_CUDA(cudaFuncSetAttribute(k_nh_rows_f32<SLOTS, P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    const unsigned grid = (unsigned)((n_groups + kNhWarps - 1) / kNhWarps);
    k_nh_rows_f32<SLOTS, P><<<grid, kNhWarps * 32, smem, s>>>(n_groups, groups, pat->indptr.get(),
                                                              pat->inc_ptr.get(), pat->rec.get(), recf, fallbacks,
                                                              residual, values);
    SKG_LAUNCH_CHECK("nh_rows_f32");
}

// With `fallbacks`: one wave of resident CTAs taking the groups grid-stride
// (the launch is a no-op when no element fell back).
template <int SLOTS, int P>
void launch_nh_rows(int n_groups, const int2 *groups, const skg_pattern *pat, const double *recd, const float *recf,
                    const unsigned char *flags, const unsigned long long *fallbacks, double *residual,
                    double *values, cudaStream_t s) {
    if (n_groups == 0) return;
    const size_t smem = (size_t)kNhWarps * SLOTS * 8;
    if (smem > 48 * 1024)
        SKG_CUDA(cudaFuncSetAttribute(k_nh_rows<SLOTS, P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    unsigned grid = (unsigned)((n_groups + kNhWarps - 1) / kNhWarps);
    if (fallbacks) {
        static int resident = 0;  // CTAs per SM, per instantiation (same on every GB300)
        if (!resident)
            SKG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, k_nh_rows<SLOTS, P>,
                                                                   kNhWarps * 32, smem));
        const unsigned wave = (unsigned)(resident > 0 ? resident : 1) * kSmCount;
        if (grid > wave) grid = wave;
    }
    k_nh_rows<SLOTS, P><<<grid, kNhWarps * 32, smem, s>>>(n_groups, groups, pat->indptr.get(),
                                                              pat->inc_ptr.get(), pat->rec.get(), recd, recf, flags,
                                                              fallbacks, residual, values);
    SKG_LAUNCH_CHECK("nh_rows");
}

// Residual gather: thread per DOF over its incidence list (element order).
__global__ void k_vector_gather(int64_t n_rows, const int32_t *__restrict__ inc_ptr, const int32_t *__restrict__ inc,
                                int L, const double *__restrict__ re, double *__restrict__ out) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rows) return;
    double acc = 0.0;
    for (int32_t it = inc_ptr[r]; it < inc_ptr[r + 1]; ++it) acc += re[inc[it]];
    out[r] = acc;
    (void)L;
}

}  // namespace

void nh_rows(const skg_pattern *pat, const GroupSet &gs, const double *recd, const float *recf,
             const unsigned char *flags, const unsigned long long *fallbacks, double *d_residual, double *d_values,
             cudaStream_t s) {
    // FP32 slots when no element fell back, double-float slots otherwise (each kernel reads the count)
    launch_nh_rows_f32<kGroupSlotsSmall, 1>(gs.n_small, gs.small, pat, recf, fallbacks, d_residual, d_values, s);
    launch_nh_rows_f32<kGroupSlotsLarge, 2>(gs.n_large, gs.large, pat, recf, fallbacks, d_residual, d_values, s);
    launch_nh_rows<kGroupSlotsSmall, 1>(gs.n_small, gs.small, pat, recd, recf, flags, fallbacks, d_residual,
                                              d_values, s);
    launch_nh_rows<kGroupSlotsLarge, 2>(gs.n_large, gs.large, pat, recd, recf, flags, fallbacks, d_residual,
                                              d_values, s);
}

// Whole-array copies of the results to the host (paths without row chunks).
void nh_download(const skg_pattern *pat, const double *d_residual, const double *d_values, double *h_residual,
                 double *h_values, cudaStream_t s) {
    if (h_values && d_values && pat->nnz)
        SKG_CUDA(cudaMemcpyAsync(h_values, d_values, (size_t)pat->nnz * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (h_residual && d_residual && pat->n_rows)
        SKG_CUDA(cudaMemcpyAsync(h_residual, d_residual, (size_t)pat->n_rows * sizeof(double),
                                 cudaMemcpyDeviceToHost, s));
}

void nh_gather(const skg_pattern *pat, const double *Ke, const double *re, double *d_residual, double *d_values,
               cudaStream_t s) {
    if (d_values && Ke) gather_element_matrices(pat, Ke, d_values, s);
    if (d_residual && re && pat->n_rows) {
        k_vector_gather<<<grid_for(pat->n_rows, 128), 128, 0, s>>>(pat->n_rows, pat->inc_ptr.get(), pat->inc.get(),
                                                                  pat->row_local, re, d_residual);
        SKG_LAUNCH_CHECK("nh_residual_gather");
    }
}

}  // namespace skg

using namespace skg;

namespace skg {
namespace {

// Plain-law residual and tangent; with h_values / h_residual (page-locked
// host) the results also go there, chunk by chunk on the fused path.
void nh_assemble(const skg_pattern *pat, const double *d_p, int64_t npts, const int32_t *d_t, int64_t ne,
                 const double *d_u, double mu, double lmbda, double wsum, double *d_residual, double *d_values,
                 double *h_residual, double *h_values, cudaStream_t s) {
    require(pat != nullptr, "pattern is NULL");
    require(pat->row_local == 12 && pat->n_elements == ne, "neo-Hookean assembly needs the vector P1 pattern");
    require(!d_values || pat->col_local == 12, "tangent output needs a pattern with CSR columns");
    require(ne == 0 || (d_p && d_t && d_u), "mesh or displacement arrays are NULL");
    DevBuf<double> u_stage;
    d_u = device_resident(d_u, pat->n_rows, u_stage, s);
    DevBuf<double> Ke(d_values ? (size_t)ne * 144 : 0, s), re(d_residual ? (size_t)ne * 12 : 0, s);
    auto elem = [&](int64_t e0, int64_t e1) {
        k_nh_ke<<<grid_for(e1 - e0, kNhKeBlock), kNhKeBlock, 0, s>>>(ne, e0, e1, d_p, npts, d_t, pat->row_dofs.get(),
                                                                    d_u, mu, lmbda, wsum, Ke.get(), re.get());
        SKG_LAUNCH_CHECK("nh_ke");
    };
    if (d_values && pat->max_row_len > 0) {  // element matrices, then fixed-order row sums
        run_passes(
            pat, ne, d_values, h_values, s, elem,
            [&](const GroupSet &gs, cudaStream_t st) {
                add_element_rows<12>(pat, Ke.get(), d_values, st, gs, re.get(), d_residual);
            },
            d_residual, h_residual);
        return;
    }
    if (ne) elem(0, ne);
    nh_gather(pat, Ke.get(), re.get(), d_residual, d_values, s);
    nh_download(pat, d_residual, d_values, h_residual, h_values, s);
}

}  // namespace
}  // namespace skg

extern "C" int skg_nh_assemble(const skg_pattern *pat, const double *d_p, int64_t npts, const int32_t *d_t,
                               int64_t ne, const double *d_u, double mu, double lmbda, double wsum,
                               double *d_residual, double *d_values, void *stream) {
    return guarded([&] {
        nh_assemble(pat, d_p, npts, d_t, ne, d_u, mu, lmbda, wsum, d_residual, d_values, nullptr, nullptr,
                    as_stream(stream));
    });
}

extern "C" int skg_nh_assemble_host(const skg_pattern *pat, const double *d_p, int64_t npts, const int32_t *d_t,
                                    int64_t ne, const double *d_u, double mu, double lmbda, double wsum,
                                    double *d_residual, double *d_values, double *h_residual, double *h_values,
                                    void *stream) {
    return guarded([&] {
        require(d_residual && d_values && h_residual && h_values, "device staging or host output is NULL");
        nh_assemble(pat, d_p, npts, d_t, ne, d_u, mu, lmbda, wsum, d_residual, d_values, h_residual, h_values,
                    as_stream(stream));
    });
}
