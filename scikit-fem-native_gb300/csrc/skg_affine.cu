// Fused assembly of scalar P1/P2 diffusion on affine tetrahedra -- the hot
// path of `asm(BilinearForm, Basis)` for w.kappa * ddot(grad u, grad v) and
// dot(mul(A, grad u), grad v) (python/skfemntv/forms.py:276-374 through
// bilinear_form_assembler.cpp:79-105 / cross_bilinear_assembler.cpp:207-247).
//
// Math.  On an affine tetrahedron every P1/P2 basis gradient is a linear
// combination of the four barycentric gradients g_k = b_k / det J (b_k the
// rows of adj J, b_0 = -(b_1+b_2+b_3)):  grad N_a = sum_k c^k_a(xi) g_k with
// c^k_a = delta_ka (P1), (4 lambda_a - 1) delta_ka (P2 vertex) and
// 4 lambda_j, 4 lambda_i on the ends of P2 edge (i, j)
// (python/skfemntv/basis.py:2224-2235).  Hence
//     K_ab = sum_{k,l} G_kl T^{kl}_ab,   G_kl = b_k . A b_l / |det J|,
//     T^{kl}_ab = sum_q w_q c^k_a(xi_q) c^l_b(xi_q),
// T tabulated on the host from the caller's quadrature rule (same rule, same
// sum as the reference, reassociated).  Only (k, l) in the supports of a and
// b contribute: 1 term for vertex-vertex, 2 vertex-edge, 4 edge-edge.
//
// Passes.
//  1. element pass (thread per element): G (4x4) from coordinates and the
//     coefficient, written to a scratch array.
//  2. row pass (CTA per row block): the block's CSR slots live in shared
//     memory; one thread per row walks the row's incidence records
//     (element, local row, column offsets) in ascending element order,
//     evaluates row a of K_e on the fly and adds it into the row's slots;
//     the block then writes its slot range out once, coalesced.  Every slot
//     is summed by one thread in a fixed order: results are bitwise
//     reproducible, with no atomics.
//
// Precision modes.
//  SKG_FP64           FP64 end to end (FP64 pipe).
//  SKG_FP64_EMULATED  element pass and row pass in double-float (FP32 pairs,
//                     error-free transformations; ~48-bit significands) and
//                     slot sums in double-float, converted to FP64 exactly:
//                     FP64-accurate (1e-12 class) on the FP32 pipe.
//  SKG_SPLIT_FP32     double-float element pass (FP64-class G), element
//                     contraction in FP32 with split hi/lo products and FP32
//                     accumulation, double-float slot sums.
// The FP32-pair modes work in units scaled by 2^-s (s from the largest
// vertex coordinate) so FP32 range holds; a mesh or coefficient outside that
// range is detected in the element pass and re-run in FP64.
#include <climits>
#include <cmath>
#include <vector>

#include "skg_common.cuh"
#include "skg_df64.cuh"

namespace skg {
namespace {

struct Support {
    int sup[10][2];
};

// Barycentric support of local basis function b: P1 and P2 vertex functions
// use lambda_b; P2 edge function 4 + k uses the two end vertices of edge k
// ((0,1),(1,2),(2,0),(0,3),(1,3),(2,3)).  Compile-time so that unrolled
// loops index registers, not local memory.
__host__ __device__ constexpr int sup_lo(int b) {
    return b < 4 ? b : (b == 4 ? 0 : b == 5 ? 1 : b == 6 ? 2 : b == 7 ? 0 : b == 8 ? 1 : 2);
}
__host__ __device__ constexpr int sup_hi(int b) {
    return b < 4 ? b : (b == 4 ? 1 : b == 5 ? 2 : b == 6 ? 0 : 3);
}

// ------------------------------------------------------------ geometry

__device__ __forceinline__ bool load_vertices(const int32_t *__restrict__ t, int64_t ne, int64_t e, int64_t npts,
                                              int32_t v[4]) {
    v[0] = t[e];
    v[1] = t[ne + e];
    v[2] = t[2 * ne + e];
    v[3] = t[3 * ne + e];
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 4; ++k) ok = ok && v[k] >= 0 && v[k] < npts;
    if (!ok) v[0] = v[1] = v[2] = v[3] = 0;
    return ok;
}

__device__ __forceinline__ double load_coef(const double *__restrict__ coef, int coef_kind, int64_t ne, int64_t e,
                                            int k) {
    // coef_kind 1: (E,3,3) row-major; 2: component-first (3,3,E)
    return coef_kind == 1 ? coef[e * 9 + k] : coef[(int64_t)k * ne + e];
}

__global__ void k_elem_fp64(int64_t ne, const double *__restrict__ p, int64_t npts, const int32_t *__restrict__ t,
                            int coef_kind, const double *__restrict__ coef, double *__restrict__ G) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    int32_t v[4];
    const bool ok = load_vertices(t, ne, e, npts, v);
    double J[9];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const double x0 = p[i * npts + v[0]];
#pragma unroll
        for (int r = 0; r < 3; ++r) J[i * 3 + r] = p[i * npts + v[r + 1]] - x0;
    }
    double b[4][3];
    b[1][0] = J[4] * J[8] - J[5] * J[7];
    b[1][1] = J[2] * J[7] - J[1] * J[8];
    b[1][2] = J[1] * J[5] - J[2] * J[4];
    b[2][0] = J[5] * J[6] - J[3] * J[8];
    b[2][1] = J[0] * J[8] - J[2] * J[6];
    b[2][2] = J[2] * J[3] - J[0] * J[5];
    b[3][0] = J[3] * J[7] - J[4] * J[6];
    b[3][1] = J[1] * J[6] - J[0] * J[7];
    b[3][2] = J[0] * J[4] - J[1] * J[3];
    const double det = J[0] * b[1][0] + J[1] * b[2][0] + J[2] * b[3][0];
#pragma unroll
    for (int i = 0; i < 3; ++i) b[0][i] = -(b[1][i] + b[2][i] + b[3][i]);
    const double inv = ok ? 1.0 / fabs(det) : __longlong_as_double(0x7ff8000000000000LL);
    double *g = G + e * 16;
    if (coef_kind == 0) {
        const double sc = (coef ? coef[e] : 1.0) * inv;
#pragma unroll
        for (int k = 0; k < 4; ++k)
#pragma unroll
            for (int l = k; l < 4; ++l) {
                const double val = sc * (b[k][0] * b[l][0] + b[k][1] * b[l][1] + b[k][2] * b[l][2]);
                g[k * 4 + l] = val;
                g[l * 4 + k] = val;
            }
    } else {
        double A[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) A[k] = load_coef(coef, coef_kind, ne, e, k);
        double Ab[4][3];
#pragma unroll
        for (int l = 0; l < 4; ++l)
#pragma unroll
            for (int i = 0; i < 3; ++i) Ab[l][i] = A[i * 3] * b[l][0] + A[i * 3 + 1] * b[l][1] + A[i * 3 + 2] * b[l][2];
#pragma unroll
        for (int k = 0; k < 4; ++k)
#pragma unroll
            for (int l = 0; l < 4; ++l)
                g[k * 4 + l] = inv * (b[k][0] * Ab[l][0] + b[k][1] * Ab[l][1] + b[k][2] * Ab[l][2]);
    }
}

__device__ __forceinline__ bool df_in_range(df64 x) {
    const float a = fabsf(x.hi);
    return a == 0.f || (a > 1e-30f && a < 1e30f);
}

// Scale exponent s: vertex coordinates times 2^-s are at most 1 in magnitude.
__global__ void k_scale(const double *__restrict__ p, int64_t n, int *__restrict__ s_out) {
    __shared__ int smax;
    if (threadIdx.x == 0) smax = INT_MIN;
    __syncthreads();
    int m = INT_MIN;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double a = fabs(p[i]);
        if (a > 0.0) m = max(m, ilogb(a) + 1);
    }
    atomicMax(&smax, m);
    __syncthreads();
    if (threadIdx.x == 0) atomicMax(s_out, smax);
}

// Element pass in double-float.  G (scaled by 2^-s) as 16 df64.
__global__ void k_elem_df64(int64_t ne, const double *__restrict__ p, int64_t npts, const int32_t *__restrict__ t,
                            int coef_kind, const double *__restrict__ coef, const int *__restrict__ s_ptr,
                            df64 *__restrict__ G, int *__restrict__ range_flag) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int s = *s_ptr;
    int32_t v[4];
    bool ok = load_vertices(t, ne, e, npts, v);
    df64 J[9];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const double x0 = p[i * npts + v[0]];
#pragma unroll
        for (int r = 0; r < 3; ++r) J[i * 3 + r] = df_from_double(p[i * npts + v[r + 1]] - x0, -s, ok);
    }
    df64 b[4][3];
#define SKG_CROSS(a, bb, c, d) df_sub(df_mul(J[a], J[bb]), df_mul(J[c], J[d]))
    b[1][0] = SKG_CROSS(4, 8, 5, 7);
    b[1][1] = SKG_CROSS(2, 7, 1, 8);
    b[1][2] = SKG_CROSS(1, 5, 2, 4);
    b[2][0] = SKG_CROSS(5, 6, 3, 8);
    b[2][1] = SKG_CROSS(0, 8, 2, 6);
    b[2][2] = SKG_CROSS(2, 3, 0, 5);
    b[3][0] = SKG_CROSS(3, 7, 4, 6);
    b[3][1] = SKG_CROSS(1, 6, 0, 7);
    b[3][2] = SKG_CROSS(0, 4, 1, 3);
#undef SKG_CROSS
    df64 det = df_add(df_add(df_mul(J[0], b[1][0]), df_mul(J[1], b[2][0])), df_mul(J[2], b[3][0]));
#pragma unroll
    for (int i = 0; i < 3; ++i) b[0][i] = df_neg(df_add(df_add(b[1][i], b[2][i]), b[3][i]));
    if (det.hi < 0.f) det = df_neg(det);
    ok = ok && det.hi > 1e-30f;
    const df64 inv = df_recip(det);
    df64 *g = G + e * 16;
    if (coef_kind == 0) {
        df64 sc = inv;
        if (coef) sc = df_mul(sc, df_from_double(coef[e], 0, ok));
#pragma unroll
        for (int k = 0; k < 4; ++k)
#pragma unroll
            for (int l = k; l < 4; ++l) {
                df64 d = df_add(df_add(df_mul(b[k][0], b[l][0]), df_mul(b[k][1], b[l][1])), df_mul(b[k][2], b[l][2]));
                d = df_mul(sc, d);
                ok = ok && df_in_range(d);
                g[k * 4 + l] = d;
                g[l * 4 + k] = d;
            }
    } else {
        df64 A[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) A[k] = df_from_double(load_coef(coef, coef_kind, ne, e, k), 0, ok);
        df64 Ab[4][3];
#pragma unroll
        for (int l = 0; l < 4; ++l)
#pragma unroll
            for (int i = 0; i < 3; ++i)
                Ab[l][i] = df_add(df_add(df_mul(A[i * 3], b[l][0]), df_mul(A[i * 3 + 1], b[l][1])),
                                  df_mul(A[i * 3 + 2], b[l][2]));
#pragma unroll
        for (int k = 0; k < 4; ++k)
#pragma unroll
            for (int l = 0; l < 4; ++l) {
                df64 d = df_add(df_add(df_mul(b[k][0], Ab[l][0]), df_mul(b[k][1], Ab[l][1])), df_mul(b[k][2], Ab[l][2]));
                d = df_mul(inv, d);
                ok = ok && df_in_range(d);
                g[k * 4 + l] = d;
            }
    }
    if (!ok) atomicExch(range_flag, 1);
}

// ------------------------------------------------------------ row pass

enum { MODE_FP64 = 0, MODE_SPLIT = 1, MODE_DF64 = 2 };

// Row pass over one row block.  Templated on the element size N (4 or 10)
// and the precision mode.  Shared memory: kBlockSlots accumulators (8 bytes
// each: double, or a df64 pair) + the T table + the support table.
template <int N, int MODE>
__global__ void __launch_bounds__(kBlockRows) k_rows_block(
    const int32_t *__restrict__ blk_row0, const int32_t *__restrict__ indptr, const int32_t *__restrict__ inc_ptr,
    const int4 *__restrict__ rec, const void *__restrict__ Gv, const double *__restrict__ Tg, Support sp,
    const int *__restrict__ s_ptr, double *__restrict__ values) {
    extern __shared__ __align__(16) unsigned char smem[];
    double *acc_d = reinterpret_cast<double *>(smem);
    df64 *acc_f = reinterpret_cast<df64 *>(smem);
    double *Td = reinterpret_cast<double *>(smem + kBlockSlots * 8);
    df64 *Tf = reinterpret_cast<df64 *>(smem + kBlockSlots * 8 + N * N * 4 * 8);
    int *sup = reinterpret_cast<int *>(smem + kBlockSlots * 8 + N * N * 4 * 16);

    const int32_t r0 = blk_row0[blockIdx.x], r1 = blk_row0[blockIdx.x + 1];
    const int32_t s0 = indptr[r0], s1 = indptr[r1];
    const int nslots = s1 - s0;
    for (int i = threadIdx.x; i < N * N * 4; i += blockDim.x) {
        const double tv = Tg[i];
        Td[i] = tv;
        const float h = (float)tv;
        Tf[i] = df64{h, (float)(tv - (double)h)};
    }
    if (threadIdx.x < N) {
        sup[2 * threadIdx.x] = sp.sup[threadIdx.x][0];
        sup[2 * threadIdx.x + 1] = sp.sup[threadIdx.x][1];
    }
    for (int i = threadIdx.x; i < nslots; i += blockDim.x) {
        if (MODE == MODE_FP64) acc_d[i] = 0.0;
        else acc_f[i] = df64{0.f, 0.f};
    }
    __syncthreads();

    const int32_t r = r0 + (int32_t)threadIdx.x;
    if (r < r1) {
        const int base = indptr[r] - s0;
        const int32_t it1 = inc_ptr[r + 1];
        for (int32_t it = inc_ptr[r]; it < it1; ++it) {
            const int4 rc = rec[it];
            const int32_t item = rc.x;
            const int32_t e = item / N;
            const int a = item - e * N;
            const unsigned ow[3] = {(unsigned)rc.y, (unsigned)rc.z, (unsigned)rc.w};
            const int ka0 = a < 4 ? a : sup[2 * a], ka1 = a < 4 ? a : sup[2 * a + 1];
            const bool edge_a = ka1 != ka0;
            if (MODE == MODE_FP64) {
                const double *g = reinterpret_cast<const double *>(Gv) + (int64_t)e * 16;
                double g0[4], g1[4];
#pragma unroll
                for (int l = 0; l < 4; ++l) {
                    g0[l] = g[ka0 * 4 + l];
                    g1[l] = edge_a ? g[ka1 * 4 + l] : 0.0;
                }
#pragma unroll
                for (int bb = 0; bb < N; ++bb) {
                    const int kb0 = sup_lo(bb), kb1 = sup_hi(bb);
                    const double *T = Td + (a * N + bb) * 4;
                    double val = g0[kb0] * T[0];
                    if (kb1 != kb0) val += g0[kb1] * T[1];
                    if (edge_a) {
                        val += g1[kb0] * T[2];
                        if (kb1 != kb0) val += g1[kb1] * T[3];
                    }
                    const int off = base + (int)((ow[bb >> 2] >> (8 * (bb & 3))) & 0xffu);
                    acc_d[off] += val;
                }
            } else {
                const df64 *g = reinterpret_cast<const df64 *>(Gv) + (int64_t)e * 16;
                df64 g0[4], g1[4];
#pragma unroll
                for (int l = 0; l < 4; ++l) {
                    g0[l] = g[ka0 * 4 + l];
                    g1[l] = edge_a ? g[ka1 * 4 + l] : df64{0.f, 0.f};
                }
#pragma unroll
                for (int bb = 0; bb < N; ++bb) {
                    const int kb0 = sup_lo(bb), kb1 = sup_hi(bb);
                    const df64 *T = Tf + (a * N + bb) * 4;
                    const bool edge_b = kb1 != kb0;
                    df64 val;
                    if (MODE == MODE_DF64) {
                        val = df_mul(g0[kb0], T[0]);
                        if (edge_b) val = df_add(val, df_mul(g0[kb1], T[1]));
                        if (edge_a) {
                            val = df_add(val, df_mul(g1[kb0], T[2]));
                            if (edge_b) val = df_add(val, df_mul(g1[kb1], T[3]));
                        }
                    } else {
                        // split products hi*hi (exact via FMA) + hi*lo + lo*hi, FP32 accumulation
                        float hsum = 0.f, corr = 0.f;
                        const df64 xs[4] = {g0[kb0], g0[kb1], g1[kb0], g1[kb1]};
                        const bool use[4] = {true, edge_b, edge_a, edge_a && edge_b};
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            if (!use[q]) continue;
                            const df64 x = xs[q], y = T[q];
                            const float ph = x.hi * y.hi;
                            corr += fmaf(x.hi, y.hi, -ph) + fmaf(x.hi, y.lo, x.lo * y.hi);
                            hsum += ph;
                        }
                        val = fast_two_sum(hsum, corr);
                    }
                    const int off = base + (int)((ow[bb >> 2] >> (8 * (bb & 3))) & 0xffu);
                    acc_f[off] = df_add(acc_f[off], val);
                }
            }
        }
    }
    __syncthreads();
    if (MODE == MODE_FP64) {
        for (int i = threadIdx.x; i < nslots; i += blockDim.x) values[s0 + i] = acc_d[i];
    } else {
        const int s = *s_ptr;
        for (int i = threadIdx.x; i < nslots; i += blockDim.x) values[s0 + i] = df_to_double(acc_f[i], s);
    }
}

// Fallback row pass (patterns without row blocks): thread per row, global
// accumulation, FP64.
template <int N>
__global__ void k_rows_global(int64_t n_rows, const int32_t *__restrict__ indptr, const int32_t *__restrict__ indices,
                              const int32_t *__restrict__ inc_ptr, const int32_t *__restrict__ inc,
                              const int32_t *__restrict__ dofs, const double *__restrict__ G,
                              const double *__restrict__ Tg, Support sp, double *__restrict__ values) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rows) return;
    const int32_t rb = indptr[r], rn = indptr[r + 1] - rb;
    for (int k = 0; k < rn; ++k) values[rb + k] = 0.;
    const int32_t *cols = indices + rb;
    for (int32_t it = inc_ptr[r]; it < inc_ptr[r + 1]; ++it) {
        const int32_t item = inc[it];
        const int64_t e = item / N;
        const int a = item - (int)(e * N);
        const double *g = G + e * 16;
        const int ka0 = sp.sup[a][0], ka1 = sp.sup[a][1];
        for (int bb = 0; bb < N; ++bb) {
            const int kb0 = sp.sup[bb][0], kb1 = sp.sup[bb][1];
            const double *T = Tg + (a * N + bb) * 4;
            double val = g[ka0 * 4 + kb0] * T[0];
            if (kb1 != kb0) val += g[ka0 * 4 + kb1] * T[1];
            if (ka1 != ka0) {
                val += g[ka1 * 4 + kb0] * T[2];
                if (kb1 != kb0) val += g[ka1 * 4 + kb1] * T[3];
            }
            const int32_t col = dofs[e * N + bb];
            const int pos = lower_bound_i32(cols, rn, col);
            if (pos < rn && cols[pos] == col) values[rb + pos] += val;
        }
    }
}

// Host: T^{kl}_{ab} from the quadrature rule, compacted to the supports.
void affine_table(int nodes, int nq, const double *X, const double *W, std::vector<double> &T, Support &sp) {
    static const int edges[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
    for (int a = 0; a < 10; ++a) sp.sup[a][0] = sp.sup[a][1] = 0;
    for (int a = 0; a < nodes; ++a) {
        if (a < 4) { sp.sup[a][0] = a; sp.sup[a][1] = a; }
        else { sp.sup[a][0] = edges[a - 4][0]; sp.sup[a][1] = edges[a - 4][1]; }
    }
    auto coeff = [&](int a, int slot, int q) -> double {
        const double x = X[q], y = X[nq + q], z = X[2 * nq + q];
        const double lam[4] = {1.0 - x - y - z, x, y, z};
        if (nodes == 4) return slot == 0 ? 1.0 : 0.0;
        if (a < 4) return slot == 0 ? 4.0 * lam[a] - 1.0 : 0.0;
        const int i = edges[a - 4][0], j = edges[a - 4][1];
        return slot == 0 ? 4.0 * lam[j] : 4.0 * lam[i];
    };
    T.assign((size_t)nodes * nodes * 4, 0.0);
    for (int a = 0; a < nodes; ++a)
        for (int b = 0; b < nodes; ++b)
            for (int u = 0; u < 2; ++u)
                for (int v = 0; v < 2; ++v) {
                    if (u == 1 && sp.sup[a][1] == sp.sup[a][0]) continue;
                    if (v == 1 && sp.sup[b][1] == sp.sup[b][0]) continue;
                    double acc = 0.0;
                    for (int q = 0; q < nq; ++q) acc += W[q] * coeff(a, u, q) * coeff(b, v, q);
                    T[((size_t)(a * nodes + b)) * 4 + u * 2 + v] = acc;
                }
}

template <int N, int MODE>
void launch_rows_block(const skg_pattern *pat, const void *G, const double *Tg, const Support &sp, const int *s_ptr,
                       double *values, cudaStream_t s) {
    const size_t smem = (size_t)kBlockSlots * 8 + (size_t)N * N * 4 * 16 + 2 * N * sizeof(int);
    static bool configured = false;  // per instantiation; attribute set once per process
    if (!configured) {
        SKG_CUDA(cudaFuncSetAttribute(k_rows_block<N, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        configured = true;
    }
    k_rows_block<N, MODE><<<pat->n_blocks, kBlockRows, smem, s>>>(pat->blk_row0.get(), pat->indptr.get(),
                                                                  pat->inc_ptr.get(), pat->rec.get(), G, Tg, sp, s_ptr,
                                                                  values);
    SKG_LAUNCH_CHECK("rows_block");
}

}  // namespace

// Shared by the C ABI entry points below.
void affine_assemble(const skg_pattern *pat, const double *d_p, int64_t npts, const int32_t *d_t, int32_t nodes,
                     int64_t ne, int32_t nq, const double *h_X, const double *h_W, int32_t coef_kind,
                     const double *d_coef, int32_t precision, double *d_values, cudaStream_t s, cudaEvent_t *ev) {
    require(pat != nullptr, "pattern is NULL");
    require(nodes == 4 || nodes == 10, "affine assembly supports P1 (4) and P2 (10) tetrahedra");
    require(ne == pat->n_elements && pat->row_local == nodes && pat->col_local == nodes,
            "mesh does not match the pattern");
    require(coef_kind == 0 || ((coef_kind == 1 || coef_kind == 2) && d_coef), "invalid coefficient kind");
    require(precision == SKG_FP64 || precision == SKG_SPLIT_FP32 || precision == SKG_FP64_EMULATED,
            "invalid precision");
    require(nq > 0 && h_X && h_W, "quadrature rule is empty");
    require(d_p && d_t, "mesh arrays are NULL");
    std::vector<double> T;
    Support sp{};
    affine_table(nodes, nq, h_X, h_W, T, sp);
    DevBuf<double> Tg(T.size(), s);
    SKG_CUDA(cudaMemcpyAsync(Tg.get(), T.data(), T.size() * 8, cudaMemcpyHostToDevice, s));
    DevBuf<double> G((size_t)ne * 16, s);  // 16 doubles or 16 df64 pairs per element
    const bool blocked = pat->n_blocks > 0;
    int mode = precision == SKG_FP64 ? MODE_FP64 : precision == SKG_SPLIT_FP32 ? MODE_SPLIT : MODE_DF64;
    if (!blocked) mode = MODE_FP64;
    DevBuf<int> misc(2, s);  // [0] scale exponent, [1] range flag
    if (mode != MODE_FP64) {
        const int init[2] = {INT_MIN, 0};
        SKG_CUDA(cudaMemcpyAsync(misc.get(), init, sizeof(init), cudaMemcpyHostToDevice, s));
        k_scale<<<64, 256, 0, s>>>(d_p, 3 * npts, misc.get());
        SKG_LAUNCH_CHECK("scale");
        if (ev) SKG_CUDA(cudaEventRecord(ev[0], s));
        if (ne) {
            k_elem_df64<<<grid_for(ne, 128), 128, 0, s>>>(ne, d_p, npts, d_t, coef_kind, d_coef, misc.get(),
                                                         reinterpret_cast<df64 *>(G.get()), misc.get() + 1);
            SKG_LAUNCH_CHECK("elem_df64");
        }
        int h_misc[2];
        SKG_CUDA(cudaMemcpyAsync(h_misc, misc.get(), sizeof(h_misc), cudaMemcpyDeviceToHost, s));
        SKG_CUDA(cudaStreamSynchronize(s));
        if (h_misc[1] != 0 || h_misc[0] == INT_MIN) mode = MODE_FP64;  // out of FP32 range: FP64 instead
    }
    if (mode == MODE_FP64) {
        if (ev) SKG_CUDA(cudaEventRecord(ev[0], s));
        if (ne) {
            k_elem_fp64<<<grid_for(ne, 128), 128, 0, s>>>(ne, d_p, npts, d_t, coef_kind, d_coef, G.get());
            SKG_LAUNCH_CHECK("elem_fp64");
        }
    }
    if (ev) SKG_CUDA(cudaEventRecord(ev[1], s));
    if (!blocked) {
        const unsigned grid = grid_for(pat->n_rows, 128);
        if (nodes == 4)
            k_rows_global<4><<<grid, 128, 0, s>>>(pat->n_rows, pat->indptr.get(), pat->indices.get(),
                                                  pat->inc_ptr.get(), pat->inc.get(), pat->col_dofs.get(), G.get(),
                                                  Tg.get(), sp, d_values);
        else
            k_rows_global<10><<<grid, 128, 0, s>>>(pat->n_rows, pat->indptr.get(), pat->indices.get(),
                                                   pat->inc_ptr.get(), pat->inc.get(), pat->col_dofs.get(), G.get(),
                                                   Tg.get(), sp, d_values);
        SKG_LAUNCH_CHECK("rows_global");
    } else {
        const int *sp_ptr = misc.get();
#define SKG_ROWS(NN, MM) launch_rows_block<NN, MM>(pat, G.get(), Tg.get(), sp, sp_ptr, d_values, s)
        if (nodes == 4) {
            if (mode == MODE_FP64) SKG_ROWS(4, MODE_FP64);
            else if (mode == MODE_SPLIT) SKG_ROWS(4, MODE_SPLIT);
            else SKG_ROWS(4, MODE_DF64);
        } else {
            if (mode == MODE_FP64) SKG_ROWS(10, MODE_FP64);
            else if (mode == MODE_SPLIT) SKG_ROWS(10, MODE_SPLIT);
            else SKG_ROWS(10, MODE_DF64);
        }
#undef SKG_ROWS
    }
    if (ev) SKG_CUDA(cudaEventRecord(ev[2], s));
}

}  // namespace skg

using namespace skg;

extern "C" int skg_h1_assemble_affine(const skg_pattern *pat, const double *d_p, int64_t npts, const int32_t *d_t,
                                      int32_t nodes, int64_t ne, const int32_t *d_dofs, int32_t nq,
                                      const double *h_X, const double *h_W, int32_t coef_kind,
                                      const double *d_coef, int32_t precision, double *d_values, void *stream) {
    return guarded([&] {
        (void)d_dofs;
        affine_assemble(pat, d_p, npts, d_t, nodes, ne, nq, h_X, h_W, coef_kind, d_coef, precision, d_values,
                        as_stream(stream), nullptr);
    });
}

extern "C" int skg_h1_assemble_affine_profiled(const skg_pattern *pat, const double *d_p, int64_t npts,
                                               const int32_t *d_t, int32_t nodes, int64_t ne,
                                               const int32_t *d_dofs, int32_t nq, const double *h_X,
                                               const double *h_W, int32_t coef_kind, const double *d_coef,
                                               int32_t precision, double *d_values, float *h_kernel_ms,
                                               void *stream) {
    return guarded([&] {
        (void)d_dofs;
        require(h_kernel_ms != nullptr, "timing output is NULL");
        cudaStream_t s = as_stream(stream);
        cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
        try {
            for (auto &e : ev) SKG_CUDA(cudaEventCreate(&e));
            affine_assemble(pat, d_p, npts, d_t, nodes, ne, nq, h_X, h_W, coef_kind, d_coef, precision, d_values, s,
                            ev);
            SKG_CUDA(cudaEventSynchronize(ev[2]));
            SKG_CUDA(cudaEventElapsedTime(&h_kernel_ms[0], ev[0], ev[1]));
            SKG_CUDA(cudaEventElapsedTime(&h_kernel_ms[1], ev[1], ev[2]));
        } catch (...) {
            for (auto &e : ev)
                if (e) cudaEventDestroy(e);
            throw;
        }
        for (auto &e : ev) cudaEventDestroy(e);
    });
}
