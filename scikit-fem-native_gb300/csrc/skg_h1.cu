// Nodal H1 (P1/P2 tetrahedra, scalar or vector) bilinear assembly.
//
// Two paths behind the C ABI:
//
// * tabulated (reference-compatible, any element/rule/coefficient kind):
//     element matrices from per-point tabulated shapes and gradients
//     (the reference's assemble_element, cpp/src/assembly/
//     bilinear_form_assembler.cpp:79-105, and contract_cross_basis,
//     cpp/include/native_fem/cross_contraction.hpp:67-84), then the
//     row-owner gather below.
//
// * affine (the hot path): for affine tetrahedra the physical gradient of
//     every P1/P2 basis function is a linear combination of the four
//     barycentric gradients, grad N_a(x_q) = sum_k c^k_a(xi_q) grad lambda_k,
//     with c^k_a = delta_ka for P1, (4 lambda_a - 1) delta_ka for P2
//     vertices and 4 lambda_j / 4 lambda_i on the two end vertices of P2
//     edge (i, j) (python/skfemntv/basis.py:2224-2235).  Hence
//         K_ab = sum_{k,l} G_kl T^{kl}_ab,
//         G_kl = |det J| grad lambda_k . A grad lambda_l      (per element)
//         T^{kl}_ab = sum_q w_q c^k_a(xi_q) c^l_b(xi_q)       (per rule)
//     T is tabulated once on the host from the caller's quadrature rule, so
//     the result equals the reference's quadrature sum up to rounding; only
//     the (k, l) in the supports of a and b (one vertex for a P1 function
//     or a P2 vertex function, two for a P2 edge function) are nonzero.
//     Pass 1 computes G per element (one thread per element); pass 2 is the
//     row-owner gather that evaluates row a of K_e on the fly.
//
// Row-owner gather: one thread owns one CSR row, walks the row's incidence
// list (element, local row) in ascending element order and adds the
// element-matrix row into the row's slots.  Every slot is written by one
// thread, contributions arrive in a fixed order, no atomics: the result is
// bitwise reproducible.
#include <vector>

#include "skg_common.cuh"

namespace skg {

namespace {

// ------------------------------------------------------------ tabulated

// Thread per (element, local row i = a*C + c): Ke[e, i, :].
__global__ void k_h1_local_tabulated(int64_t ne, int n, int C, int nq, const double *__restrict__ shape,
                                     const double *__restrict__ grad, const double *__restrict__ w,
                                     const double *__restrict__ value, const double *__restrict__ gradient,
                                     const double *__restrict__ symgrad, const double *__restrict__ divc,
                                     double *__restrict__ Ke) {
    const int L = n * C;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= ne * L) return;
    const int64_t e = tid / L;
    const int i = (int)(tid % L);
    const int a = i / C, c = i % C;
    double *row = Ke + (e * L + i) * (int64_t)L;
    for (int k = 0; k < L; ++k) {
        const int b = k / C, d = k % C;
        double acc = 0.;
        for (int q = 0; q < nq; ++q) {
            const int64_t eq = e * nq + q;
            const double *ga = grad + (eq * n + a) * 3;
            const double *gb = grad + (eq * n + b) * 3;
            const double gg = ga[0] * gb[0] + ga[1] * gb[1] + ga[2] * gb[2];
            double entry = 0.;
            if (c == d) {
                if (value) entry += value[eq] * shape[eq * n + a] * shape[eq * n + b];
                if (gradient) entry += gradient[eq] * gg;
            }
            if (symgrad) entry += 0.5 * symgrad[eq] * (ga[d] * gb[c] + (c == d ? gg : 0.));
            if (divc) entry += divc[eq] * ga[c] * gb[d];
            acc += entry * w[eq];
        }
        row[k] = acc;
    }
}

// Thread per (element, local row i = a*C + r): tensor coefficient on gradients.
__global__ void k_h1_local_tensor(int64_t ne, int n, int C, int nq, const double *__restrict__ grad,
                                  const double *__restrict__ w, const double *__restrict__ coef,
                                  double *__restrict__ Ke) {
    const int L = n * C;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= ne * L) return;
    const int64_t e = tid / L;
    const int i = (int)(tid % L);
    const int a = i / C, r = i % C;
    double *row = Ke + (e * L + i) * (int64_t)L;
    for (int k = 0; k < L; ++k) {
        const int b = k / C, cc = k % C;
        double acc = 0.;
        for (int q = 0; q < nq; ++q) {
            const int64_t eq = e * nq + q;
            const double *ga = grad + (eq * n + a) * 3;
            const double *gb = grad + (eq * n + b) * 3;
            const double *Cq = coef + (((eq * C + r) * 3) * C + cc) * 3;  // [i][c][j] with i stride C*3
            double s = 0.;
            for (int ii = 0; ii < 3; ++ii)
                for (int jj = 0; jj < 3; ++jj) s += ga[ii] * Cq[ii * C * 3 + jj] * gb[jj];
            acc += w[eq] * s;
        }
        row[k] = acc;
    }
}

// Row-owner gather of element matrices Ke (E, Lr, Lc) into CSR values.
__global__ void k_gather_rows(int64_t n_rows, const int32_t *__restrict__ indptr,
                              const int32_t *__restrict__ indices, const int32_t *__restrict__ inc_ptr,
                              const int32_t *__restrict__ inc, const int32_t *__restrict__ col_dofs,
                              int Lr, int Lc, const double *__restrict__ Ke, double *__restrict__ values) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rows) return;
    const int32_t rb = indptr[r], rn = indptr[r + 1] - rb;
    for (int k = 0; k < rn; ++k) values[rb + k] = 0.;
    const int32_t *cols = indices + rb;
    for (int32_t t = inc_ptr[r]; t < inc_ptr[r + 1]; ++t) {
        const int32_t item = inc[t];
        const int64_t e = item / Lr;
        const double *src = Ke + (int64_t)item * Lc;
        const int32_t *cd = col_dofs + e * Lc;
        for (int k = 0; k < Lc; ++k) {
            const int32_t col = cd[k];
            const int pos = lower_bound_i32(cols, rn, col);
            if (pos < rn && cols[pos] == col) values[rb + pos] += src[k];
        }
    }
}

// ------------------------------------------------------------ affine

// Per element: G (4x4, row-major) = coef * |det J| grad lambda_k . A grad lambda_l
// with grad lambda_k = b_k / det J (b_k rows of adj J for k = 1..3,
// b_0 = -(b_1 + b_2 + b_3)), i.e. G_kl = coef * b_k . A b_l / |det J|.
// Also writes det J (the reference validates geometry in Basis setup).
__device__ __forceinline__ void element_jacobian(const double *__restrict__ p, int64_t npts,
                                                 const int32_t *__restrict__ t, int64_t ne, int64_t e,
                                                 double J[9]) {
    int32_t v0 = t[e], v1 = t[ne + e], v2 = t[2 * ne + e], v3 = t[3 * ne + e];
    // out-of-range vertex ids never reach memory: the element becomes NaN
    const bool ok = v0 >= 0 && v0 < npts && v1 >= 0 && v1 < npts && v2 >= 0 && v2 < npts && v3 >= 0 && v3 < npts;
    if (!ok) v0 = v1 = v2 = v3 = 0;
    const int32_t v[3] = {v1, v2, v3};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const double x0 = p[i * npts + v0];
#pragma unroll
        for (int r = 0; r < 3; ++r) J[i * 3 + r] = ok ? p[i * npts + v[r]] - x0 : __longlong_as_double(0x7ff8000000000000LL);
    }
}

__device__ __forceinline__ void adjugate_rows(const double J[9], double b[4][3], double &det) {
    // b[k+1] = row k of adj(J) (so J^{-1} = adj / det), b[0] = -(b1+b2+b3)
    b[1][0] = J[4] * J[8] - J[5] * J[7];
    b[1][1] = J[2] * J[7] - J[1] * J[8];
    b[1][2] = J[1] * J[5] - J[2] * J[4];
    b[2][0] = J[5] * J[6] - J[3] * J[8];
    b[2][1] = J[0] * J[8] - J[2] * J[6];
    b[2][2] = J[2] * J[3] - J[0] * J[5];
    b[3][0] = J[3] * J[7] - J[4] * J[6];
    b[3][1] = J[1] * J[6] - J[0] * J[7];
    b[3][2] = J[0] * J[4] - J[1] * J[3];
    det = J[0] * b[1][0] + J[1] * b[2][0] + J[2] * b[3][0];
#pragma unroll
    for (int i = 0; i < 3; ++i) b[0][i] = -(b[1][i] + b[2][i] + b[3][i]);
}

__global__ void k_affine_element_G(int64_t ne, const double *__restrict__ p, int64_t npts,
                                   const int32_t *__restrict__ t, int coef_kind,
                                   const double *__restrict__ coef, double *__restrict__ G,
                                   double *__restrict__ det_out) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    double J[9], b[4][3], det;
    element_jacobian(p, npts, t, ne, e, J);
    adjugate_rows(J, b, det);
    const double inv = 1.0 / fabs(det);
    double *g = G + e * 16;
    if (coef_kind == 0) {
        const double s = (coef ? coef[e] : 1.0) * inv;
#pragma unroll
        for (int k = 0; k < 4; ++k)
#pragma unroll
            for (int l = k; l < 4; ++l) {
                const double v = s * (b[k][0] * b[l][0] + b[k][1] * b[l][1] + b[k][2] * b[l][2]);
                g[k * 4 + l] = v;
                g[l * 4 + k] = v;
            }
    } else {
        // coef_kind 1: (E, 3, 3) row-major per element; 2: component-first (3, 3, E)
        double A[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) A[k] = coef_kind == 1 ? coef[e * 9 + k] : coef[(int64_t)k * ne + e];
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
    if (det_out) det_out[e] = det;
}

// Support of the basis functions on the barycentric gradients:
// sup[a] = (k0, k1) (k1 = k0 for single-vertex support).
struct AffineTable {
    int n;
    int sup[10][2];
};

template <int N, bool SPLIT>
__global__ void k_affine_rows(int64_t n_rows, const int32_t *__restrict__ indptr,
                              const int32_t *__restrict__ indices, const int32_t *__restrict__ inc_ptr,
                              const int32_t *__restrict__ inc, const int32_t *__restrict__ dofs,
                              const double *__restrict__ G, const double *__restrict__ Tg, AffineTable tab,
                              double *__restrict__ values) {
    // T[a][b][s][t] staged in shared memory (FP64 and its FP32 hi/lo split)
    __shared__ double Ts[N * N * 4];
    __shared__ float Th[N * N * 4], Tl[N * N * 4];
    __shared__ int sup[N][2];
    if (threadIdx.x < N) {
        sup[threadIdx.x][0] = tab.sup[threadIdx.x][0];
        sup[threadIdx.x][1] = tab.sup[threadIdx.x][1];
    }
    for (int i = threadIdx.x; i < N * N * 4; i += blockDim.x) {
        const double v = Tg[i];
        Ts[i] = v;
        const float h = (float)v;
        Th[i] = h;
        Tl[i] = (float)(v - (double)h);
    }
    __syncthreads();
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
        const int ka0 = sup[a][0], ka1 = sup[a][1];
        const int32_t *cd = dofs + e * N;
#pragma unroll
        for (int bb = 0; bb < N; ++bb) {
            const int kb0 = sup[bb][0], kb1 = sup[bb][1];
            const int tb = ((a * N + bb) * 4);
            double val;
            if (!SPLIT) {
                val = g[ka0 * 4 + kb0] * Ts[tb + 0];
                if (kb1 != kb0) val += g[ka0 * 4 + kb1] * Ts[tb + 1];
                if (ka1 != ka0) {
                    val += g[ka1 * 4 + kb0] * Ts[tb + 2];
                    if (kb1 != kb0) val += g[ka1 * 4 + kb1] * Ts[tb + 3];
                }
            } else {
                // split-precision products: x = xh + xl, y = yh + yl,
                // x*y ~ xh*yh + (xh*yl + xl*yh), FP32 accumulation
                float acc = 0.f, corr = 0.f;
                const int idx[4] = {ka0 * 4 + kb0, ka0 * 4 + kb1, ka1 * 4 + kb0, ka1 * 4 + kb1};
                const bool use[4] = {true, kb1 != kb0, ka1 != ka0, ka1 != ka0 && kb1 != kb0};
#pragma unroll
                for (int s = 0; s < 4; ++s) {
                    if (!use[s]) continue;
                    const double x = g[idx[s]];
                    const float xh = (float)x, xl = (float)(x - (double)xh);
                    const float yh = Th[tb + s], yl = Tl[tb + s];
                    const float ph = xh * yh;
                    const float pe = fmaf(xh, yh, -ph);  // exact error of the hi product
                    acc += ph;
                    corr += pe + fmaf(xh, yl, xl * yh);
                }
                val = (double)acc + (double)corr;
            }
            const int32_t col = cd[bb];
            const int pos = lower_bound_i32(cols, rn, col);
            if (pos < rn && cols[pos] == col) values[rb + pos] += val;
        }
    }
}

}  // namespace

// Fixed-order gather of element matrices (E, Lr, Lc) into the pattern's CSR values.
void gather_element_matrices(const skg_pattern *pat, const double *Ke, double *values, cudaStream_t s) {
    if (!pat->n_rows) return;
    k_gather_rows<<<grid_for(pat->n_rows, 128), 128, 0, s>>>(pat->n_rows, pat->indptr.get(), pat->indices.get(),
                                                             pat->inc_ptr.get(), pat->inc.get(), pat->col_dofs.get(),
                                                             pat->row_local, pat->col_local, Ke, values);
    SKG_LAUNCH_CHECK("gather_rows");
}

}  // namespace skg

using namespace skg;

// Host: T^{kl}_{ab} from the quadrature rule, compacted to the supports.
static void h1_affine_table(int nodes, int nq, const double *X, const double *W, std::vector<double> &T,
                          AffineTable &tab) {
    static const int edges[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
    tab.n = nodes;
    for (int a = 0; a < nodes; ++a) {
        if (a < 4) { tab.sup[a][0] = a; tab.sup[a][1] = a; }
        else { tab.sup[a][0] = edges[a - 4][0]; tab.sup[a][1] = edges[a - 4][1]; }
    }
    // coefficient c^{sup[a][s]}_a at point q
    auto coeff = [&](int a, int s, int q) -> double {
        const double x = X[0 * nq + q], y = X[1 * nq + q], z = X[2 * nq + q];
        const double lam[4] = {1.0 - x - y - z, x, y, z};
        if (nodes == 4) return s == 0 ? 1.0 : 0.0;
        if (a < 4) return s == 0 ? 4.0 * lam[a] - 1.0 : 0.0;
        const int i = edges[a - 4][0], j = edges[a - 4][1];
        return s == 0 ? 4.0 * lam[j] : 4.0 * lam[i];
    };
    T.assign((size_t)nodes * nodes * 4, 0.0);
    for (int a = 0; a < nodes; ++a)
        for (int b = 0; b < nodes; ++b)
            for (int s = 0; s < 2; ++s)
                for (int u = 0; u < 2; ++u) {
                    if (s == 1 && tab.sup[a][1] == tab.sup[a][0]) continue;
                    if (u == 1 && tab.sup[b][1] == tab.sup[b][0]) continue;
                    double acc = 0.0;
                    for (int q = 0; q < nq; ++q) acc += W[q] * coeff(a, s, q) * coeff(b, u, q);
                    T[((size_t)(a * nodes + b)) * 4 + s * 2 + u] = acc;
                }
}

extern "C" int skg_h1_assemble_tabulated(const skg_pattern *pat, const int32_t *d_dofs, int64_t ne,
                                         int32_t nodes, int32_t comp, int32_t nq, const double *d_shape,
                                         const double *d_grad, const double *d_w, const double *d_value,
                                         const double *d_gradient, const double *d_symgrad,
                                         const double *d_div, double *d_values, double *d_scratch,
                                         void *stream) {
    return guarded([&] {
        require(pat != nullptr, "pattern is NULL");
        require(d_value || d_gradient || d_symgrad || d_div, "at least one coefficient is required");
        const int L = nodes * comp;
        require(nodes > 0 && comp > 0 && nq > 0 && ne == pat->n_elements && L == pat->row_local &&
                    L == pat->col_local,
                "tabulated arrays do not match the pattern");
        require(d_grad && d_w && (!d_value || d_shape), "tabulated geometry arrays are NULL");
        (void)d_dofs;
        cudaStream_t s = as_stream(stream);
        DevBuf<double> tmp;
        double *Ke = d_scratch;
        if (!Ke) {
            tmp = DevBuf<double>((size_t)ne * L * L, s);
            Ke = tmp.get();
        }
        if (ne) {
            k_h1_local_tabulated<<<grid_for(ne * L, 128), 128, 0, s>>>(ne, nodes, comp, nq, d_shape, d_grad, d_w,
                                                                       d_value, d_gradient, d_symgrad, d_div, Ke);
            SKG_LAUNCH_CHECK("h1_local_tabulated");
        }
        k_gather_rows<<<grid_for(pat->n_rows, 128), 128, 0, s>>>(pat->n_rows, pat->indptr.get(), pat->indices.get(),
                                                                 pat->inc_ptr.get(), pat->inc.get(),
                                                                 pat->col_dofs.get(), L, L, Ke, d_values);
        SKG_LAUNCH_CHECK("gather_rows");
    });
}

extern "C" int skg_h1_assemble_tensor_tabulated(const skg_pattern *pat, const int32_t *d_dofs, int64_t ne,
                                                int32_t nodes, int32_t comp, int32_t nq, const double *d_grad,
                                                const double *d_w, const double *d_coef, double *d_values,
                                                double *d_scratch, void *stream) {
    return guarded([&] {
        require(pat != nullptr, "pattern is NULL");
        require(d_coef && d_grad && d_w, "tensor coefficient or geometry is NULL");
        const int L = nodes * comp;
        require(nodes > 0 && comp > 0 && nq > 0 && ne == pat->n_elements && L == pat->row_local &&
                    L == pat->col_local,
                "tabulated arrays do not match the pattern");
        (void)d_dofs;
        cudaStream_t s = as_stream(stream);
        DevBuf<double> tmp;
        double *Ke = d_scratch;
        if (!Ke) {
            tmp = DevBuf<double>((size_t)ne * L * L, s);
            Ke = tmp.get();
        }
        if (ne) {
            k_h1_local_tensor<<<grid_for(ne * L, 128), 128, 0, s>>>(ne, nodes, comp, nq, d_grad, d_w, d_coef, Ke);
            SKG_LAUNCH_CHECK("h1_local_tensor");
        }
        k_gather_rows<<<grid_for(pat->n_rows, 128), 128, 0, s>>>(pat->n_rows, pat->indptr.get(), pat->indices.get(),
                                                                 pat->inc_ptr.get(), pat->inc.get(),
                                                                 pat->col_dofs.get(), L, L, Ke, d_values);
        SKG_LAUNCH_CHECK("gather_rows");
    });
}

static void affine_impl(const skg_pattern *pat, const double *d_p, int64_t npts, const int32_t *d_t, int32_t nodes,
                        int64_t ne, const int32_t *d_dofs, int32_t nq, const double *h_X, const double *h_W,
                        int32_t coef_kind, const double *d_coef, int32_t precision, double *d_values,
                        cudaStream_t s, cudaEvent_t *ev) {
    require(pat != nullptr, "pattern is NULL");
    require(nodes == 4 || nodes == 10, "affine assembly supports P1 (4) and P2 (10) tetrahedra");
    require(ne == pat->n_elements && pat->row_local == nodes && pat->col_local == nodes,
            "mesh does not match the pattern");
    require(coef_kind == 0 || ((coef_kind == 1 || coef_kind == 2) && d_coef), "invalid coefficient kind");
    require(precision == SKG_FP64 || precision == SKG_SPLIT_FP32, "invalid precision");
    require(nq > 0 && h_X && h_W, "quadrature rule is empty");
    require(d_p && d_t && d_dofs, "mesh arrays are NULL");
    std::vector<double> T;
    AffineTable tab{};
    h1_affine_table(nodes, nq, h_X, h_W, T, tab);
    DevBuf<double> Tg(T.size(), s);
    SKG_CUDA(cudaMemcpyAsync(Tg.get(), T.data(), T.size() * 8, cudaMemcpyHostToDevice, s));
    DevBuf<double> G((size_t)ne * 16, s);
    if (ev) SKG_CUDA(cudaEventRecord(ev[0], s));
    if (ne) {
        k_affine_element_G<<<grid_for(ne, 128), 128, 0, s>>>(ne, d_p, npts, d_t, coef_kind, d_coef, G.get(),
                                                             nullptr);
        SKG_LAUNCH_CHECK("affine_element_G");
    }
    if (ev) SKG_CUDA(cudaEventRecord(ev[1], s));
    const unsigned grid = grid_for(pat->n_rows, 128);
#define SKG_AFFINE_ROWS(NN, SP)                                                                          \
    k_affine_rows<NN, SP><<<grid, 128, 0, s>>>(pat->n_rows, pat->indptr.get(), pat->indices.get(),      \
                                               pat->inc_ptr.get(), pat->inc.get(), pat->col_dofs.get(), \
                                               G.get(),                                                 \
                                               Tg.get(), tab, d_values)
    if (nodes == 4) {
        if (precision == SKG_FP64) SKG_AFFINE_ROWS(4, false); else SKG_AFFINE_ROWS(4, true);
    } else {
        if (precision == SKG_FP64) SKG_AFFINE_ROWS(10, false); else SKG_AFFINE_ROWS(10, true);
    }
#undef SKG_AFFINE_ROWS
    SKG_LAUNCH_CHECK("affine_rows");
    if (ev) SKG_CUDA(cudaEventRecord(ev[2], s));
}

extern "C" int skg_h1_assemble_affine(const skg_pattern *pat, const double *d_p, int64_t npts, const int32_t *d_t,
                                      int32_t nodes, int64_t ne, const int32_t *d_dofs, int32_t nq,
                                      const double *h_X, const double *h_W, int32_t coef_kind,
                                      const double *d_coef, int32_t precision, double *d_values, void *stream) {
    return guarded([&] {
        affine_impl(pat, d_p, npts, d_t, nodes, ne, d_dofs, nq, h_X, h_W, coef_kind, d_coef, precision, d_values,
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
        require(h_kernel_ms != nullptr, "timing output is NULL");
        cudaStream_t s = as_stream(stream);
        cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
        try {
            for (auto &e : ev) SKG_CUDA(cudaEventCreate(&e));
            affine_impl(pat, d_p, npts, d_t, nodes, ne, d_dofs, nq, h_X, h_W, coef_kind, d_coef, precision,
                        d_values, s, ev);
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
