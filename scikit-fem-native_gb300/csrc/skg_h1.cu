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
// * affine (the hot path) lives in skg_affine.cu.
//
// Row-owner gather: one thread owns one CSR row, walks the row's incidence
// list (element, local row) in ascending element order and adds the
// element-matrix row into the row's slots.  Every slot is written by one
// thread, contributions arrive in a fixed order, no atomics: the result is
// bitwise reproducible.
#include <vector>

#include "skg_common.cuh"
#include "skg_rows.cuh"

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

// Thread per element for small element matrices (P1 scalar / vector, P2
// scalar).  Every kind of the tabulated form gives a symmetric matrix when
// test and trial basis coincide: K_(a,c),(b,d) = K_(b,d),(a,c) for the value,
// gradient, symmetric-gradient and divergence terms alike.  So only the blocks
// b >= a are summed over the points (in registers, two FMAs per entry and
// point: sg a_d b_c + dv a_c b_d, one on c == d, the diagonal blocks from their
// upper half), each written with its transpose into the
// thread's element matrix in shared memory, and the block stores all matrices
// coalesced.  The kernel is FP64-pipe bound; this halves its FP64
// instructions against the full block loop.
template <int NN, int CC, int BLK>
__global__ void __launch_bounds__(BLK) k_h1_local_sym(int64_t ne, int nq, const double *__restrict__ shape,
                                                      const double *__restrict__ grad, const double *__restrict__ w,
                                                      const double *__restrict__ value,
                                                      const double *__restrict__ gradient,
                                                      const double *__restrict__ symgrad,
                                                      const double *__restrict__ divc, double *__restrict__ Ke) {
    constexpr int L = NN * CC, LL = L * L, LP = LL + 1;
    extern __shared__ double stage[];  // BLK x LP
    const int64_t e0 = (int64_t)blockIdx.x * BLK;
    const int64_t e = e0 + threadIdx.x;
    const int nvalid = (int)(ne - e0 < BLK ? ne - e0 : BLK);
    double *st = stage + threadIdx.x * LP;
    if (e < ne) {
#pragma unroll
        for (int a = 0; a < NN; ++a) {
            // acc: the sg / dv products (diagonal blocks: d >= c only); accd: the
            // terms on c == d (value, gradient and the trace part of sg), per block
            double acc[NN][CC][CC], accd[NN];
#pragma unroll
            for (int b = a; b < NN; ++b) {
                accd[b] = 0.0;
#pragma unroll
                for (int c = 0; c < CC; ++c)
#pragma unroll
                    for (int d = 0; d < CC; ++d) acc[b][c][d] = 0.0;
            }
            for (int q = 0; q < nq; ++q) {
                const int64_t eq = e * nq + q;
                const double wq = w[eq];
                const double sg = symgrad ? 0.5 * symgrad[eq] * wq : 0.0;
                const double dv = divc ? divc[eq] * wq : 0.0;
                const double dg = (gradient ? gradient[eq] * wq : 0.0) + sg;
                const double va = value ? value[eq] * wq * shape[eq * NN + a] : 0.0;
                const double *gq = grad + eq * (NN * 3);
                const double ag[3] = {gq[a * 3], gq[a * 3 + 1], gq[a * 3 + 2]};
                double sa[CC], da[CC], ta[CC];
#pragma unroll
                for (int c = 0; c < CC; ++c) {
                    sa[c] = sg * ag[c];
                    da[c] = dv * ag[c];
                    ta[c] = sa[c] + da[c];
                }
#pragma unroll
                for (int b = a; b < NN; ++b) {
                    const double bg[3] = {gq[b * 3], gq[b * 3 + 1], gq[b * 3 + 2]};
                    double diag = accd[b] + dg * (ag[0] * bg[0] + ag[1] * bg[1] + ag[2] * bg[2]);
                    if (value) diag += va * shape[eq * NN + b];
                    accd[b] = diag;
#pragma unroll
                    for (int c = 0; c < CC; ++c)
#pragma unroll
                        for (int d = 0; d < CC; ++d) {
                            if (b == a && d < c) continue;  // diagonal block: symmetric in (c, d)
                            if (c == d) {
                                acc[b][c][c] += ta[c] * bg[c];
                            } else {
                                double v = acc[b][c][d] + sa[d] * bg[c];
                                acc[b][c][d] = v + da[c] * bg[d];
                            }
                        }
                }
            }
#pragma unroll
            for (int b = a; b < NN; ++b)
#pragma unroll
                for (int c = 0; c < CC; ++c)
#pragma unroll
                    for (int d = 0; d < CC; ++d) {
                        if (b == a && d < c) continue;
                        const double v = c == d ? acc[b][c][c] + accd[b] : acc[b][c][d];
                        st[(a * CC + c) * L + b * CC + d] = v;
                        if (b != a || c != d) st[(b * CC + d) * L + a * CC + c] = v;
                    }
        }
    }
    __syncthreads();
    for (int x = threadIdx.x; x < nvalid * LL; x += BLK) {
        const int el = x / LL, k = x - el * LL;
        Ke[(e0 + el) * (int64_t)LL + k] = stage[el * LP + k];
    }
}

// Thread per element for the common element shapes (NN nodes, CC components):
// the element's rows are produced node by node (the CC rows of node a, L
// entries each), block (a, b) accumulated over the points in registers, and
// staged through shared memory so that the block writes whole row bands with
// coalesced stores.  Same entries as k_h1_local_tabulated (the point weight is
// folded into each term).
template <int NN, int CC, int BLK>
__global__ void __launch_bounds__(BLK) k_h1_local_tab(int64_t ne, int nq, const double *__restrict__ shape,
                                                      const double *__restrict__ grad, const double *__restrict__ w,
                                                      const double *__restrict__ value,
                                                      const double *__restrict__ gradient,
                                                      const double *__restrict__ symgrad,
                                                      const double *__restrict__ divc, double *__restrict__ Ke) {
    constexpr int L = NN * CC, R = CC * L;  // entries of node a's row band
    __shared__ double stage[BLK * (R + 1)];
    const int64_t e0 = (int64_t)blockIdx.x * BLK;
    const int64_t e = e0 + threadIdx.x;
    const bool valid = e < ne;
    const int nvalid = (int)(ne - e0 < BLK ? ne - e0 : BLK);
    double *st = stage + threadIdx.x * (R + 1);
#pragma unroll 1
    for (int a = 0; a < NN; ++a) {
        if (valid) {
#pragma unroll 1
            for (int b = 0; b < NN; ++b) {
                double blk[CC][CC];
#pragma unroll
                for (int c = 0; c < CC; ++c)
#pragma unroll
                    for (int d = 0; d < CC; ++d) blk[c][d] = 0.0;
                for (int q = 0; q < nq; ++q) {
                    const int64_t eq = e * nq + q;
                    const double *ga = grad + (eq * NN + a) * 3, *gb = grad + (eq * NN + b) * 3;
                    const double a0 = ga[0], a1 = ga[1], a2 = ga[2], b0 = gb[0], b1 = gb[1], b2 = gb[2];
                    const double ag[3] = {a0, a1, a2}, bg[3] = {b0, b1, b2};
                    const double gg = a0 * b0 + a1 * b1 + a2 * b2;
                    const double wq = w[eq];
                    double diag = 0.0;  // terms on c == d
                    if (value) diag += value[eq] * shape[eq * NN + a] * shape[eq * NN + b] * wq;
                    if (gradient) diag += gradient[eq] * gg * wq;
                    const double sg = symgrad ? 0.5 * symgrad[eq] * wq : 0.0;
                    const double dv = divc ? divc[eq] * wq : 0.0;
                    diag += sg * gg;
#pragma unroll
                    for (int c = 0; c < CC; ++c)
#pragma unroll
                        for (int d = 0; d < CC; ++d) {
                            double v = sg * ag[d] * bg[c] + dv * ag[c] * bg[d];
                            if (c == d) v += diag;
                            blk[c][d] += v;
                        }
                }
#pragma unroll
                for (int c = 0; c < CC; ++c)
#pragma unroll
                    for (int d = 0; d < CC; ++d) st[c * L + b * CC + d] = blk[c][d];
            }
        }
        __syncthreads();
        for (int x = threadIdx.x; x < nvalid * R; x += BLK) {
            const int el = x / R, k = x - el * R;
            Ke[(e0 + el) * (int64_t)(L * L) + (int64_t)a * R + k] = stage[el * (R + 1) + k];
        }
        __syncthreads();
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

// Test x trial local matrices with a full contraction tensor (cross bases):
// thread per (element, test row i = a*Ct + r):
//   K[(a,r),(b,c)] = sum_q dx sum_ii sum_jj R_a[ii] C[e,q,r,ii,c,jj] S_b[jj]
// R_a = shape value (Rd = 1) or gradient (Rd = 3) of test function a; S_b
// likewise for the trial function b.  C (E, Q, Ct, Rd, Cc, Sd) contiguous.
__global__ void k_cross_local(int64_t ne, int nq, int nt, int Ct, int Rd, const double *__restrict__ t_shape,
                              const double *__restrict__ t_grad, int nc, int Cc, int Sd,
                              const double *__restrict__ c_shape, const double *__restrict__ c_grad,
                              const double *__restrict__ dx, const double *__restrict__ coef,
                              double *__restrict__ Ke) {
    const int Lt = nt * Ct, Lc = nc * Cc;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= ne * Lt) return;
    const int64_t e = tid / Lt;
    const int i = (int)(tid % Lt);
    const int a = i / Ct, r = i % Ct;
    double *row = Ke + (e * Lt + i) * (int64_t)Lc;
    for (int k = 0; k < Lc; ++k) {
        const int b = k / Cc, c = k % Cc;
        double acc = 0.;
        for (int q = 0; q < nq; ++q) {
            const int64_t eq = e * nq + q;
            double R[3], S[3];
            if (Rd == 1) R[0] = t_shape[eq * nt + a];
            else for (int d = 0; d < 3; ++d) R[d] = t_grad[(eq * nt + a) * 3 + d];
            if (Sd == 1) S[0] = c_shape[eq * nc + b];
            else for (int d = 0; d < 3; ++d) S[d] = c_grad[(eq * nc + b) * 3 + d];
            const double *Cq = coef + ((eq * Ct + r) * Rd) * (int64_t)(Cc * Sd) + c * Sd;
            double s = 0.;
            for (int ii = 0; ii < Rd; ++ii)
                for (int jj = 0; jj < Sd; ++jj) s += R[ii] * Cq[ii * Cc * Sd + jj] * S[jj];
            acc += dx[eq] * s;
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

// Thread per DOF: out[r] = sum of the element vector entries incident on r,
// in element order (the incidence lists are sorted by element).
__global__ void k_gather_vector(int64_t n_rows, const int32_t *__restrict__ inc_ptr, const int32_t *__restrict__ inc,
                                const double *__restrict__ le, double *__restrict__ out) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rows) return;
    double acc = 0.0;
    for (int32_t it = inc_ptr[r]; it < inc_ptr[r + 1]; ++it) acc += le[inc[it]];
    out[r] = acc;
}

}  // namespace

// Fixed-order gather of element matrices (E, Lr, Lc) into the pattern's CSR values.
void gather_element_vectors(const skg_pattern *pat, const double *le, double *out, cudaStream_t s) {
    if (!pat->n_rows) return;
    k_gather_vector<<<grid_for(pat->n_rows, 128), 128, 0, s>>>(pat->n_rows, pat->inc_ptr.get(), pat->inc.get(), le,
                                                               out);
    SKG_LAUNCH_CHECK("gather_vector");
}

void gather_element_matrices(const skg_pattern *pat, const double *Ke, double *values, cudaStream_t s) {
    if (!pat->n_rows) return;
    if (pat->max_row_len > 0 && pat->row_local == pat->col_local) {
        // row groups: shared-memory slot sums, each value written once
        switch (pat->row_local) {
            case 4: add_element_rows<4>(pat, Ke, values, s); return;
            case 6: add_element_rows<6>(pat, Ke, values, s); return;
            case 10: add_element_rows<10>(pat, Ke, values, s); return;
            case 12: add_element_rows<12>(pat, Ke, values, s); return;
            default: break;
        }
    }
    k_gather_rows<<<grid_for(pat->n_rows, 128), 128, 0, s>>>(pat->n_rows, pat->indptr.get(), pat->indices.get(),
                                                             pat->inc_ptr.get(), pat->inc.get(), pat->col_dofs.get(),
                                                             pat->row_local, pat->col_local, Ke, values);
    SKG_LAUNCH_CHECK("gather_rows");
}

}  // namespace skg

using namespace skg;

extern "C" int skg_h1_assemble_tabulated(const skg_pattern *pat, const int32_t *d_dofs, int64_t ne,
                                         int32_t nodes, int32_t comp, int32_t nq, const double *d_shape,
                                         const double *d_grad, const double *d_w, const double *d_value,
                                         const double *d_gradient, const double *d_symgrad,
                                         const double *d_div, double *d_values, double *d_scratch,
                                         void *stream) {
    return guarded([&] {
        require(pat != nullptr, "pattern is NULL");
        const int L = nodes * comp;
        require(nodes > 0 && comp > 0 && nq > 0 && ne == pat->n_elements && L == pat->row_local &&
                    L == pat->col_local,
                "tabulated arrays do not match the pattern");
        if (ne == 0) return;  // no elements: no CSR entries
        require(d_value || d_gradient || d_symgrad || d_div, "at least one coefficient is required");
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
#define SKG_TAB(NN_, CC_, BLK_)                                                                                  \
    k_h1_local_tab<NN_, CC_, BLK_><<<grid_for(ne, BLK_), BLK_, 0, s>>>(ne, nq, d_shape, d_grad, d_w, d_value,      \
                                                                      d_gradient, d_symgrad, d_div, Ke)
#define SKG_SYM(NN_, CC_, BLK_)                                                                                  \
    do {                                                                                                         \
        const int smem = BLK_ * (NN_ * CC_ * NN_ * CC_ + 1) * 8;                                                 \
        if (smem > 48 * 1024)                                                                                    \
            SKG_CUDA(cudaFuncSetAttribute(k_h1_local_sym<NN_, CC_, BLK_>,                                        \
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, smem));                   \
        k_h1_local_sym<NN_, CC_, BLK_><<<grid_for(ne, BLK_), BLK_, smem, s>>>(ne, nq, d_shape, d_grad, d_w,      \
                                                                              d_value, d_gradient, d_symgrad,   \
                                                                              d_div, Ke);                       \
    } while (0)
            if (nodes == 4 && comp == 1) SKG_SYM(4, 1, 128);
            else if (nodes == 4 && comp == 3) SKG_SYM(4, 3, 64);
            else if (nodes == 10 && comp == 1) SKG_SYM(10, 1, 64);
            else if (nodes == 10 && comp == 3) SKG_TAB(10, 3, 64);
            else
                k_h1_local_tabulated<<<grid_for(ne * L, 128), 128, 0, s>>>(ne, nodes, comp, nq, d_shape, d_grad, d_w,
                                                                           d_value, d_gradient, d_symgrad, d_div, Ke);
#undef SKG_TAB
#undef SKG_SYM
            SKG_LAUNCH_CHECK("h1_local_tabulated");
        }
        gather_element_matrices(pat, Ke, d_values, s);
    });
}

extern "C" int skg_h1_assemble_tensor_tabulated(const skg_pattern *pat, const int32_t *d_dofs, int64_t ne,
                                                int32_t nodes, int32_t comp, int32_t nq, const double *d_grad,
                                                const double *d_w, const double *d_coef, double *d_values,
                                                double *d_scratch, void *stream) {
    return guarded([&] {
        require(pat != nullptr, "pattern is NULL");
        const int L = nodes * comp;
        require(nodes > 0 && comp > 0 && nq > 0 && ne == pat->n_elements && L == pat->row_local &&
                    L == pat->col_local,
                "tabulated arrays do not match the pattern");
        if (ne == 0) return;  // no elements: no CSR entries
        require(d_coef && d_grad && d_w, "tensor coefficient or geometry is NULL");
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
        gather_element_matrices(pat, Ke, d_values, s);
    });
}


extern "C" int skg_cross_assemble_tabulated(const skg_pattern *pat, int64_t ne, int32_t nq, int32_t nt, int32_t Ct,
                                            int32_t row_kind, const double *d_t_shape, const double *d_t_grad,
                                            int32_t nc, int32_t Cc, int32_t col_kind, const double *d_c_shape,
                                            const double *d_c_grad, const double *d_dx, const double *d_coef,
                                            double *d_values, void *stream) {
    return guarded([&] {
        require(pat != nullptr, "pattern is NULL");
        require(nt > 0 && nc > 0 && Ct > 0 && Cc > 0 && nq > 0, "invalid local sizes");
        require(ne == pat->n_elements && pat->row_local == nt * Ct && pat->col_local == nc * Cc,
                "tabulated arrays do not match the pattern");
        require((row_kind == 0 || row_kind == 1) && (col_kind == 0 || col_kind == 1),
                "tensor kind must be value or gradient");
        if (ne == 0) return;  // no elements: no CSR entries
        require((row_kind == 0 ? d_t_shape : d_t_grad) && (col_kind == 0 ? d_c_shape : d_c_grad) && d_dx && d_coef,
                "tabulated geometry or coefficient arrays are NULL");
        cudaStream_t s = as_stream(stream);
        const int Lt = nt * Ct, Lc = nc * Cc;
        DevBuf<double> Ke((size_t)ne * Lt * Lc, s);
        if (ne) {
            k_cross_local<<<grid_for(ne * Lt, 128), 128, 0, s>>>(ne, nq, nt, Ct, row_kind ? 3 : 1, d_t_shape, d_t_grad,
                                                                nc, Cc, col_kind ? 3 : 1, d_c_shape, d_c_grad, d_dx,
                                                                d_coef, Ke.get());
            SKG_LAUNCH_CHECK("cross_local");
        }
        gather_element_matrices(pat, Ke.get(), d_values, s);
    });
}
