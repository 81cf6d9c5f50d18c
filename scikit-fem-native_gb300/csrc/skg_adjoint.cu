// Matrix-free energy J = u^T K(kappa) v of P1 diffusion and its adjoint.
//
// K(kappa) is the matrix `asm(w.kappa * ddot(grad u, grad v), basis)` builds
// for a P1 basis with per-element kappa (python/skfemntv/forms.py:276-374,
// bilinear_form_assembler.cpp:79-105); the reference has no adjoint, so the
// gradients below are checked against central finite differences through the
// assembled matrix and against exact directional derivatives of it.
//
// Per element (affine map with Jacobian J, columns x_k - x_0):
//   V   = |det J| * wsum                 (wsum = sum of the rule's weights)
//   a   = grad u_e = J^-T gu,  b = grad v_e = J^-T gv,
//         gu = (u1-u0, u2-u0, u3-u0), gv likewise
//   J_e = kappa_e V (a . b)
//   dJ/dkappa_e = V (a . b)
//   dJ/dJ       = kappa_e V ((a . b) J^-T - a c^T - b d^T),  c = J^-1 b, d = J^-1 a
//   dJ/dx_k     = column k-1 of dJ/dJ (k = 1..3),  dJ/dx_0 = -(sum of the columns)
//   dJ/du_m     = kappa_e V (grad lambda_m . b),  dJ/dv_m = kappa_e V (grad lambda_m . a)
// The backward pass recomputes the geometry (nothing is stored by the
// forward pass).  Element contributions to vertex / DOF gradients are summed
// by one thread per vertex / DOF over its incidence list in element order
// (fixed order, no atomics); the energy is reduced in a fixed tree order.
#include <vector>

#include "skg_common.cuh"

namespace skg {
namespace {

struct ElemAdj {
    double J[9], Ji[9], det;
};

__device__ __forceinline__ bool elem_geom(const double *__restrict__ p, int64_t npts, const int32_t *__restrict__ t,
                                          int64_t ne, int64_t e, int32_t v[4], ElemAdj &g) {
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        v[k] = t[k * ne + e];
        ok = ok && v[k] >= 0 && v[k] < npts;
    }
    if (!ok) v[0] = v[1] = v[2] = v[3] = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const double x0 = p[i * npts + v[0]];
#pragma unroll
        for (int r = 0; r < 3; ++r) g.J[i * 3 + r] = p[i * npts + v[r + 1]] - x0;
    }
    const double *J = g.J;
    const double c00 = J[4] * J[8] - J[5] * J[7], c01 = J[2] * J[7] - J[1] * J[8], c02 = J[1] * J[5] - J[2] * J[4];
    const double c10 = J[5] * J[6] - J[3] * J[8], c11 = J[0] * J[8] - J[2] * J[6], c12 = J[2] * J[3] - J[0] * J[5];
    const double c20 = J[3] * J[7] - J[4] * J[6], c21 = J[1] * J[6] - J[0] * J[7], c22 = J[0] * J[4] - J[1] * J[3];
    g.det = J[0] * c00 + J[1] * c10 + J[2] * c20;
    const double id = 1.0 / g.det;
    g.Ji[0] = c00 * id; g.Ji[1] = c01 * id; g.Ji[2] = c02 * id;
    g.Ji[3] = c10 * id; g.Ji[4] = c11 * id; g.Ji[5] = c12 * id;
    g.Ji[6] = c20 * id; g.Ji[7] = c21 * id; g.Ji[8] = c22 * id;
    return ok;
}

// J^-T y (= rows of J^-1 weighted): out_j = sum_k Ji[k][j] y_k
__device__ __forceinline__ void mul_JiT(const double Ji[9], const double y[3], double out[3]) {
#pragma unroll
    for (int j = 0; j < 3; ++j) out[j] = Ji[0 * 3 + j] * y[0] + Ji[1 * 3 + j] * y[1] + Ji[2 * 3 + j] * y[2];
}
// J^-1 y: out_i = sum_j Ji[i][j] y_j
__device__ __forceinline__ void mul_Ji(const double Ji[9], const double y[3], double out[3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i) out[i] = Ji[i * 3 + 0] * y[0] + Ji[i * 3 + 1] * y[1] + Ji[i * 3 + 2] * y[2];
}

constexpr int kRed = 256;

// Forward: per-element energies reduced per block (fixed tree order).
__global__ void __launch_bounds__(kRed) k_energy(int64_t ne, const double *__restrict__ p, int64_t npts,
                                                 const int32_t *__restrict__ t, const int32_t *__restrict__ dofs,
                                                 const double *__restrict__ kappa, const double *__restrict__ u,
                                                 const double *__restrict__ v, double wsum,
                                                 double *__restrict__ block_sums) {
    __shared__ double red[kRed];
    const int64_t e = (int64_t)blockIdx.x * kRed + threadIdx.x;
    double f = 0.0;
    if (e < ne) {
        int32_t vt[4];
        ElemAdj g;
        elem_geom(p, npts, t, ne, e, vt, g);
        const int32_t d0 = dofs[e * 4], d1 = dofs[e * 4 + 1], d2 = dofs[e * 4 + 2], d3 = dofs[e * 4 + 3];
        const double gu[3] = {u[d1] - u[d0], u[d2] - u[d0], u[d3] - u[d0]};
        const double gv[3] = {v[d1] - v[d0], v[d2] - v[d0], v[d3] - v[d0]};
        double a[3], b[3];
        mul_JiT(g.Ji, gu, a);
        mul_JiT(g.Ji, gv, b);
        f = (kappa ? kappa[e] : 1.0) * fabs(g.det) * wsum * (a[0] * b[0] + a[1] * b[1] + a[2] * b[2]);
    }
    red[threadIdx.x] = f;
    __syncthreads();
    for (int off = kRed / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) block_sums[blockIdx.x] = red[0];
}

// One warp, fixed order: lane l sums the block sums l, l + 32, ... in turn,
// then the lanes are combined by a fixed shuffle tree.
__global__ void k_sum_blocks(const double *__restrict__ in, int64_t n, double *__restrict__ out) {
    const int lane = threadIdx.x & 31;
    double s = 0.0;
    for (int64_t i = lane; i < n; i += 32) s += in[i];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if (lane == 0) *out = s;
}

// Backward, element pass: dJ/dkappa and the per-element vertex / DOF
// contributions (scaled by the upstream gradient).  contrib layout per
// element: 12 doubles dx (vertex k, coordinate i at k*3+i), 4 du, 4 dv.
__global__ void k_energy_grad_elem(int64_t ne, const double *__restrict__ p, int64_t npts,
                                   const int32_t *__restrict__ t, const int32_t *__restrict__ dofs,
                                   const double *__restrict__ kappa, const double *__restrict__ u,
                                   const double *__restrict__ v, double wsum, double gout,
                                   double *__restrict__ gkappa, double *__restrict__ contrib) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    int32_t vt[4];
    ElemAdj g;
    elem_geom(p, npts, t, ne, e, vt, g);
    const int32_t d0 = dofs[e * 4], d1 = dofs[e * 4 + 1], d2 = dofs[e * 4 + 2], d3 = dofs[e * 4 + 3];
    const double gu[3] = {u[d1] - u[d0], u[d2] - u[d0], u[d3] - u[d0]};
    const double gv[3] = {v[d1] - v[d0], v[d2] - v[d0], v[d3] - v[d0]};
    double a[3], b[3], c[3], d[3];
    mul_JiT(g.Ji, gu, a);
    mul_JiT(g.Ji, gv, b);
    mul_Ji(g.Ji, b, c);
    mul_Ji(g.Ji, a, d);
    const double phi = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
    const double V = fabs(g.det) * wsum;
    const double k = kappa ? kappa[e] : 1.0;
    if (gkappa) gkappa[e] = gout * V * phi;
    const double s = gout * k * V;
    double *out = contrib + e * 20;
    // dJ/dJ_ij = s (phi Ji[j][i] - a_i c_j - b_i d_j)
    double col_sum[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const double gJ = s * (phi * g.Ji[j * 3 + i] - a[i] * c[j] - b[i] * d[j]);
            out[(j + 1) * 3 + i] = gJ;  // vertex j+1, coordinate i
            col_sum[i] += gJ;
        }
#pragma unroll
    for (int i = 0; i < 3; ++i) out[i] = -col_sum[i];
    // grad lambda_m = J^-T e_{m-1} (m = 1..3), grad lambda_0 = -(sum)
    double gl[4][3];
#pragma unroll
    for (int m = 1; m < 4; ++m)
#pragma unroll
        for (int j = 0; j < 3; ++j) gl[m][j] = g.Ji[(m - 1) * 3 + j];
#pragma unroll
    for (int j = 0; j < 3; ++j) gl[0][j] = -(gl[1][j] + gl[2][j] + gl[3][j]);
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        out[12 + m] = s * (gl[m][0] * b[0] + gl[m][1] * b[1] + gl[m][2] * b[2]);
        out[16 + m] = s * (gl[m][0] * a[0] + gl[m][1] * a[1] + gl[m][2] * a[2]);
    }
}

// Backward, gather pass: one thread per row of an incidence list (vertex or
// DOF), summing the element contributions in element order.
//   coordinates (out_x, (3, n_rows), component-major like mesh.p) and / or
//   u / v DOFs (out_u, out_v (n_rows)); both in one walk when the vertex and
//   DOF incidence lists coincide (scalar P1 with every vertex a DOF).
__global__ void k_energy_grad_gather(int64_t n_rows, const int32_t *__restrict__ inc_ptr,
                                     const int32_t *__restrict__ inc, const double *__restrict__ contrib,
                                     double *__restrict__ out_x, double *__restrict__ out_u,
                                     double *__restrict__ out_v) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rows) return;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, su = 0.0, sv = 0.0;
    for (int32_t it = inc_ptr[r]; it < inc_ptr[r + 1]; ++it) {
        const int32_t item = inc[it];
        const int64_t e = item >> 2;
        const int k = item & 3;
        const double *c = contrib + e * 20;
        if (out_x) {
            s0 += c[k * 3];
            s1 += c[k * 3 + 1];
            s2 += c[k * 3 + 2];
        }
        if (out_u) su += c[12 + k];
        if (out_v) sv += c[16 + k];
    }
    if (out_x) {
        out_x[r] = s0;
        out_x[n_rows + r] = s1;
        out_x[2 * n_rows + r] = s2;
    }
    if (out_u) out_u[r] = su;
    if (out_v) out_v[r] = sv;
}

}  // namespace
}  // namespace skg

using namespace skg;

extern "C" int skg_p1_energy(const double *d_p, int64_t npts, const int32_t *d_t, int64_t ne, const int32_t *d_dofs,
                             const double *d_kappa, const double *d_u, const double *d_v, double wsum, double *d_out,
                             void *stream) {
    return guarded([&] {
        require(ne >= 0 && d_out && (ne == 0 || (d_p && d_t && d_dofs && d_u && d_v)), "invalid energy arguments");
        cudaStream_t s = as_stream(stream);
        const int64_t nb = ne ? (ne + kRed - 1) / kRed : 1;
        DevBuf<double> partial(nb, s);
        if (ne) {
            k_energy<<<(unsigned)nb, kRed, 0, s>>>(ne, d_p, npts, d_t, d_dofs, d_kappa, d_u, d_v, wsum, partial.get());
            SKG_LAUNCH_CHECK("energy");
        } else {
            SKG_CUDA(cudaMemsetAsync(partial.get(), 0, 8, s));
        }
        k_sum_blocks<<<1, 32, 0, s>>>(partial.get(), nb, d_out);
        SKG_LAUNCH_CHECK("energy_sum");
    });
}

extern "C" int skg_p1_energy_grad(const skg_pattern *vertex_inc, const skg_pattern *dof_inc, const double *d_p,
                                  int64_t npts, const int32_t *d_t, int64_t ne, const int32_t *d_dofs,
                                  const double *d_kappa, const double *d_u, const double *d_v, double wsum,
                                  double grad_out, double *d_gkappa, double *d_gp, double *d_gu, double *d_gv,
                                  void *stream) {
    return guarded([&] {
        require(ne >= 0 && (ne == 0 || (d_p && d_t && d_dofs && d_u && d_v)), "invalid energy arguments");
        require(!d_gp || (vertex_inc && vertex_inc->row_local == 4 && vertex_inc->n_elements == ne &&
                          vertex_inc->n_rows == npts),
                "coordinate gradients need the vertex incidence handle of this mesh");
        require((!d_gu && !d_gv) || (dof_inc && dof_inc->row_local == 4 && dof_inc->n_elements == ne),
                "DOF gradients need the DOF incidence handle of this basis");
        cudaStream_t s = as_stream(stream);
        DevBuf<double> contrib((size_t)(ne ? ne : 1) * 20, s);
        if (ne) {
            k_energy_grad_elem<<<grid_for(ne, 128), 128, 0, s>>>(ne, d_p, npts, d_t, d_dofs, d_kappa, d_u, d_v, wsum,
                                                                 grad_out, d_gkappa, contrib.get());
            SKG_LAUNCH_CHECK("energy_grad_elem");
        }
        const bool shared = vertex_inc == dof_inc;  // one incidence structure for both
        if (d_gp && shared) {
            k_energy_grad_gather<<<grid_for(npts, 128), 128, 0, s>>>(npts, vertex_inc->inc_ptr.get(),
                                                                     vertex_inc->inc.get(), contrib.get(), d_gp, d_gu,
                                                                     d_gv);
            SKG_LAUNCH_CHECK("energy_grad_xuv");
            return;
        }
        if (d_gp) {
            k_energy_grad_gather<<<grid_for(npts, 128), 128, 0, s>>>(npts, vertex_inc->inc_ptr.get(),
                                                                     vertex_inc->inc.get(), contrib.get(), d_gp,
                                                                     nullptr, nullptr);
            SKG_LAUNCH_CHECK("energy_grad_x");
        }
        if (d_gu || d_gv) {
            k_energy_grad_gather<<<grid_for(dof_inc->n_rows, 128), 128, 0, s>>>(
                dof_inc->n_rows, dof_inc->inc_ptr.get(), dof_inc->inc.get(), contrib.get(), nullptr, d_gu, d_gv);
            SKG_LAUNCH_CHECK("energy_grad_uv");
        }
    });
}
