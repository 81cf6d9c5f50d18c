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

// Geometry of element e: J and its cofactor matrix C = det J * J^-1 (row k of
// C is det J times the gradient of lambda_{k+1}); the kernels apply the
// powers of 1 / det J to a few scalars instead of forming J^-1.
struct ElemAdj {
    double C[9], det, id;  // id = 1 / det J
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
    double J[9];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const double x0 = p[i * npts + v[0]];
#pragma unroll
        for (int r = 0; r < 3; ++r) J[i * 3 + r] = p[i * npts + v[r + 1]] - x0;
    }
    double *C = g.C;
    C[0] = J[4] * J[8] - J[5] * J[7]; C[1] = J[2] * J[7] - J[1] * J[8]; C[2] = J[1] * J[5] - J[2] * J[4];
    C[3] = J[5] * J[6] - J[3] * J[8]; C[4] = J[0] * J[8] - J[2] * J[6]; C[5] = J[2] * J[3] - J[0] * J[5];
    C[6] = J[3] * J[7] - J[4] * J[6]; C[7] = J[1] * J[6] - J[0] * J[7]; C[8] = J[0] * J[4] - J[1] * J[3];
    g.det = J[0] * C[0] + J[1] * C[3] + J[2] * C[6];
    g.id = 1.0 / g.det;
    return ok;
}

// C^T y: out_j = sum_k C[k][j] y_k  (det J times J^-T y)
__device__ __forceinline__ void mul_CT(const double C[9], const double y[3], double out[3]) {
#pragma unroll
    for (int j = 0; j < 3; ++j) out[j] = C[0 * 3 + j] * y[0] + C[1 * 3 + j] * y[1] + C[2 * 3 + j] * y[2];
}
// C y: out_i = sum_j C[i][j] y_j  (det J times J^-1 y)
__device__ __forceinline__ void mul_C(const double C[9], const double y[3], double out[3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i) out[i] = C[i * 3 + 0] * y[0] + C[i * 3 + 1] * y[1] + C[i * 3 + 2] * y[2];
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
        double a[3], b[3];  // det J times grad u_e, grad v_e
        mul_CT(g.C, gu, a);
        mul_CT(g.C, gv, b);
        // kappa |det J| wsum (grad u_e . grad v_e) = kappa wsum (a . b) / |det J|
        f = (kappa ? kappa[e] : 1.0) * wsum * fabs(g.id) * (a[0] * b[0] + a[1] * b[1] + a[2] * b[2]);
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

// Element e's adjoint contributions (see k_energy_grad_elem); returns its energy.
__device__ __forceinline__ double elem_adjoint(int64_t ne, const double *__restrict__ p, int64_t npts,
                                               const int32_t *__restrict__ t, const int32_t *__restrict__ dofs,
                                               const double *__restrict__ kappa, const double *__restrict__ u,
                                               const double *__restrict__ v, double wsum, double gout,
                                               double *__restrict__ gkappa, double *__restrict__ contrib,
                                               int64_t e) {
    int32_t vt[4];
    ElemAdj g;
    elem_geom(p, npts, t, ne, e, vt, g);
    const int32_t d0 = dofs[e * 4], d1 = dofs[e * 4 + 1], d2 = dofs[e * 4 + 2], d3 = dofs[e * 4 + 3];
    const double gu[3] = {u[d1] - u[d0], u[d2] - u[d0], u[d3] - u[d0]};
    const double gv[3] = {v[d1] - v[d0], v[d2] - v[d0], v[d3] - v[d0]};
    // with tildes for the scaled quantities:  a = a~ / det, b = b~ / det,
    // c = J^-1 b = c~ / det^2, d = J^-1 a = d~ / det^2, phi = a . b = phi~ / det^2
    double a[3], b[3], c[3], d[3];
    mul_CT(g.C, gu, a);
    mul_CT(g.C, gv, b);
    mul_C(g.C, b, c);
    mul_C(g.C, a, d);
    const double phi = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
    const double aid = fabs(g.id);
    const double k = kappa ? kappa[e] : 1.0;
    if (gkappa) gkappa[e] = gout * wsum * aid * phi;  // V phi = wsum phi~ / |det|
    const double s2 = gout * k * wsum * aid;           // s / det^2 with s = gout kappa V
    const double s3 = s2 * g.id;                       // s / det^3
    double *out = contrib + e * 20;
    // dJ/dJ_ij = s (phi Ji[j][i] - a_i c_j - b_i d_j) = s / det^3 (phi~ C[j][i] - a~_i c~_j - b~_i d~_j)
    const double ph = s3 * phi;
    double as[3], bs[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        as[i] = s3 * a[i];
        bs[i] = s3 * b[i];
    }
    double col_sum[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const double gJ = ph * g.C[j * 3 + i] - as[i] * c[j] - bs[i] * d[j];
            out[(j + 1) * 3 + i] = gJ;  // vertex j+1, coordinate i
            col_sum[i] += gJ;
        }
#pragma unroll
    for (int i = 0; i < 3; ++i) out[i] = -col_sum[i];
    // dJ/du_m = s grad lambda_m . b = s c_{m-1} (m = 1..3), dJ/dv_m = s d_{m-1};
    // lambda_0's gradient is minus the sum of the others
    double du[3], dv[3];
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        du[m] = s2 * c[m];
        dv[m] = s2 * d[m];
        out[13 + m] = du[m];
        out[17 + m] = dv[m];
    }
    out[12] = -(du[0] + du[1] + du[2]);
    out[16] = -(dv[0] + dv[1] + dv[2]);
    return k * wsum * aid * phi;  // the element energy, as k_energy forms it
}

// Backward, element pass: dJ/dkappa and the per-element vertex / DOF
// contributions (scaled by the upstream gradient).  contrib layout per
// element: 12 doubles dx (vertex k, coordinate i at k*3+i), 4 du, 4 dv.
// WITH_J: the element energies are also reduced per block exactly as
// k_energy does (same expression, same tree), so that one pass gives J and
// its gradients.
template <bool WITH_J>
__global__ void __launch_bounds__(kRed) k_energy_grad_elem(int64_t ne, const double *__restrict__ p, int64_t npts,
                                                           const int32_t *__restrict__ t,
                                                           const int32_t *__restrict__ dofs,
                                                           const double *__restrict__ kappa,
                                                           const double *__restrict__ u,
                                                           const double *__restrict__ v, double wsum, double gout,
                                                           double *__restrict__ gkappa, double *__restrict__ contrib,
                                                           double *__restrict__ block_sums) {
    const int64_t e = (int64_t)blockIdx.x * kRed + threadIdx.x;
    double f = 0.0;
    if (e < ne) f = elem_adjoint(ne, p, npts, t, dofs, kappa, u, v, wsum, gout, gkappa, contrib, e);
    if constexpr (WITH_J) {
        __shared__ double red[kRed];
        red[threadIdx.x] = f;
        __syncthreads();
        for (int off = kRed / 2; off > 0; off >>= 1) {
            if (threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
            __syncthreads();
        }
        if (threadIdx.x == 0) block_sums[blockIdx.x] = red[0];
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

namespace {
void energy_grad(const skg_pattern *vertex_inc, const skg_pattern *dof_inc, const double *d_p, int64_t npts,
                 const int32_t *d_t, int64_t ne, const int32_t *d_dofs, const double *d_kappa, const double *d_u,
                 const double *d_v, double wsum, double grad_out, double *d_energy, double *d_gkappa, double *d_gp,
                 double *d_gu, double *d_gv, cudaStream_t s) {
    {
        require(ne >= 0 && (ne == 0 || (d_p && d_t && d_dofs && d_u && d_v)), "invalid energy arguments");
        require(!d_gp || (vertex_inc && vertex_inc->row_local == 4 && vertex_inc->n_elements == ne &&
                          vertex_inc->n_rows == npts),
                "coordinate gradients need the vertex incidence handle of this mesh");
        require((!d_gu && !d_gv) || (dof_inc && dof_inc->row_local == 4 && dof_inc->n_elements == ne),
                "DOF gradients need the DOF incidence handle of this basis");
        DevBuf<double> contrib((size_t)(ne ? ne : 1) * 20, s);
        const int64_t nb = ne ? (ne + kRed - 1) / kRed : 1;
        DevBuf<double> partial(d_energy ? nb : 0, s);
        if (ne) {
            if (d_energy)
                k_energy_grad_elem<true><<<(unsigned)nb, kRed, 0, s>>>(ne, d_p, npts, d_t, d_dofs, d_kappa, d_u, d_v,
                                                                       wsum, grad_out, d_gkappa, contrib.get(),
                                                                       partial.get());
            else
                k_energy_grad_elem<false><<<(unsigned)nb, kRed, 0, s>>>(ne, d_p, npts, d_t, d_dofs, d_kappa, d_u,
                                                                        d_v, wsum, grad_out, d_gkappa, contrib.get(),
                                                                        nullptr);
            SKG_LAUNCH_CHECK("energy_grad_elem");
        } else if (d_energy) {
            SKG_CUDA(cudaMemsetAsync(partial.get(), 0, 8, s));
        }
        if (d_energy) {
            k_sum_blocks<<<1, 32, 0, s>>>(partial.get(), nb, d_energy);
            SKG_LAUNCH_CHECK("energy_sum");
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
    }
}
}  // namespace

extern "C" int skg_p1_energy_grad(const skg_pattern *vertex_inc, const skg_pattern *dof_inc, const double *d_p,
                                  int64_t npts, const int32_t *d_t, int64_t ne, const int32_t *d_dofs,
                                  const double *d_kappa, const double *d_u, const double *d_v, double wsum,
                                  double grad_out, double *d_gkappa, double *d_gp, double *d_gu, double *d_gv,
                                  void *stream) {
    return guarded([&] {
        energy_grad(vertex_inc, dof_inc, d_p, npts, d_t, ne, d_dofs, d_kappa, d_u, d_v, wsum, grad_out, nullptr,
                    d_gkappa, d_gp, d_gu, d_gv, as_stream(stream));
    });
}

extern "C" int skg_p1_energy_value_and_grad(const skg_pattern *vertex_inc, const skg_pattern *dof_inc,
                                            const double *d_p, int64_t npts, const int32_t *d_t, int64_t ne,
                                            const int32_t *d_dofs, const double *d_kappa, const double *d_u,
                                            const double *d_v, double wsum, double grad_out, double *d_energy,
                                            double *d_gkappa, double *d_gp, double *d_gu, double *d_gv,
                                            void *stream) {
    return guarded([&] {
        require(d_energy != nullptr, "energy output is NULL");
        energy_grad(vertex_inc, dof_inc, d_p, npts, d_t, ne, d_dofs, d_kappa, d_u, d_v, wsum, grad_out, d_energy,
                    d_gkappa, d_gp, d_gu, d_gv, as_stream(stream));
    });
}
