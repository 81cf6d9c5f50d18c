// Device helpers shared by the plain neo-Hookean kernel and the MLP
// surrogate: P1 element geometry, displacement gradient, the plain law, and
// the element residual / tangent from a first Piola stress and a tangent
// tensor.
#pragma once

#include "skg_common.cuh"

namespace skg {

struct NhGeom {
    double g[4][3];  // barycentric gradients grad lambda_a
    double V;        // |det J| * sum of weights
    bool ok;
};

__device__ __forceinline__ void nh_geometry(const double *__restrict__ p, int64_t npts, const int32_t *__restrict__ t,
                                            int64_t ne, int64_t e, double wsum, NhGeom &g) {
    int32_t v[4];
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
    const double c00 = J[4] * J[8] - J[5] * J[7], c01 = J[2] * J[7] - J[1] * J[8], c02 = J[1] * J[5] - J[2] * J[4];
    const double c10 = J[5] * J[6] - J[3] * J[8], c11 = J[0] * J[8] - J[2] * J[6], c12 = J[2] * J[3] - J[0] * J[5];
    const double c20 = J[3] * J[7] - J[4] * J[6], c21 = J[1] * J[6] - J[0] * J[7], c22 = J[0] * J[4] - J[1] * J[3];
    const double det = J[0] * c00 + J[1] * c10 + J[2] * c20;
    const double id = 1.0 / det;
    // rows of J^-1 are grad lambda_1..3
    g.g[1][0] = c00 * id; g.g[1][1] = c01 * id; g.g[1][2] = c02 * id;
    g.g[2][0] = c10 * id; g.g[2][1] = c11 * id; g.g[2][2] = c12 * id;
    g.g[3][0] = c20 * id; g.g[3][1] = c21 * id; g.g[3][2] = c22 * id;
#pragma unroll
    for (int j = 0; j < 3; ++j) g.g[0][j] = -(g.g[1][j] + g.g[2][j] + g.g[3][j]);
    g.V = fabs(det) * wsum;
    g.ok = ok;
}

// Gu[c][j] = sum_a u[dof(a, c)] g_a[j]; element DOFs ordered node-major then
// component (dof (a, c) at local index 3a + c).
__device__ __forceinline__ void displacement_gradient(const NhGeom &g, const int32_t *__restrict__ dofs,
                                                      const double *__restrict__ u, double Gu[9]) {
#pragma unroll
    for (int k = 0; k < 9; ++k) Gu[k] = 0.0;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double ua = u[dofs[a * 3 + c]];
#pragma unroll
            for (int j = 0; j < 3; ++j) Gu[c * 3 + j] += ua * g.g[a][j];
        }
}

// First Piola stress P and what the tangent needs: F^-T and ln J.
struct NhLaw {
    double P[9], FiT[9], lnJ, J;
};

__device__ __forceinline__ void nh_plain_law(const double Gu[9], double mu, double lmbda, NhLaw &L) {
    double F[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) F[k] = Gu[k] + ((k % 4) == 0 ? 1.0 : 0.0);
    const double c00 = F[4] * F[8] - F[5] * F[7], c01 = F[2] * F[7] - F[1] * F[8], c02 = F[1] * F[5] - F[2] * F[4];
    const double c10 = F[5] * F[6] - F[3] * F[8], c11 = F[0] * F[8] - F[2] * F[6], c12 = F[2] * F[3] - F[0] * F[5];
    const double c20 = F[3] * F[7] - F[4] * F[6], c21 = F[1] * F[6] - F[0] * F[7], c22 = F[0] * F[4] - F[1] * F[3];
    const double J = F[0] * c00 + F[1] * c10 + F[2] * c20;
    const double id = 1.0 / J;
    // F^-1 = adj / J; F^-T[i][j] = F^-1[j][i]
    const double Fi[9] = {c00 * id, c01 * id, c02 * id, c10 * id, c11 * id, c12 * id, c20 * id, c21 * id, c22 * id};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) L.FiT[i * 3 + j] = Fi[j * 3 + i];
    L.J = J;
    L.lnJ = log(J);
#pragma unroll
    for (int k = 0; k < 9; ++k) L.P[k] = mu * (F[k] - L.FiT[k]) + lmbda * L.lnJ * L.FiT[k];
}

// Element residual (12) and tangent (12 x 12, row (a,i), column (b,k)) of
// the plain law.
__device__ __forceinline__ void write_nh_element(const NhGeom &g, const NhLaw &L, double mu, double lmbda,
                                                 double *__restrict__ Ke, double *__restrict__ re) {
    if (re) {
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int c = 0; c < 3; ++c)
                re[a * 3 + c] = g.V * (L.P[c * 3] * g.g[a][0] + L.P[c * 3 + 1] * g.g[a][1] + L.P[c * 3 + 2] * g.g[a][2]);
    }
    if (!Ke) return;
    double h[4][3];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int i = 0; i < 3; ++i)
            h[a][i] = L.FiT[i * 3] * g.g[a][0] + L.FiT[i * 3 + 1] * g.g[a][1] + L.FiT[i * 3 + 2] * g.g[a][2];
    const double c2 = mu - lmbda * L.lnJ;
    for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b) {
            const double gg = g.g[a][0] * g.g[b][0] + g.g[a][1] * g.g[b][1] + g.g[a][2] * g.g[b][2];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const double val = (i == k ? mu * gg : 0.0) + c2 * h[b][i] * h[a][k] + lmbda * h[a][i] * h[b][k];
                    Ke[(a * 3 + i) * 12 + b * 3 + k] = g.V * val;
                }
        }
}

}  // namespace skg
