// Fused neo-Hookean row pass: per-element records in, CSR tangent values and
// the residual vector out, no element matrices in memory.
//
// Plain record (FP64, kNhRecD doubles per element):
//   [0, 12)  g_a = grad lambda_a          [12, 24) h_a = F^-T g_a
//   [24, 33) V P (first Piola times measure)
//   33: mu V    34: (mu - lambda ln J) V    35: lambda V
// so that K_(a,i),(b,k) = mu V d_ik g_a.g_b + c2 V h_b,i h_a,k + lambda V h_a,i h_b,k
// and r_(a,i) = sum_j (V P)_ij g_a,j.
//
// Surrogate record (FP32, kNhRecF floats per element): the element tangent
// rows [12 (3a + i) .. +12) = K_(a,i),(b,k) = sum_JL g_a,J (V A)_iJkL g_b,L,
// then [144, 156) the residual entries r_(a,i) = sum_j (V P)_ij g_a,j.
#pragma once

#include "skg_common.cuh"
#include "skg_df64.cuh"
#include "skg_nh.cuh"
#include "skg_rows.cuh"

namespace skg {

constexpr int kNhRecD = 36;
constexpr int kNhRecF = 156;

__device__ __forceinline__ void write_plain_record(const NhGeom &g, const NhLaw &L, double mu, double lmbda,
                                                   double *__restrict__ r) {
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            r[a * 3 + j] = g.g[a][j];
            r[12 + a * 3 + j] = L.FiT[j * 3] * g.g[a][0] + L.FiT[j * 3 + 1] * g.g[a][1] + L.FiT[j * 3 + 2] * g.g[a][2];
        }
#pragma unroll
    for (int k = 0; k < 9; ++k) r[24 + k] = g.V * L.P[k];
    r[33] = mu * g.V;
    r[34] = (mu - lmbda * L.lnJ) * g.V;
    r[35] = lmbda * g.V;
}

// Surrogate row pass; `fallbacks` (device) counts the call's elements sent
// to the plain law: FP32 slots when it is zero, double-float slots otherwise.
void nh_rows(const skg_pattern *pat, const GroupSet &gs, const double *recd, const float *recf,
             const unsigned char *flags, const unsigned long long *fallbacks, double *d_residual, double *d_values,
             cudaStream_t s);

// Residual and tangent from per-element arrays (patterns without row groups).
void nh_gather(const skg_pattern *pat, const double *Ke, const double *re, double *d_residual, double *d_values,
               cudaStream_t s);

// Whole-array copies of the results to the host (paths without row chunks).
void nh_download(const skg_pattern *pat, const double *d_residual, const double *d_values, double *h_residual,
                 double *h_values, cudaStream_t s);

}  // namespace skg
