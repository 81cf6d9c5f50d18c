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
// (the contraction of A with g_a and g_b written out).  One thread per element
// computes the 12 residual and 144 tangent entries; they are summed into the
// residual vector and the CSR values by the fixed-order gathers (one thread
// per DOF / CSR row, element order), so results are bitwise reproducible.
//
// The surrogate entry point replaces the law by a small MLP on the
// invariants (see skg_mlp.cu) with a per-element fallback to this law.
#include "skg_common.cuh"
#include "skg_nh.cuh"

namespace skg {

void gather_element_matrices(const skg_pattern *pat, const double *Ke, double *values, cudaStream_t s);

namespace {

__global__ void k_nh_element(int64_t ne, const double *__restrict__ p, int64_t npts, const int32_t *__restrict__ t,
                             const int32_t *__restrict__ dofs, const double *__restrict__ u, double mu, double lmbda,
                             double wsum, double *__restrict__ Ke, double *__restrict__ re) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    NhGeom g;
    nh_geometry(p, npts, t, ne, e, wsum, g);
    double Gu[9];
    displacement_gradient(g, dofs + e * 12, u, Gu);
    NhLaw law;
    nh_plain_law(Gu, mu, lmbda, law);
    write_nh_element(g, law, mu, lmbda, Ke ? Ke + e * 144 : nullptr, re ? re + e * 12 : nullptr);
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

extern "C" int skg_nh_assemble(const skg_pattern *pat, const double *d_p, int64_t npts, const int32_t *d_t,
                               int64_t ne, const double *d_u, double mu, double lmbda, double wsum,
                               double *d_residual, double *d_values, void *stream) {
    return guarded([&] {
        require(pat != nullptr, "pattern is NULL");
        require(pat->row_local == 12 && pat->n_elements == ne, "neo-Hookean assembly needs the vector P1 pattern");
        require(!d_values || pat->col_local == 12, "tangent output needs a pattern with CSR columns");
        require(d_p && d_t && d_u, "mesh or displacement arrays are NULL");
        cudaStream_t s = as_stream(stream);
        DevBuf<double> Ke(d_values ? (size_t)ne * 144 : 0, s), re(d_residual ? (size_t)ne * 12 : 0, s);
        if (ne) {
            k_nh_element<<<grid_for(ne, 128), 128, 0, s>>>(ne, d_p, npts, d_t, pat->row_dofs.get(), d_u, mu, lmbda,
                                                          wsum, Ke.get(), re.get());
            SKG_LAUNCH_CHECK("nh_element");
        }
        nh_gather(pat, Ke.get(), re.get(), d_residual, d_values, s);
    });
}
