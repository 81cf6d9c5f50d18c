// Linear-form (load / residual vector) assembly: the GPU counterpart of
// LinearFormAssembler (cpp/src/assembly/linear_form_assembler.cpp:41-154),
//   r[dof(a, c)] += sum_q w (f_c N_a + G_cj dN_a/dx_j).
// One thread per DOF walks the DOF's incidence list (element, local dof) in
// ascending element order, so the sum per DOF is made in a fixed order
// without atomics.
#include "skg_common.cuh"

namespace skg {
namespace {

__global__ void k_linear_rows(int64_t n_rows, const int32_t *__restrict__ inc_ptr, const int32_t *__restrict__ inc,
                              int n, int C, int nq, const double *__restrict__ shape, const double *__restrict__ grad,
                              const double *__restrict__ w, const double *__restrict__ value,
                              const double *__restrict__ gradient, double *__restrict__ out) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rows) return;
    const int L = n * C;
    double acc = 0.;
    for (int32_t t = inc_ptr[r]; t < inc_ptr[r + 1]; ++t) {
        const int32_t item = inc[t];
        const int64_t e = item / L;
        const int i = item - (int)(e * L);
        const int a = i / C, c = i % C;
        double local = 0.;
        for (int q = 0; q < nq; ++q) {
            const int64_t eq = e * nq + q;
            double contrib = 0.;
            if (value) contrib += shape[eq * n + a] * value[eq * C + c];
            if (gradient) {
                const double *g = grad + (eq * n + a) * 3;
                const double *G = gradient + (eq * C + c) * 3;
                contrib += g[0] * G[0] + g[1] * G[1] + g[2] * G[2];
            }
            local += w[eq] * contrib;
        }
        acc += local;
    }
    out[r] = acc;
}

}  // namespace
}  // namespace skg

using namespace skg;

extern "C" int skg_linear_assemble_tabulated(const skg_pattern *pat, const int32_t *d_dofs, int64_t ne,
                                             int32_t nodes, int32_t comp, int32_t nq, const double *d_shape,
                                             const double *d_grad, const double *d_w, const double *d_value,
                                             const double *d_gradient, double *d_out, void *stream) {
    return guarded([&] {
        require(pat != nullptr, "pattern is NULL");
        require(ne == pat->n_elements && pat->row_local == nodes * comp, "tabulated arrays do not match the pattern");
        (void)d_dofs;
        cudaStream_t s = as_stream(stream);
        if (!pat->n_rows) return;
        if (ne == 0) {  // no elements: a zero vector
            require(d_out != nullptr, "output is NULL");
            SKG_CUDA(cudaMemsetAsync(d_out, 0, (size_t)pat->n_rows * sizeof(double), s));
            return;
        }
        require(d_value || d_gradient, "at least one coefficient is required");
        require(d_w && (!d_value || d_shape) && (!d_gradient || d_grad), "tabulated geometry arrays are NULL");
        k_linear_rows<<<grid_for(pat->n_rows, 128), 128, 0, s>>>(pat->n_rows, pat->inc_ptr.get(), pat->inc.get(), nodes,
                                                                 comp, nq, d_shape, d_grad, d_w, d_value, d_gradient,
                                                                 d_out);
        SKG_LAUNCH_CHECK("linear_rows");
    });
}
