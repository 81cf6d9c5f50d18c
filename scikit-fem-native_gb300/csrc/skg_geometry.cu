// Per-(element, point) geometry tabulation, the GPU counterpart of the
// reference's tabulate_basis_geometry (cpp/src/assembly/basis_geometry.cpp
// :49-209).  One thread per (element, point); the reference-basis tables
// (shape and gradients at the quadrature points, element and geometry
// basis) are staged in shared memory.  This translation unit is compiled
// without floating-point contraction and keeps the reference's operation
// order, so its outputs equal the reference's bit for bit.
#include <cmath>
#include <cstring>
#include <sstream>
#include <iomanip>
#include <vector>

#include <algorithm>
#include <climits>

#include "skg_common.cuh"

namespace skg {
namespace {

__global__ void k_tabulate(int64_t ne, int nq, int n, int G, const double *__restrict__ p, int64_t npts,
                           const int32_t *__restrict__ t, const double *__restrict__ tables,
                           double *__restrict__ o_shape, double *__restrict__ o_grad, double *__restrict__ o_dx,
                           double *__restrict__ o_x, double *__restrict__ o_det, double *__restrict__ o_tol,
                           double *__restrict__ o_cond, int32_t *__restrict__ oob) {
    extern __shared__ double tab[];
    // tables: shape (Q,n) | refgrad (Q,n,3) | gshape (Q,G) | grefgrad (Q,G,3) | W (Q)
    const int total = nq * n * 4 + nq * G * 4 + nq;
    for (int i = threadIdx.x; i < total; i += blockDim.x) tab[i] = tables[i];
    __syncthreads();
    const double *shape = tab, *refgrad = tab + nq * n, *gshape = refgrad + nq * n * 3;
    const double *grefgrad = gshape + nq * G, *W = grefgrad + nq * G * 3;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= ne * nq) return;
    const int64_t e = tid / nq;
    const int q = (int)(tid % nq);
    double J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, x[3] = {0, 0, 0};
    for (int a = 0; a < G; ++a) {
        const int32_t v = t[(int64_t)a * ne + e];
        if (v < 0 || v >= npts) { *oob = 1; continue; }
        for (int i = 0; i < 3; ++i) {
            const double c = p[i * npts + v];
            x[i] += gshape[q * G + a] * c;
            for (int j = 0; j < 3; ++j) J[i * 3 + j] += c * grefgrad[(q * G + a) * 3 + j];
        }
    }
    const int64_t eq = e * nq + q;
    if (o_x)
        for (int i = 0; i < 3; ++i) o_x[eq * 3 + i] = x[i];
    double s = 0.;
    for (int i = 0; i < 9; ++i) s = fmax(s, fabs(J[i]));
    const double sp = s * s * s;
    const double tol = 64. * 2.220446049250313e-16 * sp;
    const double det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
                       J[2] * (J[3] * J[7] - J[4] * J[6]);
    o_det[eq] = det;
    o_tol[eq] = tol;
    if (!isfinite(det) || !isfinite(tol) || !(fabs(det) > tol)) return;
    double Ji[9];
    Ji[0] = (J[4] * J[8] - J[5] * J[7]) / det;
    Ji[1] = (J[2] * J[7] - J[1] * J[8]) / det;
    Ji[2] = (J[1] * J[5] - J[2] * J[4]) / det;
    Ji[3] = (J[5] * J[6] - J[3] * J[8]) / det;
    Ji[4] = (J[0] * J[8] - J[2] * J[6]) / det;
    Ji[5] = (J[2] * J[3] - J[0] * J[5]) / det;
    Ji[6] = (J[3] * J[7] - J[4] * J[6]) / det;
    Ji[7] = (J[1] * J[6] - J[0] * J[7]) / det;
    Ji[8] = (J[0] * J[4] - J[1] * J[3]) / det;
    double jn = 0., in = 0.;
    for (int i = 0; i < 9; ++i) { jn += J[i] * J[i]; in += Ji[i] * Ji[i]; }
    if (o_cond) o_cond[eq] = sqrt(jn * in);
    if (o_dx) o_dx[eq] = fabs(det) * W[q];
    for (int a = 0; a < n; ++a) {
        if (o_shape) o_shape[eq * n + a] = shape[q * n + a];
        if (o_grad)
            for (int j = 0; j < 3; ++j) {
                double g = 0.;
                for (int k = 0; k < 3; ++k) g += refgrad[(q * n + a) * 3 + k] * Ji[k * 3 + j];
                o_grad[(eq * n + a) * 3 + j] = g;
            }
    }
}

// First invalid element in element order (near-singular first, then
// orientation change), basis_geometry.cpp:178-205.
__global__ void k_validate(int64_t ne, int nq, const double *__restrict__ det, const double *__restrict__ tol,
                           unsigned long long *bad) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    bool badq = false;
    for (int q = 0; q < nq; ++q) {
        const double d = det[e * nq + q], tl = tol[e * nq + q];
        if (!(isfinite(d) && isfinite(tl) && fabs(d) > tl)) badq = true;
    }
    if (!badq) {
        const bool neg = det[e * nq] < 0.;
        for (int q = 1; q < nq; ++q)
            if ((det[e * nq + q] < 0.) != neg) badq = true;
    }
    if (badq) atomicMin(bad, (unsigned long long)e);
}

// Geometry diagnostics (basis.py:2296-2356) as one reduction over the
// (element, point) arrays: smallest and largest determinant, the smallest
// scaled determinant |det| / (tol / (64 eps)) with its first flat index (the
// first occurrence, as numpy's argmin), the largest condition number with its
// first flat index, and the elements whose first point has a negative
// determinant.  Per block, then one block over the block results.
struct GeomDiag {
    double det_min, det_max, scaled_min, cond_max;
    long long scaled_at, cond_at, negative;
};

__device__ __forceinline__ void diag_merge(GeomDiag &a, const GeomDiag &b) {
    a.det_min = fmin(a.det_min, b.det_min);
    a.det_max = fmax(a.det_max, b.det_max);
    if (b.scaled_min < a.scaled_min || (b.scaled_min == a.scaled_min && b.scaled_at < a.scaled_at)) {
        a.scaled_min = b.scaled_min;
        a.scaled_at = b.scaled_at;
    }
    if (b.cond_max > a.cond_max || (b.cond_max == a.cond_max && b.cond_at < a.cond_at)) {
        a.cond_max = b.cond_max;
        a.cond_at = b.cond_at;
    }
    a.negative += b.negative;
}

__device__ __forceinline__ GeomDiag diag_identity() {
    return GeomDiag{INFINITY, -INFINITY, INFINITY, -INFINITY, LLONG_MAX, LLONG_MAX, 0};
}

constexpr int kDiagThreads = 256;

__device__ __forceinline__ void diag_block_reduce(GeomDiag v, GeomDiag *out) {
    __shared__ GeomDiag sh[kDiagThreads];
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = kDiagThreads / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) diag_merge(sh[threadIdx.x], sh[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

__global__ void __launch_bounds__(kDiagThreads) k_geom_diag(int64_t n, int nq, const double *__restrict__ det,
                                                            const double *__restrict__ tol,
                                                            const double *__restrict__ cond, GeomDiag *part) {
    const double unit = 64.0 * __DBL_EPSILON__;
    GeomDiag v = diag_identity();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double d = det[i];
        v.det_min = fmin(v.det_min, d);
        v.det_max = fmax(v.det_max, d);
        const double sc = fabs(d) / (tol[i] / unit);
        if (sc < v.scaled_min) {  // i increases along the thread's walk: the first index wins ties
            v.scaled_min = sc;
            v.scaled_at = i;
        }
        const double c = cond[i];
        if (c > v.cond_max) {
            v.cond_max = c;
            v.cond_at = i;
        }
        if (i % nq == 0 && d < 0.0) ++v.negative;
    }
    diag_block_reduce(v, part + blockIdx.x);
}

__global__ void __launch_bounds__(kDiagThreads) k_geom_diag_final(int n_parts, const GeomDiag *__restrict__ part,
                                                                  GeomDiag *out) {
    GeomDiag v = diag_identity();
    for (int i = threadIdx.x; i < n_parts; i += blockDim.x) diag_merge(v, part[i]);
    diag_block_reduce(v, out);
}

}  // namespace
}  // namespace skg

using namespace skg;

extern "C" int skg_geometry_diagnostics(const double *d_det, const double *d_tol, const double *d_cond,
                                        int64_t n_elements, int32_t nq, double *h_values, int64_t *h_indices,
                                        void *stream) {
    return guarded([&] {
        require(n_elements > 0 && nq > 0, "geometry diagnostics need at least one element and point");
        require(d_det && d_tol && d_cond && h_values && h_indices, "diagnostics arrays are NULL");
        cudaStream_t s = as_stream(stream);
        const int64_t n = n_elements * (int64_t)nq;
        const int parts = (int)std::min<int64_t>(2 * kSmCount, (n + kDiagThreads - 1) / kDiagThreads);
        DevBuf<GeomDiag> part((size_t)parts + 1, s);
        k_geom_diag<<<parts, kDiagThreads, 0, s>>>(n, nq, d_det, d_tol, d_cond, part.get());
        SKG_LAUNCH_CHECK("geom_diag");
        k_geom_diag_final<<<1, kDiagThreads, 0, s>>>(parts, part.get(), part.get() + parts);
        SKG_LAUNCH_CHECK("geom_diag_final");
        GeomDiag r;
        SKG_CUDA(cudaMemcpyAsync(&r, part.get() + parts, sizeof(r), cudaMemcpyDeviceToHost, s));
        SKG_CUDA(cudaStreamSynchronize(s));
        h_values[0] = r.det_min;
        h_values[1] = r.det_max;
        h_values[2] = r.scaled_min;
        h_values[3] = r.cond_max;
        h_indices[0] = r.scaled_at;
        h_indices[1] = r.cond_at;
        h_indices[2] = r.negative;
    });
}

extern "C" int skg_tabulate_geometry(const double *d_p, int64_t npts, const int32_t *d_t, int32_t gnodes,
                                     int64_t ne, int32_t nq, int32_t nodes, const double *h_shape,
                                     const double *h_refgrad, const double *h_gshape, const double *h_grefgrad,
                                     const double *h_w, double *d_shape, double *d_grad, double *d_dx,
                                     double *d_x, double *d_det, double *d_tol, double *d_cond, int64_t *h_bad,
                                     void *stream) {
    return guarded([&] {
        require(nq > 0 && nodes > 0 && gnodes > 0 && ne >= 0, "invalid basis geometry sizes");
        require(h_shape && h_refgrad && h_gshape && h_grefgrad && h_w, "reference tables are NULL");
        require(ne == 0 || (d_p && d_t), "mesh arrays are NULL");
        if (h_bad) { h_bad[0] = -1; h_bad[1] = -1; h_bad[2] = 0; }
        cudaStream_t s = as_stream(stream);
        const int total = nq * nodes * 4 + nq * gnodes * 4 + nq;
        require(total * 8 <= 200 * 1024, "quadrature tables exceed shared memory");
        std::vector<double> tables;
        tables.reserve(total);
        tables.insert(tables.end(), h_shape, h_shape + nq * nodes);
        tables.insert(tables.end(), h_refgrad, h_refgrad + nq * nodes * 3);
        tables.insert(tables.end(), h_gshape, h_gshape + nq * gnodes);
        tables.insert(tables.end(), h_grefgrad, h_grefgrad + nq * gnodes * 3);
        tables.insert(tables.end(), h_w, h_w + nq);
        DevBuf<double> dtab(total, s);
        SKG_CUDA(cudaMemcpyAsync(dtab.get(), tables.data(), total * 8, cudaMemcpyHostToDevice, s));
        DevBuf<double> det_tmp, tol_tmp;
        double *det = d_det, *tol = d_tol;
        if (!det) { det_tmp = DevBuf<double>((size_t)ne * nq, s); det = det_tmp.get(); }
        if (!tol) { tol_tmp = DevBuf<double>((size_t)ne * nq, s); tol = tol_tmp.get(); }
        DevBuf<int32_t> oob(1, s);
        DevBuf<unsigned long long> bad(1, s);
        SKG_CUDA(cudaMemsetAsync(oob.get(), 0, 4, s));
        SKG_CUDA(cudaMemsetAsync(bad.get(), 0xff, 8, s));
        const size_t smem = (size_t)total * 8;
        if (smem > 48 * 1024)
            SKG_CUDA(cudaFuncSetAttribute(k_tabulate, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        if (ne) {
            k_tabulate<<<grid_for(ne * nq, 128), 128, smem, s>>>(ne, nq, nodes, gnodes, d_p, npts, d_t, dtab.get(),
                                                                  d_shape, d_grad, d_dx, d_x, det, tol, d_cond,
                                                                  oob.get());
            SKG_LAUNCH_CHECK("tabulate_geometry");
            k_validate<<<grid_for(ne, 128), 128, 0, s>>>(ne, nq, det, tol, bad.get());
            SKG_LAUNCH_CHECK("validate_geometry");
        }
        int32_t h_oob = 0;
        unsigned long long h_first = ~0ull;
        SKG_CUDA(cudaMemcpyAsync(&h_oob, oob.get(), 4, cudaMemcpyDeviceToHost, s));
        SKG_CUDA(cudaMemcpyAsync(&h_first, bad.get(), 8, cudaMemcpyDeviceToHost, s));
        SKG_CUDA(cudaStreamSynchronize(s));
        require(!h_oob, "connectivity index is out of bounds", SKG_ERANGE);
        if (h_first != ~0ull) {
            const int64_t e = (int64_t)h_first;
            std::vector<double> dd(nq), tt(nq);
            SKG_CUDA(cudaMemcpy(dd.data(), det + e * nq, nq * 8, cudaMemcpyDeviceToHost));
            SKG_CUDA(cudaMemcpy(tt.data(), tol + e * nq, nq * 8, cudaMemcpyDeviceToHost));
            int qbad = -1, reason = 0;
            for (int q = 0; q < nq && qbad < 0; ++q)
                if (!(std::isfinite(dd[q]) && std::isfinite(tt[q]) && std::fabs(dd[q]) > tt[q])) { qbad = q; reason = 1; }
            if (qbad < 0) {
                const bool neg = dd[0] < 0.;
                for (int q = 1; q < nq && qbad < 0; ++q)
                    if ((dd[q] < 0.) != neg) { qbad = q; reason = 2; }
            }
            if (h_bad) { h_bad[0] = e; h_bad[1] = qbad; h_bad[2] = reason; }
            std::ostringstream m;
            m << "invalid element geometry: cell=" << e << ", quadrature_point=" << qbad << std::scientific
              << std::setprecision(17) << ", determinant=" << dd[qbad] << ", tolerance=" << tt[qbad]
              << (reason == 1 ? ", reason=near_singular_or_non_finite" : ", reason=orientation_change");
            fail(SKG_EGEOM, m.str());
        }
    });
}
