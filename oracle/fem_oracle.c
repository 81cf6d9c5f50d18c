/*
 * CPU oracle for the finite-element assembly hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C, the algorithms of
 * the reference package (scikit-fem-native, `skfemntv` 0.3.1) that the GPU
 * backend replaces.  It is used by the test-suite as the checker, by
 * `__graft_entry__.smoke()` as the checker, and by `bench.py` as the timed CPU
 * baseline.  The GPU product path never calls into it.
 *
 * Every function cites the reference source it follows (paths relative to
 * the reference project root).  The restatement keeps the reference's
 * summation order wherever the reference's serial path has one, so the
 * single-threaded oracle reproduces the reference's floating-point results
 * bit for bit (checked against fixtures generated by the reference itself).
 *
 * Threading follows the reference's runtime: colored element sets processed
 * one color after another (cpp/src/assembly/bilinear_form_assembler.cpp:62-70)
 * with an OpenMP parallel-for inside each color.
 */
#include <math.h>
#include <float.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define FO_OK 0
#define FO_EINVAL 1
#define FO_ENOMEM 2
#define FO_EGEOM 3

static int fo_threads(int requested) {
#ifdef _OPENMP
    if (requested <= 0) return 1;
    return requested;
#else
    (void)requested;
    return 1;
#endif
}

int fo_max_threads(void) {
#ifdef _OPENMP
    return omp_get_num_procs();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* Geometry: cpp/src/assembly/basis_geometry.cpp:18-47 (det / cofactor inverse)
 * and 49-209 (per (e,q) Jacobian, tolerance, inverse, condition number, dx,
 * physical gradients, physical points, then serial validation).            */

static double fo_det(const double *m, int dim) {
    if (dim == 2) return m[0] * m[3] - m[1] * m[2];
    return m[0] * (m[4] * m[8] - m[5] * m[7]) -
           m[1] * (m[3] * m[8] - m[5] * m[6]) +
           m[2] * (m[3] * m[7] - m[4] * m[6]);
}

static void fo_inverse(const double *m, double *r, int dim) {
    const double d = fo_det(m, dim);
    if (dim == 2) {
        r[0] = m[3] / d; r[1] = -m[1] / d; r[2] = -m[2] / d; r[3] = m[0] / d;
        return;
    }
    r[0] = (m[4] * m[8] - m[5] * m[7]) / d;
    r[1] = (m[2] * m[7] - m[1] * m[8]) / d;
    r[2] = (m[1] * m[5] - m[2] * m[4]) / d;
    r[3] = (m[5] * m[6] - m[3] * m[8]) / d;
    r[4] = (m[0] * m[8] - m[2] * m[6]) / d;
    r[5] = (m[2] * m[3] - m[0] * m[5]) / d;
    r[6] = (m[3] * m[7] - m[4] * m[6]) / d;
    r[7] = (m[1] * m[6] - m[0] * m[7]) / d;
    r[8] = (m[0] * m[4] - m[1] * m[3]) / d;
}

/* bad_reason: 0 none, 1 near_singular_or_non_finite, 2 orientation_change,
 * 3 connectivity out of bounds.  Outputs at invalid points are left as the
 * caller initialised them (the reference leaves them unset and raises). */
int fo_tabulate_geometry(int dim, int64_t npts, const double *p,
                         int64_t gnodes, int64_t ne, const int64_t *t,
                         int64_t nq, int64_t nodes, const double *shape,
                         const double *refgrad, const double *gshape,
                         const double *grefgrad, const double *w,
                         double *o_shape, double *o_grad, double *o_dx,
                         double *o_x, double *o_det, double *o_tol,
                         double *o_cond, int threads, int64_t *bad_cell,
                         int64_t *bad_q, int *bad_reason) {
    int oob = 0;
    *bad_cell = -1; *bad_q = -1; *bad_reason = 0;
    if (dim != 2 && dim != 3) return FO_EINVAL;
#pragma omp parallel for num_threads(fo_threads(threads)) schedule(static) reduction(|:oob)
    for (int64_t e = 0; e < ne; ++e) {
        for (int64_t q = 0; q < nq; ++q) {
            double J[9] = {0}, Ji[9] = {0}, x[3] = {0};
            for (int64_t a = 0; a < gnodes; ++a) {
                const int64_t v = t[a * ne + e];
                if (v < 0 || v >= npts) { oob = 1; continue; }
                for (int i = 0; i < dim; ++i) {
                    const double c = p[i * npts + v];
                    x[i] += gshape[q * gnodes + a] * c;
                    for (int j = 0; j < dim; ++j)
                        J[i * dim + j] += c * grefgrad[(q * gnodes + a) * dim + j];
                }
            }
            for (int i = 0; i < dim; ++i) o_x[(e * nq + q) * dim + i] = x[i];
            double s = 0.;
            for (int i = 0; i < dim * dim; ++i) s = fmax(s, fabs(J[i]));
            const double sp = dim == 2 ? s * s : s * s * s;
            const double tol = 64. * DBL_EPSILON * sp;
            const double det = fo_det(J, dim);
            o_det[e * nq + q] = det;
            o_tol[e * nq + q] = tol;
            if (!isfinite(det) || !isfinite(tol) || !(fabs(det) > tol)) continue;
            fo_inverse(J, Ji, dim);
            double jn = 0., in = 0.;
            for (int i = 0; i < dim * dim; ++i) { jn += J[i] * J[i]; in += Ji[i] * Ji[i]; }
            o_cond[e * nq + q] = sqrt(jn * in);
            o_dx[e * nq + q] = fabs(det) * w[q];
            for (int64_t a = 0; a < nodes; ++a) {
                o_shape[(e * nq + q) * nodes + a] = shape[q * nodes + a];
                for (int j = 0; j < dim; ++j) {
                    double g = 0.;
                    for (int k = 0; k < dim; ++k)
                        g += refgrad[(q * nodes + a) * dim + k] * Ji[k * dim + j];
                    o_grad[((e * nq + q) * nodes + a) * dim + j] = g;
                }
            }
        }
    }
    if (oob) { *bad_reason = 3; return FO_EINVAL; }
    /* serial validation in element order: basis_geometry.cpp:178-205 */
    for (int64_t e = 0; e < ne; ++e) {
        for (int64_t q = 0; q < nq; ++q) {
            const double det = o_det[e * nq + q], tol = o_tol[e * nq + q];
            if (isfinite(det) && isfinite(tol) && fabs(det) > tol) continue;
            *bad_cell = e; *bad_q = q; *bad_reason = 1;
            return FO_EGEOM;
        }
        const int neg = o_det[e * nq] < 0.;
        for (int64_t q = 1; q < nq; ++q) {
            if ((o_det[e * nq + q] < 0.) == neg) continue;
            *bad_cell = e; *bad_q = q; *bad_reason = 2;
            return FO_EGEOM;
        }
    }
    return FO_OK;
}

/* ------------------------------------------------------------------------ */
/* CSR pattern + scatter map + greedy coloring.
 * Pattern: per-row sorted unique columns, bilinear_form_assembler.cpp:111-116
 * (same rule in cross_bilinear_assembler.cpp:311-320 and
 * edge_topology.cpp:86-154).  Scatter map by lower_bound: 117-120.
 * Greedy first-fit coloring over element order: 121-140.                    */

typedef struct fo_pattern {
    int64_t ne, lr, lc, nrows, nnz;
    int64_t *indptr, *indices, *scatter; /* scatter (ne, lr, lc) absolute slots */
    int64_t ncolors;
    int64_t *color_ptr, *color_elems;    /* elements grouped by color, in order */
} fo_pattern;

static int cmp_i64(const void *a, const void *b) {
    const int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
    return (x > y) - (x < y);
}

static int64_t lower_bound_i64(const int64_t *b, int64_t n, int64_t key) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        const int64_t mid = lo + (hi - lo) / 2;
        if (b[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

void fo_pattern_free(fo_pattern *h) {
    if (!h) return;
    free(h->indptr); free(h->indices); free(h->scatter);
    free(h->color_ptr); free(h->color_elems);
    free(h);
}

/* row_dofs (ne, lr) and col_dofs (ne, lc), element-major (the reference's
 * `dofs (E, nodes, comp)` flattened).  nrows = max(row_dofs)+1 unless given. */
fo_pattern *fo_pattern_build(const int64_t *row_dofs, const int64_t *col_dofs,
                             int64_t ne, int64_t lr, int64_t lc, int64_t nrows,
                             int with_coloring) {
    fo_pattern *h = (fo_pattern *)calloc(1, sizeof(fo_pattern));
    if (!h) return NULL;
    h->ne = ne; h->lr = lr; h->lc = lc;
    if (nrows < 0) {
        nrows = 0;
        for (int64_t i = 0; i < ne * lr; ++i) if (row_dofs[i] + 1 > nrows) nrows = row_dofs[i] + 1;
    }
    h->nrows = nrows;
    /* bucket all (row, col) candidates by row: counting sort */
    int64_t *cnt = (int64_t *)calloc((size_t)nrows + 1, sizeof(int64_t));
    const int64_t total = ne * lr * lc;
    int64_t *cand = (int64_t *)malloc((size_t)(total > 0 ? total : 1) * sizeof(int64_t));
    h->indptr = (int64_t *)calloc((size_t)nrows + 1, sizeof(int64_t));
    if (!cnt || !cand || !h->indptr) { free(cnt); free(cand); fo_pattern_free(h); return NULL; }
    for (int64_t e = 0; e < ne; ++e)
        for (int64_t i = 0; i < lr; ++i) cnt[row_dofs[e * lr + i] + 1] += lc;
    for (int64_t r = 0; r < nrows; ++r) cnt[r + 1] += cnt[r];
    int64_t *cur = (int64_t *)malloc((size_t)(nrows > 0 ? nrows : 1) * sizeof(int64_t));
    memcpy(cur, cnt, (size_t)nrows * sizeof(int64_t));
    for (int64_t e = 0; e < ne; ++e)
        for (int64_t i = 0; i < lr; ++i) {
            const int64_t r = row_dofs[e * lr + i];
            for (int64_t j = 0; j < lc; ++j) cand[cur[r]++] = col_dofs[e * lc + j];
        }
    free(cur);
    int64_t nnz = 0;
    for (int64_t r = 0; r < nrows; ++r) {
        int64_t *x = cand + cnt[r];
        const int64_t n = cnt[r + 1] - cnt[r];
        qsort(x, (size_t)n, sizeof(int64_t), cmp_i64);
        int64_t u = 0;
        for (int64_t k = 0; k < n; ++k)
            if (u == 0 || x[k] != x[u - 1]) x[u++] = x[k];
        h->indptr[r + 1] = h->indptr[r] + u;
        nnz += u;
    }
    h->nnz = nnz;
    h->indices = (int64_t *)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(int64_t));
    for (int64_t r = 0; r < nrows; ++r)
        memcpy(h->indices + h->indptr[r], cand + cnt[r],
               (size_t)(h->indptr[r + 1] - h->indptr[r]) * sizeof(int64_t));
    free(cand); free(cnt);
    h->scatter = (int64_t *)malloc((size_t)(total > 0 ? total : 1) * sizeof(int64_t));
    for (int64_t e = 0; e < ne; ++e)
        for (int64_t i = 0; i < lr; ++i) {
            const int64_t r = row_dofs[e * lr + i];
            const int64_t *b = h->indices + h->indptr[r];
            const int64_t n = h->indptr[r + 1] - h->indptr[r];
            for (int64_t j = 0; j < lc; ++j)
                h->scatter[(e * lr + i) * lc + j] =
                    h->indptr[r] + lower_bound_i64(b, n, col_dofs[e * lc + j]);
        }
    if (with_coloring) {
        /* first-fit greedy over elements in order; a color is blocked when
         * any of the element's row dofs already carries it */
        int64_t *elem_color = (int64_t *)malloc((size_t)(ne > 0 ? ne : 1) * sizeof(int64_t));
        int64_t *dptr = (int64_t *)calloc((size_t)nrows + 1, sizeof(int64_t));
        for (int64_t e = 0; e < ne; ++e)
            for (int64_t i = 0; i < lr; ++i) dptr[row_dofs[e * lr + i] + 1]++;
        for (int64_t r = 0; r < nrows; ++r) dptr[r + 1] += dptr[r];
        int64_t *dcol = (int64_t *)malloc((size_t)(dptr[nrows] > 0 ? dptr[nrows] : 1) * sizeof(int64_t));
        int64_t *dlen = (int64_t *)calloc((size_t)nrows + 1, sizeof(int64_t));
        int64_t cap = 64, ncol = 0;
        int64_t *mark = (int64_t *)calloc((size_t)cap, sizeof(int64_t));
        for (int64_t e = 0; e < ne; ++e) {
            const int64_t gen = e + 1;
            for (int64_t i = 0; i < lr; ++i) {
                const int64_t r = row_dofs[e * lr + i];
                for (int64_t k = 0; k < dlen[r]; ++k) mark[dcol[dptr[r] + k]] = gen;
            }
            int64_t c = 0;
            while (c < ncol && mark[c] == gen) ++c;
            if (c == ncol) {
                ++ncol;
                if (ncol > cap) {
                    mark = (int64_t *)realloc(mark, (size_t)(2 * cap) * sizeof(int64_t));
                    memset(mark + cap, 0, (size_t)cap * sizeof(int64_t));
                    cap *= 2;
                }
            }
            elem_color[e] = c;
            for (int64_t i = 0; i < lr; ++i) {
                const int64_t r = row_dofs[e * lr + i];
                dcol[dptr[r] + dlen[r]++] = c;
            }
        }
        h->ncolors = ncol;
        h->color_ptr = (int64_t *)calloc((size_t)ncol + 1, sizeof(int64_t));
        h->color_elems = (int64_t *)malloc((size_t)(ne > 0 ? ne : 1) * sizeof(int64_t));
        for (int64_t e = 0; e < ne; ++e) h->color_ptr[elem_color[e] + 1]++;
        for (int64_t c = 0; c < ncol; ++c) h->color_ptr[c + 1] += h->color_ptr[c];
        int64_t *fill = (int64_t *)malloc((size_t)(ncol > 0 ? ncol : 1) * sizeof(int64_t));
        memcpy(fill, h->color_ptr, (size_t)ncol * sizeof(int64_t));
        for (int64_t e = 0; e < ne; ++e) h->color_elems[fill[elem_color[e]]++] = e;
        free(fill); free(mark); free(dlen); free(dcol); free(dptr); free(elem_color);
    }
    return h;
}

int64_t fo_pattern_nnz(const fo_pattern *h) { return h->nnz; }
int64_t fo_pattern_nrows(const fo_pattern *h) { return h->nrows; }
int64_t fo_pattern_ncolors(const fo_pattern *h) { return h->ncolors; }

void fo_pattern_copy(const fo_pattern *h, int64_t *indptr, int64_t *indices, int64_t *scatter) {
    if (indptr) memcpy(indptr, h->indptr, (size_t)(h->nrows + 1) * sizeof(int64_t));
    if (indices) memcpy(indices, h->indices, (size_t)h->nnz * sizeof(int64_t));
    if (scatter) memcpy(scatter, h->scatter, (size_t)(h->ne * h->lr * h->lc) * sizeof(int64_t));
}

/* ------------------------------------------------------------------------ */
/* Nodal bilinear assembly: bilinear_form_assembler.cpp:79-105, per element
 * q -> a -> b -> c -> d straight into the CSR slot.                         */

typedef struct {
    int64_t nodes, comp, nq, dim, L;
    const double *shape, *grad, *w, *value, *gradient, *symgrad, *div;
    const int64_t *scatter;
    double *values;
} fo_bil_args;

static void fo_bil_element(const fo_bil_args *A, int64_t e) {
    const int64_t n = A->nodes, C = A->comp, D = A->dim, L = A->L;
    for (int64_t q = 0; q < A->nq; ++q) {
        const int64_t eq = e * A->nq + q;
        for (int64_t a = 0; a < n; ++a)
            for (int64_t b = 0; b < n; ++b) {
                double diag = 0.;
                if (A->value) diag += A->value[eq] * A->shape[eq * n + a] * A->shape[eq * n + b];
                if (A->gradient)
                    for (int64_t j = 0; j < D; ++j)
                        diag += A->gradient[eq] * A->grad[(eq * n + a) * D + j] *
                                A->grad[(eq * n + b) * D + j];
                for (int64_t c = 0; c < C; ++c)
                    for (int64_t d = 0; d < C; ++d) {
                        double entry = (c == d ? diag : 0.);
                        if (A->symgrad) {
                            double s = A->grad[(eq * n + a) * D + d] * A->grad[(eq * n + b) * D + c];
                            if (c == d)
                                for (int64_t j = 0; j < D; ++j)
                                    s += A->grad[(eq * n + a) * D + j] * A->grad[(eq * n + b) * D + j];
                            entry += .5 * A->symgrad[eq] * s;
                        }
                        if (A->div)
                            entry += A->div[eq] * A->grad[(eq * n + a) * D + c] *
                                     A->grad[(eq * n + b) * D + d];
                        const int64_t i = a * C + c, k = b * C + d;
                        A->values[A->scatter[(e * L + i) * L + k]] += entry * A->w[eq];
                    }
            }
    }
}

int fo_bilinear_assemble(const fo_pattern *h, int64_t nodes, int64_t comp, int64_t nq,
                         int64_t dim, const double *shape, const double *grad,
                         const double *w, const double *value, const double *gradient,
                         const double *symgrad, const double *div, int threads,
                         double *values) {
    if (!value && !gradient && !symgrad && !div) return FO_EINVAL;
    fo_bil_args A = {nodes, comp, nq, dim, nodes * comp, shape, grad, w, value, gradient,
                     symgrad, div, h->scatter, values};
    memset(values, 0, (size_t)h->nnz * sizeof(double));
    const int nt = fo_threads(threads);
    if (nt <= 1 || !h->color_ptr) {
        for (int64_t e = 0; e < h->ne; ++e) fo_bil_element(&A, e);
        return FO_OK;
    }
    for (int64_t c = 0; c < h->ncolors; ++c) {
        const int64_t b = h->color_ptr[c], en = h->color_ptr[c + 1];
#pragma omp parallel for num_threads(nt) schedule(static)
        for (int64_t k = b; k < en; ++k) fo_bil_element(&A, h->color_elems[k]);
    }
    return FO_OK;
}

/* ------------------------------------------------------------------------ */
/* Rectangular (test x trial) assembly with scalar or full tensor coefficient:
 * cross_bilinear_assembler.cpp:207-247 with contract_cross_basis /
 * contract_scalar_cross_basis (cpp/include/native_fem/cross_contraction.hpp
 * 20-98).  row_kind/col_kind: 0 value, 1 gradient.  tensor coefficient layout
 * (E,Q,rc,[rd],cc,[cd]) C-contiguous; scalar coefficient (E,Q) or NULL = 1. */

typedef struct {
    int64_t rn, cn, rc, cc, nq, rdim, cdim, rl, cl;
    int rkind, ckind, tensor;
    const double *rshape, *cshape, *rgrad, *cgrad, *w, *coef;
    const int64_t *scatter;
    double *values;
} fo_cross_args;

static inline double fo_basis_at(const double *shape, const double *grad, int kind,
                                 int64_t nodes, int64_t dim, int64_t eq, int64_t a, int64_t i) {
    if (kind == 0) return shape[eq * nodes + a];
    return grad[(eq * nodes + a) * dim + i];
}

static inline double fo_coef_at(const fo_cross_args *A, int64_t eq, int64_t r, int64_t i,
                                int64_t c, int64_t j) {
    if (!A->tensor) {
        if (r != c) return 0.;
        if (A->rkind == 1 && i != j) return 0.;
        return A->coef ? A->coef[eq] : 1.;
    }
    int64_t idx = eq;
    idx = idx * A->rc + r;
    if (A->rkind == 1) idx = idx * A->rdim + i;
    idx = idx * A->cc + c;
    if (A->ckind == 1) idx = idx * A->cdim + j;
    return A->coef[idx];
}

static void fo_cross_entity(const fo_cross_args *A, int64_t e) {
    const int64_t rdir = A->rkind == 1 ? A->rdim : 1, cdir = A->ckind == 1 ? A->cdim : 1;
    for (int64_t q = 0; q < A->nq; ++q) {
        const int64_t eq = e * A->nq + q;
        const double scale = A->w[eq];
        for (int64_t a = 0; a < A->rn; ++a)
            for (int64_t b = 0; b < A->cn; ++b) {
                if (!A->tensor) {
                    const double material = A->coef ? A->coef[eq] : 1.;
                    double s;
                    if (A->rkind == 0) {
                        s = A->rshape[eq * A->rn + a] * A->cshape[eq * A->cn + b];
                    } else {
                        s = 0.;
                        for (int64_t d = 0; d < A->rdim; ++d)
                            s += A->rgrad[(eq * A->rn + a) * A->rdim + d] *
                                 A->cgrad[(eq * A->cn + b) * A->cdim + d];
                    }
                    const double entry = scale * material * s;
                    for (int64_t r = 0; r < A->rc; ++r) {
                        const int64_t i = a * A->rc + r, j = b * A->cc + r;
                        A->values[A->scatter[(e * A->rl + i) * A->cl + j]] += entry;
                    }
                } else {
                    for (int64_t r = 0; r < A->rc; ++r)
                        for (int64_t c = 0; c < A->cc; ++c) {
                            double res = 0.;
                            for (int64_t i = 0; i < rdir; ++i)
                                for (int64_t j = 0; j < cdir; ++j)
                                    res += fo_basis_at(A->rshape, A->rgrad, A->rkind, A->rn, A->rdim, eq, a, i) *
                                           fo_coef_at(A, eq, r, i, c, j) *
                                           fo_basis_at(A->cshape, A->cgrad, A->ckind, A->cn, A->cdim, eq, b, j);
                            const int64_t ii = a * A->rc + r, jj = b * A->cc + c;
                            A->values[A->scatter[(e * A->rl + ii) * A->cl + jj]] += scale * res;
                        }
                }
            }
    }
}

int fo_cross_assemble(const fo_pattern *h, int64_t rn, int64_t cn, int64_t rc, int64_t cc,
                      int64_t nq, int64_t rdim, int64_t cdim, const double *rshape,
                      const double *cshape, const double *rgrad, const double *cgrad,
                      const double *w, const double *coef, int tensor, int rkind, int ckind,
                      int threads, double *values) {
    fo_cross_args A = {rn, cn, rc, cc, nq, rdim, cdim, rn * rc, cn * cc, rkind, ckind, tensor,
                       rshape, cshape, rgrad, cgrad, w, coef, h->scatter, values};
    if (tensor && !coef) return FO_EINVAL;
    memset(values, 0, (size_t)h->nnz * sizeof(double));
    const int nt = fo_threads(threads);
    if (nt <= 1 || !h->color_ptr) {
        for (int64_t e = 0; e < h->ne; ++e) fo_cross_entity(&A, e);
        return FO_OK;
    }
    for (int64_t c = 0; c < h->ncolors; ++c) {
        const int64_t b = h->color_ptr[c], en = h->color_ptr[c + 1];
#pragma omp parallel for num_threads(nt) schedule(static)
        for (int64_t k = b; k < en; ++k) fo_cross_entity(&A, h->color_elems[k]);
    }
    return FO_OK;
}

/* ------------------------------------------------------------------------ */
/* Linear form f.v + G:grad v: linear_form_assembler.cpp:41-154.  The serial
 * path only (per-thread private vectors + reduction, 71-91, give the same sum
 * with a different association).  value: (E,Q,C) or constant (C); gradient:
 * (E,Q,C,D) or constant (C,D).                                              */
int fo_linear_assemble(const int64_t *dofs, int64_t ne, int64_t nodes, int64_t comp,
                       int64_t nq, int64_t dim, const double *shape, const double *grad,
                       const double *w, const double *value, int value_const,
                       const double *gradient, int grad_const, int64_t ndofs,
                       double *out) {
    if (!value && !gradient) return FO_EINVAL;
    memset(out, 0, (size_t)ndofs * sizeof(double));
    if ((!value || value_const) && (!gradient || grad_const)) {
        for (int64_t e = 0; e < ne; ++e)
            for (int64_t a = 0; a < nodes; ++a)
                for (int64_t c = 0; c < comp; ++c) {
                    double local = 0.;
                    for (int64_t q = 0; q < nq; ++q) {
                        double contrib = 0.;
                        if (value) contrib += shape[(e * nq + q) * nodes + a] * value[c];
                        if (gradient)
                            for (int64_t j = 0; j < dim; ++j)
                                contrib += grad[((e * nq + q) * nodes + a) * dim + j] * gradient[c * dim + j];
                        local += w[e * nq + q] * contrib;
                    }
                    out[dofs[(e * nodes + a) * comp + c]] += local;
                }
        return FO_OK;
    }
    for (int64_t e = 0; e < ne; ++e)
        for (int64_t q = 0; q < nq; ++q)
            for (int64_t a = 0; a < nodes; ++a)
                for (int64_t c = 0; c < comp; ++c) {
                    double contrib = 0.;
                    if (value)
                        contrib += shape[(e * nq + q) * nodes + a] *
                                   value[value_const ? c : (e * nq + q) * comp + c];
                    if (gradient)
                        for (int64_t j = 0; j < dim; ++j)
                            contrib += grad[((e * nq + q) * nodes + a) * dim + j] *
                                       gradient[grad_const ? c * dim + j : ((e * nq + q) * comp + c) * dim + j];
                    out[dofs[(e * nodes + a) * comp + c]] += w[e * nq + q] * contrib;
                }
    return FO_OK;
}

/* ------------------------------------------------------------------------ */
/* Oriented edge topology: cpp/src/assembly/edge_topology.cpp:30-84.
 * First-seen global edge ids in cell-major, local-edge-major order; edge key
 * is the ascending vertex pair; sign +1 when the local edge's first vertex is
 * the smaller one.  Open-addressing hash table (the reference uses an
 * unordered_map; only the first-seen numbering matters).                    */

static const int FO_TET_EDGES[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};

static uint64_t fo_mix(uint64_t x) {
    x ^= x >> 33; x *= 0xff51afd7ed558ccdULL; x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL; x ^= x >> 33;
    return x;
}

/* corners x ne connectivity (node-major like mesh.t).  edges_out must hold
 * 2 x (ne*nedge) entries (first row = smaller vertex, second = larger, packed
 * with stride ne*nedge); the number of edges is returned in *n_edges.
 * Returns FO_EINVAL and *bad_cell when a cell repeats a corner vertex.      */
int fo_edge_topology(const int64_t *t, int64_t ne, int dim, int64_t *edges_out,
                     int64_t *elem_edges, int8_t *signs, int64_t *n_edges,
                     int64_t *bad_cell) {
    const int corners = dim == 2 ? 3 : 4, nedge = dim == 2 ? 3 : 6;
    *bad_cell = -1;
    const int64_t cap_items = ne * nedge;
    int64_t cap = 16;
    while (cap < 2 * cap_items) cap <<= 1;
    int64_t *keys_a = (int64_t *)malloc((size_t)cap * sizeof(int64_t));
    int64_t *keys_b = (int64_t *)malloc((size_t)cap * sizeof(int64_t));
    int64_t *ids = (int64_t *)malloc((size_t)cap * sizeof(int64_t));
    if (!keys_a || !keys_b || !ids) { free(keys_a); free(keys_b); free(ids); return FO_ENOMEM; }
    for (int64_t i = 0; i < cap; ++i) ids[i] = -1;
    int64_t count = 0;
    const int64_t stride = cap_items;
    for (int64_t cell = 0; cell < ne; ++cell) {
        for (int f = 0; f < corners; ++f)
            for (int s = f + 1; s < corners; ++s)
                if (t[f * ne + cell] == t[s * ne + cell]) {
                    *bad_cell = cell;
                    free(keys_a); free(keys_b); free(ids);
                    return FO_EINVAL;
                }
        for (int l = 0; l < nedge; ++l) {
            const int64_t v0 = t[FO_TET_EDGES[l][0] * ne + cell];
            const int64_t v1 = t[FO_TET_EDGES[l][1] * ne + cell];
            const int64_t lo = v0 < v1 ? v0 : v1, hi = v0 < v1 ? v1 : v0;
            uint64_t hsh = fo_mix((uint64_t)lo * 0x9E3779B97F4A7C15ULL ^ (uint64_t)hi) & (uint64_t)(cap - 1);
            int64_t id;
            for (;;) {
                if (ids[hsh] < 0) {
                    ids[hsh] = count; keys_a[hsh] = lo; keys_b[hsh] = hi;
                    edges_out[count] = lo; edges_out[stride + count] = hi;
                    id = count++;
                    break;
                }
                if (keys_a[hsh] == lo && keys_b[hsh] == hi) { id = ids[hsh]; break; }
                hsh = (hsh + 1) & (uint64_t)(cap - 1);
            }
            elem_edges[l * ne + cell] = id;
            signs[l * ne + cell] = (int8_t)(v0 == lo ? 1 : -1);
        }
    }
    *n_edges = count;
    free(keys_a); free(keys_b); free(ids);
    return FO_OK;
}

/* ------------------------------------------------------------------------ */
/* TetN1 local matrices: edge_topology.cpp:156-233.  values/curls (E,6,3,Q),
 * dx/mass/curl (E,Q), out (E,6,6): sum over q of dx*(mass v.v + curl c.c). */
int fo_integrate_tet_n1(const double *values, const double *curls, const double *dx,
                        const double *mass, const double *curlc, int64_t ne, int64_t nq,
                        int include_mass, int include_curl, int threads, double *out) {
    const int64_t L = 6, C = 3;
#pragma omp parallel for num_threads(fo_threads(threads)) schedule(static)
    for (int64_t cell = 0; cell < ne; ++cell)
        for (int64_t r = 0; r < L; ++r)
            for (int64_t c = 0; c < L; ++c) {
                double res = 0.;
                for (int64_t p = 0; p < nq; ++p) {
                    double vd = 0., cd = 0.;
                    for (int64_t k = 0; k < C; ++k) {
                        const int64_t ro = ((cell * L + r) * C + k) * nq + p;
                        const int64_t co = ((cell * L + c) * C + k) * nq + p;
                        if (include_mass) vd += values[ro] * values[co];
                        if (include_curl) cd += curls[ro] * curls[co];
                    }
                    const int64_t o = cell * nq + p;
                    res += dx[o] * (mass[o] * vd + curlc[o] * cd);
                }
                out[(cell * L + r) * L + c] = res;
            }
    return FO_OK;
}

/* np.add.at(data, scatter.ravel(), elements.ravel()) in index order:
 * python/skfemntv/hcurl_assembler.py:94-97. */
void fo_add_at(double *data, int64_t ndata, const int64_t *idx, const double *vals, int64_t n) {
    memset(data, 0, (size_t)ndata * sizeof(double));
    for (int64_t i = 0; i < n; ++i) data[idx[i]] += vals[i];
}
