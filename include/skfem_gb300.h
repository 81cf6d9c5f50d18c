/*
 * skfem_gb300.h -- C ABI of the GB300 finite-element assembly backend.
 *
 * A drop-in for the native layer (`_skfn`, pybind11) that scikit-fem-native's
 * Python wrappers call on the matrix-assembly path.  Every entry point below
 * names the reference interface it replaces (paths relative to the reference
 * project root).
 *
 * Conventions
 *  - Plain C: pointers and sizes only.  `d_` arguments are device pointers
 *    (CUDA global memory), `h_` arguments host pointers.
 *  - Every call returns an int status (SKG_OK = 0); the message of the last
 *    failure on the calling thread is available from skg_last_error().  No
 *    C++ exception crosses this boundary.
 *  - Work is enqueued on the caller's stream (`stream` is a cudaStream_t,
 *    NULL = legacy default stream).  Calls documented as "synchronous" wait
 *    for their own work before returning (setup paths that report data-
 *    dependent errors).
 *  - Outputs are caller-owned.  Handles (skg_pattern) own their device
 *    memory until destroyed.
 *  - Connectivity is int32 on the device; sizes are int64.
 *  - Arrays use the reference's own layouts: mesh coordinates (3, npts),
 *    mesh connectivity (nodes, elements) node-major like `mesh.t`, per-point
 *    coefficients (elements, points) like `basis.dx`.
 *  - Element-matrix sums into CSR slots are made in a fixed order (element
 *    index ascending, then local index), so repeated calls give identical
 *    bits.
 */
#ifndef SKFEM_GB300_H
#define SKFEM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SKG_OK 0
#define SKG_EINVAL 1    /* invalid argument / shape (the reference raises ValueError) */
#define SKG_ENOMEM 2    /* device allocation failed */
#define SKG_ECUDA 3     /* CUDA runtime error */
#define SKG_EGEOM 4     /* invalid element geometry (ValueError in the reference) */
#define SKG_ERANGE 5    /* index out of range (ValueError in the reference) */
#define SKG_EUNSUPPORTED 6

/* Precision of the element contraction. */
#define SKG_FP64 0          /* FP64 end to end */
#define SKG_SPLIT_FP32 1    /* FP32 hi+lo split products, FP32 accumulation; FP64-class geometry and slot sums */
#define SKG_FP64_EMULATED 2 /* FP64-accurate: double-float (FP32 pair) arithmetic throughout, exact FP64 output */

/* Library version (major*10000 + minor*100 + patch). */
int skg_version(void);

/* Message of the last failure on the calling thread ("" when none). */
const char *skg_last_error(void);

/* Measured FP64 FMA throughput of the current device (FMAs per second /
 * 1e9), from one full-grid launch of independent FMA chains timed with CUDA
 * events on the stream; the FP64 roof for reporting the FP64 passes.
 * Synchronous. */
int skg_fp64_fma_rate(double *h_gfma, void *stream);

/* 1 when kernels on the current device may read and write pageable host
 * memory directly (Grace-Blackwell: address translation over NVLink-C2C).
 * The host side then lets kernels read coefficients from, and write CSR
 * values to, host buffers without staging copies.  No counterpart in the
 * reference (CPU-only). */
int skg_device_pageable_access(int32_t *out);

/* ------------------------------------------------------------------ */
/* Sparsity pattern.                                                    */
/* Replaces the pattern build of BilinearFormAssembler                  */
/* (cpp/src/assembly/bilinear_form_assembler.cpp:111-120),              */
/* CrossBilinearAssembler (cpp/src/assembly/cross_bilinear_assembler.cpp */
/* :311-320) and build_edge_csr_pattern                                 */
/* (cpp/src/assembly/edge_topology.cpp:86-154): per-row sorted unique   */
/* columns, identical indptr/indices.  The handle also keeps, per row,  */
/* the (element, local row) incidences in ascending order, which fixes  */
/* the summation order of every assembly on this pattern.               */

typedef struct skg_pattern skg_pattern;

/* d_row_dofs (n_elements, row_local), d_col_dofs (n_elements, col_local),
 * element-major (the reference's `dofs (E, nodes, components)`).  n_rows /
 * n_cols: matrix shape (rows must exceed every row dof).  With d_col_dofs
 * NULL only the row incidence lists are built (nnz = 0): the handle then
 * serves vector (linear-form) assembly.  Synchronous. */
int skg_pattern_create(const int32_t *d_row_dofs, const int32_t *d_col_dofs,
                       int64_t n_elements, int32_t row_local, int32_t col_local,
                       int64_t n_rows, int64_t n_cols, void *stream,
                       skg_pattern **out);
int skg_pattern_destroy(skg_pattern *pattern);
/* nnz and shape of the pattern. */
int skg_pattern_info(const skg_pattern *pattern, int64_t *nnz, int64_t *n_rows,
                     int64_t *n_cols);
/* Longest row of a pattern with row groups (the fused row passes, which
 * write each CSR value exactly once), 0 when the pattern has none.  No
 * counterpart in the reference. */
int skg_pattern_row_groups(const skg_pattern *pattern, int32_t *max_row_len);
/* Copy the CSR structure out: d_indptr (n_rows+1) int64, d_indices (nnz) int32.
 * Either may be NULL.  (BilinearFormAssembler.indptr / .indices views.) */
int skg_pattern_export(const skg_pattern *pattern, int64_t *d_indptr,
                       int32_t *d_indices, void *stream);

/* ------------------------------------------------------------------ */
/* Geometry tabulation.                                                 */
/* Replaces tabulate_basis_geometry                                     */
/* (cpp/src/assembly/basis_geometry.cpp:49-209): per (element, point)   */
/* isoparametric Jacobian, scale-aware determinant tolerance, cofactor  */
/* inverse, condition number, dx = |det| w, physical gradients and      */
/* points, then the reference's validation (first failing element in    */
/* element order; near-singular before orientation change).             */
/* Tables (host, copied): shape (Q,nodes), refgrad (Q,nodes,3),         */
/* gshape (Q,gnodes), grefgrad (Q,gnodes,3), W (Q).  Output arrays      */
/* (device, any may be NULL): shape (E,Q,nodes), grad (E,Q,nodes,3),    */
/* dx (E,Q), x (E,Q,3), det, tol, cond (E,Q).  Synchronous; on a        */
/* validation failure returns SKG_EGEOM with h_bad = {cell, point,      */
/* reason (1 near_singular_or_non_finite, 2 orientation_change)} and    */
/* the message formatted as the reference's.                            */
int skg_tabulate_geometry(const double *d_p, int64_t npts, const int32_t *d_t,
                          int32_t gnodes, int64_t n_elements, int32_t nq,
                          int32_t nodes, const double *h_shape,
                          const double *h_refgrad, const double *h_gshape,
                          const double *h_grefgrad, const double *h_w,
                          double *d_shape, double *d_grad, double *d_dx,
                          double *d_x, double *d_det, double *d_tol,
                          double *d_cond, int64_t *h_bad, void *stream);

/* Geometry diagnostics of a tabulated basis in one device reduction:    */
/* replaces the host-side reductions of Basis._update_geometry_diagnostics */
/* (python/skfemntv/basis.py:2296-2356) over det, tol, cond (E,Q).      */
/* h_values = {min det, max det, min |det| / (tol / (64 eps)), max cond} */
/* h_indices = {flat index of that smallest scaled determinant, flat     */
/* index of the largest condition number (first occurrence each, as      */
/* numpy's argmin / argmax), elements whose first point has det < 0}.    */
/* Requires E, Q > 0.  Synchronous.                                      */
int skg_geometry_diagnostics(const double *d_det, const double *d_tol, const double *d_cond,
                             int64_t n_elements, int32_t nq, double *h_values,
                             int64_t *h_indices, void *stream);

/* ------------------------------------------------------------------ */
/* Nodal H1 bilinear assembly from tabulated geometry.                  */
/* Replaces BilinearFormAssembler.assemble                              */
/* (cpp/src/assembly/bilinear_form_assembler.cpp:39-105):               */
/*   K[a c, b d] += w (v N_a N_b + g grad N_a . grad N_b) delta_cd      */
/*                  + 1/2 s (...) + div (...)                            */
/* d_dofs (E, nodes*comp); shape (E,Q,nodes), grad (E,Q,nodes,3),       */
/* w (E,Q); coefficients (E,Q) or NULL (at least one required).         */
/* d_values (nnz) is overwritten.  d_scratch: NULL, or E*L*L doubles    */
/* (L = nodes*comp) for the element matrices.                            */
int skg_h1_assemble_tabulated(const skg_pattern *pattern, const int32_t *d_dofs,
                              int64_t n_elements, int32_t nodes, int32_t comp,
                              int32_t nq, const double *d_shape,
                              const double *d_grad, const double *d_w,
                              const double *d_value, const double *d_gradient,
                              const double *d_symgrad, const double *d_div,
                              double *d_values, double *d_scratch, void *stream);

/* Test x trial assembly with a full tensor coefficient on gradients.
 * Replaces CrossBilinearAssembler.assemble(coefficient, "gradient",
 * "gradient") (cpp/src/assembly/cross_bilinear_assembler.cpp:55-107,
 * 207-247; cpp/include/native_fem/cross_contraction.hpp:67-84) for one shared
 * basis: K[a r, b c] += w sum_ij gradN_a[i] C[e,q,r,i,c,j] gradN_b[j].
 * d_coef (E,Q,comp,3,comp,3). */
int skg_h1_assemble_tensor_tabulated(const skg_pattern *pattern,
                                     const int32_t *d_dofs, int64_t n_elements,
                                     int32_t nodes, int32_t comp, int32_t nq,
                                     const double *d_grad, const double *d_w,
                                     const double *d_coef, double *d_values,
                                     double *d_scratch, void *stream);
/* Cross-basis (test x trial) assembly with a caller-supplied contraction
 * tensor: NativeCrossBilinearForm.assemble_tensor(row_kind, column_kind, C)
 * and .assemble(kind, c) (python/skfemntv/bilinear_form.py:102-367,
 * cpp/src/assembly/cross_bilinear_assembler.cpp:55-107).  Kinds: 0 value,
 * 1 gradient.  Test tabulation nt functions (shape (E,Q,nt) / grad
 * (E,Q,nt,3)), Ct components; trial likewise; d_dx (E,Q); d_coef
 * (E,Q,Ct,[3],Cc,[3]).  Pattern: test DOFs (E, nt*Ct) x trial DOFs
 * (E, nc*Cc). */
int skg_cross_assemble_tabulated(const skg_pattern *pattern, int64_t n_elements,
                                 int32_t nq, int32_t nt, int32_t Ct, int32_t row_kind,
                                 const double *d_t_shape, const double *d_t_grad,
                                 int32_t nc, int32_t Cc, int32_t col_kind,
                                 const double *d_c_shape, const double *d_c_grad,
                                 const double *d_dx, const double *d_coef,
                                 double *d_values, void *stream);

/* ------------------------------------------------------------------ */
/* Fused scalar P1/P2 assembly straight from mesh coordinates.          */
/* Replaces the whole `asm(BilinearForm, Basis)` chain for             */
/*   w.kappa * ddot(grad u, grad v)      (coef_kind 0: scalar)           */
/*   dot(mul(w.A, grad u), grad v)       (coef_kind 1: 3x3 tensor)       */
/* on affine tetrahedra (python/skfemntv/forms.py:276-374 ->            */
/* bilinear_form.py:13-99 / 102-367 -> the two native assemblers):      */
/* geometry, element contraction and the fixed-order CSR sum in one     */
/* pass, without tabulated per-point arrays.                            */
/*  d_p (3, npts); d_t (nodes, E) with nodes 4 (P1) or 10 (P2, the      */
/*  mesh must be affine: edge nodes at midpoints).  The scalar DOFs are  */
/*  the pattern's (skg_pattern_create).  h_X (3,Q), h_W (Q): the rule.   */
/*  coef_kind 0: d_coef per element (E) or NULL for 1.                   */
/*  coef_kind 1: d_coef per element (E,3,3), row-major A[i][j].          */
/*  coef_kind 2: d_coef per element, component-first (3,3,E) (the        */
/*  reference's public (3,3,E,Q) layout with the point axis dropped).     */
/*  precision: SKG_FP64, SKG_FP64_EMULATED or SKG_SPLIT_FP32 (the last   */
/*  two fall back to SKG_FP64 when the mesh or coefficient leaves FP32    */
/*  range after a power-of-two rescaling).                                */
/*  d_values (nnz) is overwritten.                                       */
int skg_h1_assemble_affine(const skg_pattern *pattern, const double *d_p,
                           int64_t npts, const int32_t *d_t, int32_t nodes,
                           int64_t n_elements, int32_t nq, const double *h_X,
                           const double *h_W, int32_t coef_kind,
                           const double *d_coef, int32_t precision,
                           double *d_values, void *stream);

/* Same as skg_h1_assemble_affine, and writes the duration of its two
 * kernels (element pass, row pass) in milliseconds to h_kernel_ms[0..1],
 * measured with CUDA events on `stream`.  Synchronous. */
int skg_h1_assemble_affine_profiled(const skg_pattern *pattern, const double *d_p,
                                    int64_t npts, const int32_t *d_t, int32_t nodes,
                                    int64_t n_elements, int32_t nq, const double *h_X,
                                    const double *h_W, int32_t coef_kind,
                                    const double *d_coef, int32_t precision,
                                    double *d_values, float *h_kernel_ms, void *stream);
/* As skg_h1_assemble_affine, the values also delivered to page-locked host
 * memory h_values (nnz): the row pass runs in row chunks and each chunk's
 * values are copied while the next chunk is assembled (d_values is the
 * device staging buffer).  Stream-ordered; h_values is complete when the
 * stream is.  No counterpart in the reference (host-only). */
int skg_h1_assemble_affine_host(const skg_pattern *pattern, const double *d_p,
                                int64_t npts, const int32_t *d_t, int32_t nodes,
                                int64_t n_elements, int32_t nq, const double *h_X,
                                const double *h_W, int32_t coef_kind,
                                const double *d_coef, int32_t precision, double *d_values,
                                double *h_values, void *stream);

/* Allocation-free variant of skg_h1_assemble_affine (no counterpart in
 * the reference).  For callers that cannot let a library allocate device
 * memory: applications that give all device memory to their own pool
 * allocator and forbid other allocations, and solvers that re-assemble
 * inside a time-stepping loop where cudaMalloc / cudaFree (which may
 * synchronise the device) is not allowed.  Same arguments as
 * skg_h1_assemble_affine and the same results to rounding (P1, and P2 in
 * FP64 or double-float, sum rows evaluated from per-element G instead of
 * stored element matrices: same mathematics, slower at scale); it calls no
 * cudaMalloc, cudaFree or allocating library routine.  Its scratch is a
 * fixed static device array of the library (32 MiB plus a small table),
 * held on every GPU that loads the library until the process exits;
 * meshes of more than SKG_NOALLOC_MAX_ELEMENTS elements are rejected with
 * SKG_EINVAL.  The first call on a device looks up the array's device
 * address on that device and keeps it for the life of the process (so make
 * that first call before any stream capture; after cudaDeviceReset the
 * kept address is stale and the process must not call this again).  Each
 * call copies the quadrature table from host memory into the array.  In
 * SKG_FP64_EMULATED and SKG_SPLIT_FP32 it synchronises the host with
 * `stream` once per call, to read the range flag that decides between the
 * FP32-pair kernels and SKG_FP64; SKG_FP64 does not synchronise.  All calls
 * share the array and each call overwrites what the last one left there:
 * calls that overlap on the GPU (on different streams, or from different
 * host threads) race and must be serialised by the caller. */
#define SKG_NOALLOC_MAX_ELEMENTS 262144
int skg_h1_assemble_affine_noalloc(const skg_pattern *pattern, const double *d_p,
                                   int64_t npts, const int32_t *d_t, int32_t nodes,
                                   int64_t n_elements, int32_t nq, const double *h_X,
                                   const double *h_W, int32_t coef_kind,
                                   const double *d_coef, int32_t precision,
                                   double *d_values, void *stream);

/* P1 forms with per-element coefficients on affine tets: the value,
 * gradient, symmetric-gradient and divergence kinds of
 * BilinearFormAssembler.assemble (cpp/src/assembly/bilinear_form_assembler.cpp:79-105,
 * reached from NativeBilinearForm.assemble, python/skfemntv/bilinear_form.py:13-99)
 * for a scalar (comp 1) or vector (comp 3) P1 basis whose coefficients are
 * constant on every element, straight from coordinates: no tabulated
 * basis data is read.  Each kind takes a per-element array d_k (E) or, when
 * that is NULL, the constant c_k (0 leaves the term out).  The point sums use
 * the caller's rule h_X (3,Q), h_W (Q) (weight sum and P1 mass table), so
 * results match the tabulated path to rounding.  d_t (G, E) with G >= 4
 * vertex rows (a P1 field on a P2 geometry mesh uses its vertices; the map
 * must be affine).  d_values (nnz) is overwritten; with h_values non-NULL
 * (page-locked) the values are also delivered there in row chunks as in
 * skg_h1_assemble_affine_host.  Stream-ordered. */
int skg_p1_assemble_affine_forms(const skg_pattern *pattern, const double *d_p,
                                 int64_t npts, const int32_t *d_t, int64_t n_elements,
                                 int32_t comp, int32_t nq, const double *h_X,
                                 const double *h_W, const double *d_value,
                                 const double *d_gradient, const double *d_symgrad,
                                 const double *d_div, double c_value, double c_gradient,
                                 double c_symgrad, double c_div, double *d_values,
                                 double *h_values, void *stream);

/* ------------------------------------------------------------------ */
/* Nedelec N1 (lowest-order H(curl)) on affine tets.                    */

/* First-seen oriented edge numbering.  Replaces build_oriented_edge_topology
 * (cpp/src/assembly/edge_topology.cpp:30-84) and MeshTet2.from_mesh's edge
 * numbering (python/skfemntv/basis.py:644-658): global edge ids in cell-
 * major, local-edge-major first-seen order, key = ascending vertex pair,
 * sign +1 when the local edge runs from the smaller vertex.
 * d_t (4, E); outputs d_edges (2, 6E capacity, packed row stride 6E),
 * d_elem_edges (6, E), d_signs (6, E) int8.  *h_n_edges receives the edge
 * count.  A cell that repeats a corner vertex gives SKG_EINVAL with
 * h_bad_cell set.  Synchronous. */
int skg_edge_topology(const int32_t *d_t, int64_t n_elements, int32_t *d_edges,
                      int32_t *d_elem_edges, int8_t *d_signs, int64_t *h_n_edges,
                      int64_t *h_bad_cell, void *stream);

/* TetN1 Maxwell assembly K = sum_q dx (mass v_a.v_b + curl c_a.c_b).
 * Replaces TetN1Assembler.assemble_maxwell / assemble_mass /
 * assemble_curl_curl (python/skfemntv/hcurl_assembler.py:160-215 with
 * integrate_tet_n1, cpp/src/assembly/edge_topology.cpp:156-233, and the
 * np.add.at scatter, hcurl_assembler.py:94-97), straight from coordinates:
 * affine Jacobian, covariant Piola values J^-T phi, curls J c / det J,
 * orientation signs.  d_mass / d_curl: per element (E) or NULL for 1;
 * include flags select the terms.  h_X (3,Q), h_W (Q).  pattern built on
 * d_elem_edges^T.  d_values (nnz) overwritten. */
int skg_n1_assemble(const skg_pattern *pattern, const double *d_p, int64_t npts,
                    const int32_t *d_t, const int32_t *d_elem_edges,
                    const int8_t *d_signs, int64_t n_elements, int32_t nq,
                    const double *h_X, const double *h_W, const double *d_mass,
                    const double *d_curl, int32_t include_mass,
                    int32_t include_curl, int32_t precision, double *d_values,
                    void *stream);

/* skg_n1_assemble with the values also written to the page-locked host
 * array h_values (nnz), for callers that want the host CSR matrix
 * (TetN1Assembler.assemble_maxwell returns one, hcurl_assembler.py:160-215).
 * d_values (nnz, device) is the staging array.  On a row-grouped pattern the
 * element and row passes run over row chunks and each chunk's values are
 * copied while later chunks run; the stream has the host values once it
 * reaches the end of the call's work. */
int skg_n1_assemble_host(const skg_pattern *pattern, const double *d_p, int64_t npts,
                         const int32_t *d_t, const int32_t *d_elem_edges,
                         const int8_t *d_signs, int64_t n_elements, int32_t nq,
                         const double *h_X, const double *h_W, const double *d_mass,
                         const double *d_curl, int32_t include_mass,
                         int32_t include_curl, int32_t precision, double *d_values,
                         double *h_values, void *stream);

/* Per-point coefficients: d_mass / d_curl (E, Q) (not NULL); the explicit
 * quadrature loop of integrate_tet_n1 (edge_topology.cpp:156-233) on the
 * mapped basis computed in the kernel. */
int skg_n1_assemble_pointwise(const skg_pattern *pattern, const double *d_p,
                              int64_t npts, const int32_t *d_t, const int8_t *d_signs,
                              int64_t n_elements, int32_t nq, const double *h_X,
                              const double *h_W, const double *d_mass,
                              const double *d_curl, int32_t include_mass,
                              int32_t include_curl, double *d_values, void *stream);
/* N1 vector load r = int f . phi (TetN1LinearAssembler.assemble_vector_load,
 * hcurl_assembler.py:218-246): f (3, E, Q) at the rule's points; pattern:
 * element edge DOFs (E, 6), incidence only; d_out (N), summed per DOF in
 * element order. */
int skg_n1_vector_load(const skg_pattern *pattern, const double *d_p, int64_t npts,
                       const int32_t *d_t, const int8_t *d_signs, int64_t n_elements,
                       int32_t nq, const double *h_X, const double *h_W,
                       const double *d_f, double *d_out, void *stream);

/* N1 element matrices d_out (E, 6, 6), row = test edge, FP64: the
 * assembly's element pass written to the caller's buffer.  Replaces
 * integrate_tet_n1 (cpp/src/assembly/edge_topology.cpp:156-233, bound in
 * cpp/src/bindings.cpp) and AffineTetN1Basis.element_mass_matrices /
 * element_curl_curl_matrices (python/skfemntv/hcurl_basis.py:376-386).
 * d_mass / d_curl: NULL for 1, else per element (E) for coef_per_point 0
 * or per point (E, Q) for 1; include flags select the terms. */
int skg_n1_element_matrices(const double *d_p, int64_t npts, const int32_t *d_t,
                            const int8_t *d_signs, int64_t n_elements, int32_t nq,
                            const double *h_X, const double *h_W, const double *d_mass,
                            const double *d_curl, int32_t coef_per_point,
                            int32_t include_mass, int32_t include_curl, double *d_out,
                            void *stream);

/* A global edge field u (n_edges) at the rule's points h_X (3, Q), written
 * component-first to d_out (3, E, Q): values (curl 0) or vector curls
 * (curl 1) of the mapped, oriented basis.  Replaces AffineTetN1Basis
 * .evaluate / .evaluate_curl (python/skfemntv/hcurl_basis.py:418-432).
 * d_elem_edges (6, E) int32, d_signs (6, E) int8. */
int skg_n1_evaluate(const double *d_p, int64_t npts, const int32_t *d_t,
                    const int32_t *d_elem_edges, const int8_t *d_signs,
                    int64_t n_elements, int64_t n_edges, int32_t nq, const double *h_X,
                    const double *d_coefficients, int32_t curl, double *d_out,
                    void *stream);

/* Edge-moment interpolation, AffineTetN1Basis.interpolate_edge_moments
 * (python/skfemntv/hcurl_basis.py:388-416), in two device passes around the
 * caller's field: skg_n1_edge_points writes x = p_a + (p_b - p_a) t_q for
 * each global edge (a, b) of d_edges (2, n_edges) int32 and parameter h_param
 * (Q) to d_out (3, n_edges * Q), edge-major; skg_n1_edge_moments sums
 * m = sum_q w_q f(x_q) . (p_b - p_a) over the field values d_values
 * (3, n_edges * Q) into d_out (n_edges). */
int skg_n1_edge_points(const double *d_p, int64_t npts, const int32_t *d_edges,
                       int64_t n_edges, int32_t nq, const double *h_param, double *d_out,
                       void *stream);
int skg_n1_edge_moments(const double *d_p, int64_t npts, const int32_t *d_edges,
                        int64_t n_edges, int32_t nq, const double *h_weights,
                        const double *d_values, double *d_out, void *stream);

/* ------------------------------------------------------------------ */
/* Linear forms.  Replaces LinearFormAssembler.assemble                 */
/* (cpp/src/assembly/linear_form_assembler.cpp:41-154):                 */
/*   r[dof(a,c)] += sum_q w (f_c N_a + G_cj dN_a/dx_j)                  */
/* value (E,Q,comp) or NULL, gradient (E,Q,comp,3) or NULL.  The sum    */
/* per DOF is made in element order (deterministic).  d_out (n_dofs).   */
int skg_linear_assemble_tabulated(const skg_pattern *pattern,
                                  const int32_t *d_dofs, int64_t n_elements,
                                  int32_t nodes, int32_t comp, int32_t nq,
                                  const double *d_shape, const double *d_grad,
                                  const double *d_w, const double *d_value,
                                  const double *d_gradient, double *d_out,
                                  void *stream);

/* ------------------------------------------------------------------ */
/* Adjoint of J = u^T K(kappa) v for P1 diffusion (no counterpart in    */
/* the reference, which has no autograd; K(kappa) is the matrix of      */
/* asm(w.kappa * ddot(grad u, grad v), basis), python/skfemntv/forms.py  */
/* :276-374 with bilinear_form_assembler.cpp:79-105, assembled          */
/* matrix-free).  d_t (4, E) vertex connectivity, d_dofs (E, 4) element */
/* DOFs, kappa (E) or NULL = 1, u / v (N), wsum = sum of the quadrature  */
/* weights.  Energy reduced in a fixed order into d_out (1 double).     */
int skg_p1_energy(const double *d_p, int64_t npts, const int32_t *d_t,
                  int64_t n_elements, const int32_t *d_dofs,
                  const double *d_kappa, const double *d_u, const double *d_v,
                  double wsum, double *d_out, void *stream);

/* Gradients of grad_out * J: d_gkappa (E), d_gp (3, npts) (needs the
 * incidence-only handle of the vertex connectivity, d_t^T with npts rows),
 * d_gu / d_gv (N) (needs the incidence-only handle of the DOF map); any
 * output may be NULL.  When the DOFs are the vertices (scalar P1, every
 * vertex a DOF) the same handle may be passed twice: all gradients are then
 * gathered in one walk.  Geometry is recomputed, nothing is kept from the
 * forward call. */
int skg_p1_energy_grad(const skg_pattern *vertex_incidence,
                       const skg_pattern *dof_incidence, const double *d_p,
                       int64_t npts, const int32_t *d_t, int64_t n_elements,
                       const int32_t *d_dofs, const double *d_kappa,
                       const double *d_u, const double *d_v, double wsum,
                       double grad_out, double *d_gkappa, double *d_gp,
                       double *d_gu, double *d_gv, void *stream);

/* skg_p1_energy_grad that also writes J itself to d_energy (1): the element
 * pass reduces the element energies exactly as skg_p1_energy does (same
 * value, same summation order) while it forms the adjoint contributions, so
 * one call gives J and its gradients (for a forward pass that knows the
 * gradients will be needed).  The gradients are those of grad_out * J. */
int skg_p1_energy_value_and_grad(const skg_pattern *vertex_incidence,
                                 const skg_pattern *dof_incidence, const double *d_p,
                                 int64_t npts, const int32_t *d_t, int64_t n_elements,
                                 const int32_t *d_dofs, const double *d_kappa,
                                 const double *d_u, const double *d_v, double wsum,
                                 double grad_out, double *d_energy, double *d_gkappa,
                                 double *d_gp, double *d_gu, double *d_gv, void *stream);

/* ------------------------------------------------------------------ */
/* Neo-Hookean residual and tangent on vector P1 tetrahedra.  Replaces   */
/* the reference's oracle pipeline for the law of                        */
/* benchmarks/skfem_neo_hookean.py:8-52: NativeLinearForm residual        */
/* (linear_form_assembler.cpp:41-154) + NativeCrossBilinearForm tensor    */
/* tangent (cross_bilinear_assembler.cpp:207-247).  Pattern: element DOFs */
/* (E, 12), with CSR columns when the tangent is wanted.  u (N), in      */
/* device memory or in host memory the device can read (then copied to   */
/* the device first, coalesced); outputs d_residual (N) and d_values     */
/* (nnz), either may be NULL.                                             */
int skg_nh_assemble(const skg_pattern *pattern, const double *d_p, int64_t npts,
                    const int32_t *d_t, int64_t n_elements, const double *d_u,
                    double mu, double lmbda, double wsum, double *d_residual,
                    double *d_values, void *stream);
/* skg_nh_assemble with the residual and tangent values also written to the
 * page-locked host arrays h_residual (N) and h_values (nnz); d_residual and
 * d_values are the device staging arrays (both required).  On a row-grouped
 * pattern the element and row passes run over row chunks and each chunk's
 * rows are copied while later chunks run. */
int skg_nh_assemble_host(const skg_pattern *pattern, const double *d_p, int64_t npts,
                         const int32_t *d_t, int64_t n_elements, const double *d_u,
                         double mu, double lmbda, double wsum, double *d_residual,
                         double *d_values, double *h_residual, double *h_values,
                         void *stream);

/* Learned closure (no counterpart in the reference): an MLP
 * 3 -> 64 -> 64 -> 1 (tanh) with a linear input -> output skip, on the
 * invariant features (I1-3, I2-3, ln J), predicts the strain energy; float32
 * parameters, skg_mlp_param_count() floats (weights, then feature mean/std,
 * output scale/shift and the stress-normalisation constant). */
int skg_mlp_param_count(void);
/* Training samples F = I + G, G_ij ~ N(0, sigma^2) from a counter-based
 * generator; features (n, 3) and targets (n, 4) = W, dW/df (plain law). */
int skg_mlp_dataset(int64_t n, uint64_t seed, double sigma, double mu,
                    double lmbda, float *d_features, float *d_targets,
                    void *stream);
/* Loss (energy + beta * feature-gradient misfit, normalised units) and its
 * gradient over samples perm[offset .. offset+batch) (mod n); fixed-order
 * reduction. */
int skg_mlp_loss_grad(const float *d_params, const float *d_features,
                      const float *d_targets, int64_t n, const int64_t *d_perm,
                      int64_t offset, int32_t batch, float beta, float *d_grad,
                      float *d_loss, void *stream);
/* `steps` Adam steps (cosine learning-rate schedule lr0 -> lr_min) on the
 * device; h_last_loss receives the last batch loss.  Sets the
 * stress-normalisation constant of the final weights. */
int skg_mlp_train(float *d_params, const float *d_features,
                  const float *d_targets, int64_t n, const int64_t *d_perm,
                  int32_t steps, int32_t batch, float lr0, float lr_min,
                  float beta, float *d_adam_m, float *d_adam_v, int32_t step0,
                  float *h_last_loss, void *stream);
/* L-BFGS refinement (history `history`, Armijo backtracking) over the fixed
 * samples perm[offset .. offset+count) (mod n): loss and gradient on the
 * device, two-loop recursion on the host in FP64; up to `iters` iterations,
 * *h_loss receives the final loss.  Sets the stress-normalisation constant. */
int skg_mlp_refine(float *d_params, const float *d_features,
                   const float *d_targets, int64_t n, const int64_t *d_perm,
                   int64_t offset, int32_t count, int32_t iters, int32_t history,
                   float beta, double *h_loss, void *stream);
/* psi, d psi/dx (3), d2 psi/dx2 (9) per normalised input x (n, 3) -> (n, 13). */
int skg_mlp_eval(const float *d_params, const float *d_x, int64_t n,
                 float *d_out, void *stream);
/* Neo-Hookean residual / tangent with the MLP energy; elements whose
 * features leave the trained box d_box = (min[3], max[3]) or whose stress
 * differs from the plain law by more than tol (relative) use the FP64
 * plain law; *h_fallback receives their number (synchronous when given). */
int skg_nh_assemble_surrogate(const skg_pattern *pattern, const double *d_p,
                              int64_t npts, const int32_t *d_t, int64_t n_elements,
                              const double *d_u, double mu, double lmbda,
                              double wsum, const float *d_params,
                              const float *d_box, float tol, double *d_residual,
                              double *d_values, int64_t *h_fallback, void *stream);
/* skg_nh_assemble_surrogate with host outputs, as skg_nh_assemble_host. */
int skg_nh_assemble_surrogate_host(const skg_pattern *pattern, const double *d_p,
                                   int64_t npts, const int32_t *d_t,
                                   int64_t n_elements, const double *d_u, double mu,
                                   double lmbda, double wsum, const float *d_params,
                                   const float *d_box, float tol, double *d_residual,
                                   double *d_values, double *h_residual,
                                   double *h_values, int64_t *h_fallback, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SKFEM_GB300_H */
