// Lowest-order Nedelec (N1, Whitney edge) elements on affine tetrahedra.
//
// Edge topology: the reference numbers global edges in first-seen order
// while walking cells and their local edges (0,1),(1,2),(2,0),(0,3),(1,3),
// (2,3) (cpp/src/assembly/edge_topology.cpp:30-84).  That sequential rule is
// reproduced exactly in parallel: every (cell, local edge) item is inserted
// into a device hash table keyed by its ascending vertex pair, keeping the
// smallest item index (its first occurrence); items that are their key's
// first occurrence are flagged, an exclusive scan of the flags in item order
// gives each first occurrence its edge id, and every item takes the id of
// its key's first occurrence.
//
// Assembly (TetN1Assembler.assemble_maxwell, python/skfemntv/
// hcurl_assembler.py:160-215): with barycentric gradients g_k = b_k / det J
// (b_k rows of adj J, b_0 = -(b_1+b_2+b_3)), the mapped basis of directed
// edge a = (i, j) is J^-T phi_a = lambda_i g_j - lambda_j g_i and its curl
// J c_a / det J (c_a = 2 ghat_i x ghat_j), each times the orientation sign
// (python/skfemntv/hcurl_basis.py:353-364, _hcurl_mapping.py:46-97).  For
// coefficients constant per element the quadrature sum collapses to
//   M_ab = mass * s_a s_b sum_{k,l} (b_k.b_l / |det|) Tm^{kl}_ab,
//   Tm^{kl}_ab = sum_q w_q d^k_a(xi_q) d^l_b(xi_q)   (host table, per rule)
//   C_ab = curl * s_a s_b (sum_q w_q) (J c_a).(J c_b) / |det|.
// Per-point coefficients use the explicit quadrature loop.  The 6x6 element
// matrices then go through the same fixed-order row-owner gather as H1.
#include <climits>
#include <vector>

#include "skg_common.cuh"
#include "skg_df64.cuh"
#include "skg_rows.cuh"

namespace skg {

void gather_element_matrices(const skg_pattern *pat, const double *Ke, double *values, cudaStream_t s);
void gather_element_vectors(const skg_pattern *pat, const double *le, double *out, cudaStream_t s);

namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x ^= x >> 33; x *= 0xff51afd7ed558ccdULL; x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL; x ^= x >> 33;
    return x;
}

__constant__ int kEdge[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};

constexpr unsigned long long kEmpty = ~0ull;

__global__ void k_edge_insert(const int32_t *__restrict__ t, int64_t ne, unsigned long long *keys,
                              int32_t *first, uint64_t mask, int32_t *bad_cell, int32_t *overflow) {
    const int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= ne * 6) return;
    const int64_t cell = item / 6;
    const int l = (int)(item % 6);
    if (l == 0) {
        int32_t v[4];
        for (int k = 0; k < 4; ++k) v[k] = t[k * ne + cell];
        for (int f = 0; f < 4; ++f)
            for (int g = f + 1; g < 4; ++g)
                if (v[f] == v[g]) atomicMin(bad_cell, (int32_t)cell);
    }
    const int32_t a = t[kEdge[l][0] * ne + cell], b = t[kEdge[l][1] * ne + cell];
    const uint32_t lo = (uint32_t)min(a, b), hi = (uint32_t)max(a, b);
    const unsigned long long key = ((unsigned long long)lo << 32) | hi;
    uint64_t h = mix64(key) & mask;
    for (uint64_t probe = 0; probe <= mask; ++probe) {
        const unsigned long long prev = atomicCAS(&keys[h], kEmpty, key);
        if (prev == kEmpty || prev == key) {
            atomicMin(&first[h], (int32_t)item);
            return;
        }
        h = (h + 1) & mask;
    }
    *overflow = 1;
}

__global__ void k_edge_flag(const int32_t *__restrict__ t, int64_t ne, const unsigned long long *keys,
                            const int32_t *first, uint64_t mask, int32_t *flag, int32_t *slot_of) {
    const int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= ne * 6) return;
    const int64_t cell = item / 6;
    const int l = (int)(item % 6);
    const int32_t a = t[kEdge[l][0] * ne + cell], b = t[kEdge[l][1] * ne + cell];
    const uint32_t lo = (uint32_t)min(a, b), hi = (uint32_t)max(a, b);
    const unsigned long long key = ((unsigned long long)lo << 32) | hi;
    uint64_t h = mix64(key) & mask;
    for (uint64_t probe = 0; probe <= mask; ++probe) {
        if (keys[h] == key) break;
        h = (h + 1) & mask;
    }
    slot_of[item] = (int32_t)h;
    flag[item] = first[h] == (int32_t)item ? 1 : 0;
}

__global__ void k_edge_emit(const int32_t *__restrict__ t, int64_t ne, const int32_t *first,
                            const int32_t *slot_of, const int32_t *flag, const int32_t *scan, int32_t *edges,
                            int32_t *elem_edges, int8_t *signs) {
    const int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= ne * 6) return;
    const int64_t cell = item / 6;
    const int l = (int)(item % 6);
    const int32_t a = t[kEdge[l][0] * ne + cell], b = t[kEdge[l][1] * ne + cell];
    const int32_t id = scan[first[slot_of[item]]];
    elem_edges[l * ne + cell] = id;
    signs[l * ne + cell] = (int8_t)(a < b ? 1 : -1);
    if (flag[item]) {
        edges[id] = min(a, b);
        edges[ne * 6 + id] = max(a, b);
    }
}

// ---------------------------------------------------------------- assembly

struct N1Table {
    double Tm[6][6][4];  // [a][b][s*2+t], s/t index the support (i, j) of a / b
    double wsum;
};

// The same table as FP32 (hi, lo) pairs for the split-precision pass.
struct N1TableF {
    float2 Tm[6][6][4];
    float2 wsum;
};

__device__ __forceinline__ void n1_geometry(const double *__restrict__ p, int64_t npts,
                                            const int32_t *__restrict__ t, int64_t ne, int64_t e, double J[9],
                                            double b[4][3], double &det) {
    int32_t v0 = t[e], v1 = t[ne + e], v2 = t[2 * ne + e], v3 = t[3 * ne + e];
    // out-of-range vertex ids never reach memory: the element becomes NaN
    const bool ok = v0 >= 0 && v0 < npts && v1 >= 0 && v1 < npts && v2 >= 0 && v2 < npts && v3 >= 0 && v3 < npts;
    if (!ok) v0 = v1 = v2 = v3 = 0;
    const int32_t v[3] = {v1, v2, v3};
    for (int i = 0; i < 3; ++i) {
        const double x0 = p[i * npts + v0];
        for (int r = 0; r < 3; ++r) J[i * 3 + r] = ok ? p[i * npts + v[r]] - x0 : __longlong_as_double(0x7ff8000000000000LL);
    }
    b[1][0] = J[4] * J[8] - J[5] * J[7];
    b[1][1] = J[2] * J[7] - J[1] * J[8];
    b[1][2] = J[1] * J[5] - J[2] * J[4];
    b[2][0] = J[5] * J[6] - J[3] * J[8];
    b[2][1] = J[0] * J[8] - J[2] * J[6];
    b[2][2] = J[2] * J[3] - J[0] * J[5];
    b[3][0] = J[3] * J[7] - J[4] * J[6];
    b[3][1] = J[1] * J[6] - J[0] * J[7];
    b[3][2] = J[0] * J[4] - J[1] * J[3];
    det = J[0] * b[1][0] + J[1] * b[2][0] + J[2] * b[3][0];
    for (int i = 0; i < 3; ++i) b[0][i] = -(b[1][i] + b[2][i] + b[3][i]);
}

// Reference curls c_a = 2 ghat_i x ghat_j for the directed local edges.
__constant__ double kRefCurl[6][3] = {{0, -2, 2}, {0, 0, 2}, {-2, 0, 2}, {-2, 2, 0}, {0, -2, 0}, {2, 0, 0}};

// Local edges (i, j) and the reference curls c_a = 2 ghat_i x ghat_j as
// compile-time functions (the fully unrolled element kernel folds them).
__host__ __device__ constexpr int edge_v(int a, int k) {
    return k == 0 ? (a == 0 ? 0 : a == 1 ? 1 : a == 2 ? 2 : a == 3 ? 0 : a == 4 ? 1 : 2)
                  : (a == 0 ? 1 : a == 1 ? 2 : a == 2 ? 0 : 3);
}
__host__ __device__ constexpr double ref_curl(int a, int i) {
    constexpr double c[6][3] = {{0, -2, 2}, {0, 0, 2}, {-2, 0, 2}, {-2, 2, 0}, {0, -2, 0}, {2, 0, 0}};
    return c[a][i];
}

constexpr int kN1Block = 128;

// Per-element coefficients, closed form: K_ac = s_a s_c (mu sum_uv G T + nu
// (J c_a . J c_c) wsum / |det|) with G = b_k . b_l / |det|; the 21 entries of
// the symmetric 6 x 6 matrix, stores staged through shared memory (FP64).
// The curl term as c_a^T H c_c with H = 4 nu wsum J^T J / |det| (the
// reference curls c_a have entries 0 and +-2): signed sums of H's entries.
__global__ void __launch_bounds__(kN1Block) k_n1_elem_fast(int64_t ne, int64_t e_begin, int64_t e_end,
                                                            const double *__restrict__ p, int64_t npts,
                                                            const int32_t *__restrict__ t,
                                                            const int8_t *__restrict__ signs, N1Table tab,
                                                            const double *__restrict__ mass,
                                                            const double *__restrict__ curl, int inc_mass,
                                                            int inc_curl, double *__restrict__ Ke) {
    __shared__ double stage[kN1Block * 37];
    const int64_t e0 = e_begin + (int64_t)blockIdx.x * kN1Block;
    const int64_t e = e0 + threadIdx.x;
    if (e < e_end) {
        double J[9], b[4][3], det;
        n1_geometry(p, npts, t, ne, e, J, b, det);
        const double inv = 1.0 / fabs(det);
        const double mu = inc_mass ? (mass ? mass[e] : 1.0) : 0.0;
        const double nu = inc_curl ? (curl ? curl[e] : 1.0) * inv * tab.wsum : 0.0;
        // mu b_k . b_l / |det J|: dot products for k, l >= 1, row 0 from
        // b_0 = -(b_1 + b_2 + b_3); mu / |det J| scales the six products once
        const double mi = mu * inv;
        double Gm[4][4];
#pragma unroll
        for (int k = 1; k < 4; ++k)
#pragma unroll
            for (int l = k; l < 4; ++l) {
                Gm[k][l] = (b[k][0] * b[l][0] + b[k][1] * b[l][1] + b[k][2] * b[l][2]) * mi;
                Gm[l][k] = Gm[k][l];
            }
#pragma unroll
        for (int l = 1; l < 4; ++l) {
            Gm[0][l] = -(Gm[1][l] + Gm[2][l] + Gm[3][l]);
            Gm[l][0] = Gm[0][l];
        }
        Gm[0][0] = -(Gm[0][1] + Gm[0][2] + Gm[0][3]);
        // curl term nu (J c_a).(J c_c) = c_a^T (nu J^T J) c_c: with H = 4 nu J^T J (6 entries) and the
        // reference curls' entries +-2, each entry is a signed sum of 1 to 4 entries of H
        double H[3][3];
        const double nu4 = 4.0 * nu;
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int q = r; q < 3; ++q) {
                H[r][q] = nu4 * (J[r] * J[q] + J[3 + r] * J[3 + q] + J[6 + r] * J[6 + q]);
                H[q][r] = H[r][q];
            }
        // orientation signs (+1 / -1) applied as a sign-bit flip of the FP64 value
        uint32_t neg[6];
#pragma unroll
        for (int a = 0; a < 6; ++a) neg[a] = signs[a * ne + e] < 0 ? 1u : 0u;
        double *st = stage + threadIdx.x * 37;
#pragma unroll
        for (int a = 0; a < 6; ++a)
#pragma unroll
            for (int c = a; c < 6; ++c) {
                double val = 0.0;
                bool first = true;
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int q = 0; q < 3; ++q)
                        if (ref_curl(a, r) != 0.0 && ref_curl(c, q) != 0.0) {
                            const double h = (ref_curl(a, r) > 0.0) == (ref_curl(c, q) > 0.0) ? H[r][q] : -H[r][q];
                            val = first ? h : val + h;
                            first = false;
                        }
#pragma unroll
                for (int u = 0; u < 2; ++u)
#pragma unroll
                    for (int v = 0; v < 2; ++v) val += Gm[edge_v(a, u)][edge_v(c, v)] * tab.Tm[a][c][u * 2 + v];
                const unsigned long long flip = (unsigned long long)(neg[a] ^ neg[c]) << 63;
                val = __longlong_as_double((long long)((unsigned long long)__double_as_longlong(val) ^ flip));
                st[a * 6 + c] = val;
                st[c * 6 + a] = val;
            }
    }
    __syncthreads();
    const int nvalid = (int)(e_end - e0 < kN1Block ? e_end - e0 : kN1Block);
    for (int i = threadIdx.x; i < nvalid * 36; i += kN1Block) {
        const int el = i / 36, q = i - el * 36;
        Ke[(e0 + el) * 36 + q] = stage[el * 37 + q];
    }
}

// Split precision without FP64 arithmetic beyond the edge differences: the
// geometry in double-float with coordinates scaled by 2^-s (G = b_k.b_l / |det|
// then carries 2^-s and nu = curl / |det| 2^3s, J c 2^-s), the entries
// contracted in FP32 with split products (hi hi + hi lo + lo hi) and FP32
// accumulation of the products' high and low parts; the mass term (scale 2^-s)
// and the curl term (2^s) are converted to FP64 by integer bit arithmetic with
// the scale applied to the exponent (exact), then added.  *range_bad is set
// when a value leaves the FP32 range (the caller then recomputes in FP64).
__global__ void __launch_bounds__(kN1Block) k_n1_elem_df(int64_t ne, int64_t e_begin, int64_t e_end,
                                                          const double *__restrict__ p, int64_t npts,
                                                          const int32_t *__restrict__ t,
                                                          const int8_t *__restrict__ signs, N1TableF tab,
                                                          const double *__restrict__ mass,
                                                          const double *__restrict__ curl, int inc_mass,
                                                          int inc_curl, const int *__restrict__ s_ptr,
                                                          int *__restrict__ range_bad, double *__restrict__ Ke) {
    __shared__ double stage[kN1Block * 37];
    const int sc = *s_ptr;
    const int64_t e0 = e_begin + (int64_t)blockIdx.x * kN1Block;
    const int64_t e = e0 + threadIdx.x;
    if (e < e_end) {
        int32_t v[4];
        bool ok = true;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            v[k] = t[k * ne + e];
            ok = ok && v[k] >= 0 && v[k] < npts;
        }
        if (!ok) v[0] = v[1] = v[2] = v[3] = 0;
        df64 J[9];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const double x0 = p[i * npts + v[0]];
#pragma unroll
            for (int r = 0; r < 3; ++r) J[i * 3 + r] = df_from_double(p[i * npts + v[r + 1]] - x0, -sc, ok);
        }
        df64 b[4][3];
#define SKG_CROSS(a, bb, c, d) df_add_fast(df_mul(J[a], J[bb]), df_neg(df_mul(J[c], J[d])))
        b[1][0] = SKG_CROSS(4, 8, 5, 7);
        b[1][1] = SKG_CROSS(2, 7, 1, 8);
        b[1][2] = SKG_CROSS(1, 5, 2, 4);
        b[2][0] = SKG_CROSS(5, 6, 3, 8);
        b[2][1] = SKG_CROSS(0, 8, 2, 6);
        b[2][2] = SKG_CROSS(2, 3, 0, 5);
        b[3][0] = SKG_CROSS(3, 7, 4, 6);
        b[3][1] = SKG_CROSS(1, 6, 0, 7);
        b[3][2] = SKG_CROSS(0, 4, 1, 3);
#undef SKG_CROSS
        df64 det = df_add_fast(df_add_fast(df_mul(J[0], b[1][0]), df_mul(J[1], b[2][0])), df_mul(J[2], b[3][0]));
#pragma unroll
        for (int i = 0; i < 3; ++i) b[0][i] = df_neg(df_add_fast(df_add_fast(b[1][i], b[2][i]), b[3][i]));
        if (det.hi < 0.f) det = df_neg(det);
        ok = ok && det.hi > 1e-30f;
        const df64 inv = df_recip(det);
        float2 G2[4][4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
#pragma unroll
            for (int l = k; l < 4; ++l) {
                const df64 d = df_mul(inv, df_add_fast(df_add_fast(df_mul(b[k][0], b[l][0]), df_mul(b[k][1], b[l][1])),
                                                       df_mul(b[k][2], b[l][2])));
                ok = ok && df_in_range(d);
                G2[k][l] = G2[l][k] = make_float2(d.hi, d.lo);
            }
        // curl term (J c_a).(J c_c) = c_a^T (J^T J) c_c: H = 4 J^T J in double-float (6 entries; the
        // reference curls' entries are +-2), each entry a signed sum of 1 to 4 of H's (hi, lo) pairs
        float2 H2[3][3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int q = r; q < 3; ++q) {
                const df64 h = df_add_fast(df_add_fast(df_mul(J[r], J[q]), df_mul(J[3 + r], J[3 + q])),
                                           df_mul(J[6 + r], J[6 + q]));
                H2[r][q] = H2[q][r] = make_float2(4.f * h.hi, 4.f * h.lo);
            }
        const df64 mu = inc_mass ? df_from_double(mass ? mass[e] : 1.0, 0, ok) : df64{0.f, 0.f};
        df64 nu{0.f, 0.f};
        if (inc_curl) {
            nu = df_mul(df_mul(df_from_double(curl ? curl[e] : 1.0, 0, ok), inv), df64{tab.wsum.x, tab.wsum.y});
            ok = ok && df_in_range(nu);
        }
        float sg[6];
#pragma unroll
        for (int a = 0; a < 6; ++a) sg[a] = (float)signs[a * ne + e];
        double *st = stage + threadIdx.x * 37;
#pragma unroll
        for (int a = 0; a < 6; ++a)
#pragma unroll
            for (int c = a; c < 6; ++c) {
                float mh = 0.f, ml = 0.f;
#pragma unroll
                for (int u = 0; u < 2; ++u)
#pragma unroll
                    for (int w = 0; w < 2; ++w) {
                        const float2 g = G2[edge_v(a, u)][edge_v(c, w)];
                        const float2 tt = tab.Tm[a][c][u * 2 + w];
                        const float ph = g.x * tt.x;
                        mh += ph;
                        ml += fmaf(g.x, tt.x, -ph) + fmaf(g.x, tt.y, g.y * tt.x);
                    }
                float ch = 0.f, cl = 0.f;
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int q = 0; q < 3; ++q)
                        if (ref_curl(a, r) != 0.0 && ref_curl(c, q) != 0.0) {
                            const float2 h = H2[r][q];
                            if ((ref_curl(a, r) > 0.0) == (ref_curl(c, q) > 0.0)) {
                                ch += h.x;
                                cl += h.y;
                            } else {
                                ch -= h.x;
                                cl -= h.y;
                            }
                        }
                const float m = mh + ml, cc = ch + cl;
                // mass term (scale 2^-s) and curl term (scale 2^s) as (hi, lo) pairs
                const float mth = mu.hi * m, ctl_h = nu.hi * cc;
                const df64 mt = fast_two_sum(mth, fmaf(mu.hi, m, -mth) + mu.lo * m);
                const df64 ct = fast_two_sum(ctl_h, fmaf(nu.hi, cc, -ctl_h) + nu.lo * cc);
                // unscaled in the FP64 exponent (exact), then one FP64 add
                double dv = df_to_double(mt, sc) + df_to_double(ct, -sc);
                if (sg[a] * sg[c] < 0.f) dv = -dv;
                st[a * 6 + c] = dv;
                st[c * 6 + a] = dv;
            }
        if (!ok) *range_bad = 1;
    }
    __syncthreads();
    const int nvalid = (int)(e_end - e0 < kN1Block ? e_end - e0 : kN1Block);
    for (int i = threadIdx.x; i < nvalid * 36; i += kN1Block) {
        const int el = i / 36, q = i - el * 36;
        Ke[(e0 + el) * 36 + q] = stage[el * 37 + q];
    }
}

// Thread per element: Ke (E, 6, 6).  mass/curl: per element (qstride 0) or
// per point (qstride 1, explicit quadrature loop); NULL = 1.
__global__ void k_n1_element(int64_t ne, const double *__restrict__ p, int64_t npts, const int32_t *__restrict__ t,
                             const int8_t *__restrict__ signs, int nq, const double *__restrict__ Xq,
                             const double *__restrict__ Wq, N1Table tab, const double *__restrict__ mass,
                             const double *__restrict__ curl, int qstride, int inc_mass, int inc_curl,
                             double *__restrict__ Ke) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    double J[9], b[4][3], det;
    n1_geometry(p, npts, t, ne, e, J, b, det);
    const double adet = fabs(det), inv = 1.0 / adet;
    double s[6];
    for (int a = 0; a < 6; ++a) s[a] = (double)signs[a * ne + e];
    double Jc[6][3];
    for (int a = 0; a < 6; ++a)
        for (int i = 0; i < 3; ++i)
            Jc[a][i] = J[i * 3 + 0] * kRefCurl[a][0] + J[i * 3 + 1] * kRefCurl[a][1] + J[i * 3 + 2] * kRefCurl[a][2];
    double K[6][6];
    if (qstride == 0) {
        const double mu = inc_mass ? (mass ? mass[e] : 1.0) : 0.0;
        const double nu = inc_curl ? (curl ? curl[e] : 1.0) : 0.0;
        double Gm[4][4];
        for (int k = 0; k < 4; ++k)
            for (int l = 0; l < 4; ++l) Gm[k][l] = (b[k][0] * b[l][0] + b[k][1] * b[l][1] + b[k][2] * b[l][2]) * inv;
        for (int a = 0; a < 6; ++a)
            for (int c = a; c < 6; ++c) {
                const int ai = kEdge[a][0], aj = kEdge[a][1], ci = kEdge[c][0], cj = kEdge[c][1];
                const int ka[2] = {ai, aj}, kc[2] = {ci, cj};
                double m = 0.;
                for (int u = 0; u < 2; ++u)
                    for (int v = 0; v < 2; ++v) m += Gm[ka[u]][kc[v]] * tab.Tm[a][c][u * 2 + v];
                const double cc = (Jc[a][0] * Jc[c][0] + Jc[a][1] * Jc[c][1] + Jc[a][2] * Jc[c][2]) * inv * tab.wsum;
                const double val = s[a] * s[c] * (mu * m + nu * cc);
                K[a][c] = val;
                K[c][a] = val;
            }
    } else {
        for (int a = 0; a < 6; ++a)
            for (int c = 0; c < 6; ++c) K[a][c] = 0.;
        for (int q = 0; q < nq; ++q) {
            const double x = Xq[q], y = Xq[nq + q], z = Xq[2 * nq + q];
            const double lam[4] = {1.0 - x - y - z, x, y, z};
            const double dx = adet * Wq[q];
            const double mu = inc_mass ? (mass ? mass[e * nq + q] : 1.0) : 0.0;
            const double nu = inc_curl ? (curl ? curl[e * nq + q] : 1.0) : 0.0;
            double phi[6][3];
            for (int a = 0; a < 6; ++a) {
                const int i = kEdge[a][0], j = kEdge[a][1];
                for (int d = 0; d < 3; ++d) phi[a][d] = (lam[i] * b[j][d] - lam[j] * b[i][d]) / det;
            }
            for (int a = 0; a < 6; ++a)
                for (int c = 0; c < 6; ++c) {
                    const double vv = phi[a][0] * phi[c][0] + phi[a][1] * phi[c][1] + phi[a][2] * phi[c][2];
                    const double ccv = (Jc[a][0] * Jc[c][0] + Jc[a][1] * Jc[c][1] + Jc[a][2] * Jc[c][2]) / (det * det);
                    K[a][c] += dx * (mu * vv + nu * ccv) * s[a] * s[c];
                }
        }
    }
    double *out = Ke + e * 36;
    for (int a = 0; a < 6; ++a)
        for (int c = 0; c < 6; ++c) {
            out[a * 6 + c] = K[a][c];
        }
}

// Vector load f . phi: local_a = s_a sum_q sum_i phi_a,i(x_q) f_i(e, q) |det| w_q
// with phi_a = lambda_i grad lambda_j - lambda_j grad lambda_i (TetN1LinearAssembler).
__global__ void k_n1_load(int64_t ne, const double *__restrict__ p, int64_t npts, const int32_t *__restrict__ t,
                          const int8_t *__restrict__ signs, int nq, const double *__restrict__ Xq,
                          const double *__restrict__ Wq, const double *__restrict__ f, double *__restrict__ le) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    double J[9], b[4][3], det;
    n1_geometry(p, npts, t, ne, e, J, b, det);
    const double adet = fabs(det), idet = 1.0 / det;
    double acc[6] = {0, 0, 0, 0, 0, 0};
    const int64_t EQ = ne * (int64_t)nq;
    for (int q = 0; q < nq; ++q) {
        const double x = Xq[q], y = Xq[nq + q], z = Xq[2 * nq + q];
        const double lam[4] = {1.0 - x - y - z, x, y, z};
        const double dx = adet * Wq[q];
        const double fx = f[e * nq + q], fy = f[EQ + e * nq + q], fz = f[2 * EQ + e * nq + q];
#pragma unroll
        for (int a = 0; a < 6; ++a) {
            const int i = edge_v(a, 0), j = edge_v(a, 1);
            double dot = 0.0;
            dot += (lam[i] * b[j][0] - lam[j] * b[i][0]) * idet * fx;
            dot += (lam[i] * b[j][1] - lam[j] * b[i][1]) * idet * fy;
            dot += (lam[i] * b[j][2] - lam[j] * b[i][2]) * idet * fz;
            acc[a] += dot * dx;
        }
    }
#pragma unroll
    for (int a = 0; a < 6; ++a) le[e * 6 + a] = (double)signs[a * ne + e] * acc[a];
}

}  // namespace
}  // namespace skg

using namespace skg;

extern "C" int skg_edge_topology(const int32_t *d_t, int64_t ne, int32_t *d_edges, int32_t *d_elem_edges,
                                 int8_t *d_signs, int64_t *h_n_edges, int64_t *h_bad_cell, void *stream) {
    return guarded([&] {
        require(ne >= 0 && (ne == 0 || (d_t && d_edges && d_elem_edges && d_signs)), "invalid edge topology arguments");
        require(ne * 6 < INT_MAX, "mesh too large for 32-bit edge items");
        if (h_bad_cell) *h_bad_cell = -1;
        if (h_n_edges) *h_n_edges = 0;
        if (ne == 0) return;
        cudaStream_t s = as_stream(stream);
        const int64_t items = ne * 6;
        uint64_t cap = 64;
        while (cap < (uint64_t)(2 * items)) cap <<= 1;
        DevBuf<unsigned long long> keys(cap, s);
        DevBuf<int32_t> first(cap, s), flag(items + 1, s), slot_of(items, s), scan(items + 1, s), misc(2, s);
        SKG_CUDA(cudaMemsetAsync(keys.get(), 0xff, cap * 8, s));
        SKG_CUDA(cudaMemsetAsync(first.get(), 0x7f, cap * 4, s));
        const int32_t init[2] = {INT_MAX, 0};
        SKG_CUDA(cudaMemcpyAsync(misc.get(), init, 8, cudaMemcpyHostToDevice, s));
        k_edge_insert<<<grid_for(items, 256), 256, 0, s>>>(d_t, ne, keys.get(), first.get(), cap - 1, misc.get(),
                                                          misc.get() + 1);
        SKG_LAUNCH_CHECK("edge_insert");
        int32_t h_misc[2];
        SKG_CUDA(cudaMemcpyAsync(h_misc, misc.get(), 8, cudaMemcpyDeviceToHost, s));
        SKG_CUDA(cudaStreamSynchronize(s));
        if (h_misc[0] != INT_MAX) {
            if (h_bad_cell) *h_bad_cell = h_misc[0];
            fail(SKG_EINVAL, "cell " + std::to_string(h_misc[0]) + " repeats a corner vertex");
        }
        require(h_misc[1] == 0, "edge hash table overflow", SKG_ECUDA);
        k_edge_flag<<<grid_for(items, 256), 256, 0, s>>>(d_t, ne, keys.get(), first.get(), cap - 1, flag.get(),
                                                        slot_of.get());
        SKG_LAUNCH_CHECK("edge_flag");
        exclusive_scan_i32(flag.get(), scan.get(), items, s);
        k_edge_emit<<<grid_for(items, 256), 256, 0, s>>>(d_t, ne, first.get(), slot_of.get(), flag.get(), scan.get(),
                                                        d_edges, d_elem_edges, d_signs);
        SKG_LAUNCH_CHECK("edge_emit");
        int32_t n_edges = 0;
        SKG_CUDA(cudaMemcpyAsync(&n_edges, scan.get() + items, 4, cudaMemcpyDeviceToHost, s));
        SKG_CUDA(cudaStreamSynchronize(s));
        if (h_n_edges) *h_n_edges = n_edges;
    });
}

static void n1_table(int nq, const double *X, const double *W, N1Table &tab) {
    static const int edges[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
    // d^{k}_a: for directed edge (i, j), phi = lambda_i g_j - lambda_j g_i,
    // so the coefficient of g_i is -lambda_j (support slot 0) and of g_j is
    // lambda_i (support slot 1).
    auto d = [&](int a, int slot, int q) {
        const double x = X[q], y = X[nq + q], z = X[2 * nq + q];
        const double lam[4] = {1.0 - x - y - z, x, y, z};
        const int i = edges[a][0], j = edges[a][1];
        return slot == 0 ? -lam[j] : lam[i];
    };
    tab.wsum = 0.;
    for (int q = 0; q < nq; ++q) tab.wsum += W[q];
    for (int a = 0; a < 6; ++a)
        for (int c = 0; c < 6; ++c)
            for (int u = 0; u < 2; ++u)
                for (int v = 0; v < 2; ++v) {
                    double acc = 0.;
                    for (int q = 0; q < nq; ++q) acc += W[q] * d(a, u, q) * d(c, v, q);
                    tab.Tm[a][c][u * 2 + v] = acc;
                }
}

namespace skg {
namespace {

// Element matrices by the closed form, then CSR row sums.  h_values
// (optional, page-locked host): the values are also copied there; on a
// row-grouped pattern the element and row passes then interleave over row
// chunks so that the copies overlap them (run_passes).
void n1_assemble(const skg_pattern *pat, const double *d_p, int64_t npts, const int32_t *d_t, const int8_t *d_signs,
                 int64_t ne, int32_t nq, const double *h_X, const double *h_W, const double *d_mass,
                 const double *d_curl, int32_t include_mass, int32_t include_curl, int32_t precision,
                 double *d_values, double *h_values, cudaStream_t s) {
    N1Table tab;
    n1_table(nq, h_X, h_W, tab);
    DevBuf<double> Ke((size_t)ne * 36, s);
    auto elem64 = [&](int64_t e0, int64_t e1) {
        k_n1_elem_fast<<<grid_for(e1 - e0, kN1Block), kN1Block, 0, s>>>(ne, e0, e1, d_p, npts, d_t, d_signs, tab,
                                                                      d_mass, d_curl, include_mass, include_curl,
                                                                      Ke.get());
        SKG_LAUNCH_CHECK("n1_element");
    };
    auto rows = [&](const GroupSet &gs, cudaStream_t st) { add_element_rows<6>(pat, Ke.get(), d_values, st, gs); };
    const bool groups = pat->max_row_len > 0;
    if (precision == SKG_SPLIT_FP32 && ne) {
        // element pass in split precision over all elements first (its range
        // check decides whether the FP64 pass replaces it), then the row pass
        N1TableF tf;
        for (int a = 0; a < 6; ++a)
            for (int c = 0; c < 6; ++c)
                for (int k = 0; k < 4; ++k) {
                    const double v = tab.Tm[a][c][k];
                    const float h = (float)v;
                    tf.Tm[a][c][k] = make_float2(h, (float)(v - (double)h));
                }
        const float wh = (float)tab.wsum;
        tf.wsum = make_float2(wh, (float)(tab.wsum - (double)wh));
        DevBuf<int> misc(2, s);  // [0] scale exponent, [1] range flag
        const int init[2] = {INT_MIN, 0};
        SKG_CUDA(cudaMemcpyAsync(misc.get(), init, sizeof(init), cudaMemcpyHostToDevice, s));
        launch_scale_exponent(d_p, 3 * npts, misc.get(), s);
        k_n1_elem_df<<<grid_for(ne, kN1Block), kN1Block, 0, s>>>(ne, 0, ne, d_p, npts, d_t, d_signs, tf, d_mass,
                                                                 d_curl, include_mass, include_curl, misc.get(),
                                                                 misc.get() + 1, Ke.get());
        SKG_LAUNCH_CHECK("n1_element_df");
        int h_misc[2];
        SKG_CUDA(cudaMemcpyAsync(h_misc, misc.get(), sizeof(h_misc), cudaMemcpyDeviceToHost, s));
        SKG_CUDA(cudaStreamSynchronize(s));
        if (h_misc[1] != 0 || h_misc[0] == INT_MIN) elem64(0, ne);  // out of FP32 range: FP64 instead
        if (groups) {
            run_row_pass(pat, d_values, h_values, s, rows);
            return;
        }
    } else if (h_values && groups) {
        run_passes(pat, ne, d_values, h_values, s, elem64, rows);
        return;
    } else if (ne) {
        elem64(0, ne);
    }
    gather_element_matrices(pat, Ke.get(), d_values, s);
    if (h_values && pat->nnz)
        SKG_CUDA(cudaMemcpyAsync(h_values, d_values, (size_t)pat->nnz * sizeof(double), cudaMemcpyDeviceToHost, s));
}

}  // namespace
}  // namespace skg

extern "C" int skg_n1_assemble(const skg_pattern *pat, const double *d_p, int64_t npts, const int32_t *d_t,
                               const int32_t *d_elem_edges, const int8_t *d_signs, int64_t ne, int32_t nq,
                               const double *h_X, const double *h_W, const double *d_mass, const double *d_curl,
                               int32_t include_mass, int32_t include_curl, int32_t precision, double *d_values,
                               void *stream) {
    return guarded([&] {
        require(pat != nullptr, "pattern is NULL");
        require(ne == pat->n_elements && pat->row_local == 6 && pat->col_local == 6, "mesh does not match the pattern");
        require(nq > 0 && h_X && h_W, "quadrature rule is empty");
        require(ne == 0 || (d_p && d_t && d_signs), "mesh arrays are NULL");
        (void)d_elem_edges;
        n1_assemble(pat, d_p, npts, d_t, d_signs, ne, nq, h_X, h_W, d_mass, d_curl, include_mass, include_curl,
                    precision, d_values, nullptr, as_stream(stream));
    });
}

extern "C" int skg_n1_assemble_host(const skg_pattern *pat, const double *d_p, int64_t npts, const int32_t *d_t,
                                    const int32_t *d_elem_edges, const int8_t *d_signs, int64_t ne, int32_t nq,
                                    const double *h_X, const double *h_W, const double *d_mass, const double *d_curl,
                                    int32_t include_mass, int32_t include_curl, int32_t precision, double *d_values,
                                    double *h_values, void *stream) {
    return guarded([&] {
        require(pat != nullptr, "pattern is NULL");
        require(ne == pat->n_elements && pat->row_local == 6 && pat->col_local == 6, "mesh does not match the pattern");
        require(nq > 0 && h_X && h_W, "quadrature rule is empty");
        require(ne == 0 || (d_p && d_t && d_signs), "mesh arrays are NULL");
        require(d_values && h_values, "device staging or host output is NULL");
        (void)d_elem_edges;
        n1_assemble(pat, d_p, npts, d_t, d_signs, ne, nq, h_X, h_W, d_mass, d_curl, include_mass, include_curl,
                    precision, d_values, h_values, as_stream(stream));
    });
}

// Per-point coefficients (mass/curl (E, Q)): explicit quadrature loop.
extern "C" int skg_n1_assemble_pointwise(const skg_pattern *pat, const double *d_p, int64_t npts,
                                         const int32_t *d_t, const int8_t *d_signs, int64_t ne, int32_t nq,
                                         const double *h_X, const double *h_W, const double *d_mass,
                                         const double *d_curl, int32_t include_mass, int32_t include_curl,
                                         double *d_values, void *stream) {
    return guarded([&] {
        require(pat != nullptr, "pattern is NULL");
        require(ne == pat->n_elements && pat->row_local == 6 && pat->col_local == 6, "mesh does not match the pattern");
        require(nq > 0 && h_X && h_W, "quadrature rule is empty");
        cudaStream_t s = as_stream(stream);
        N1Table tab;
        n1_table(nq, h_X, h_W, tab);
        std::vector<double> xw(4 * (size_t)nq);
        for (int i = 0; i < 3 * nq; ++i) xw[i] = h_X[i];
        for (int q = 0; q < nq; ++q) xw[3 * nq + q] = h_W[q];
        DevBuf<double> dxw(xw.size(), s);
        SKG_CUDA(cudaMemcpyAsync(dxw.get(), xw.data(), xw.size() * 8, cudaMemcpyHostToDevice, s));
        DevBuf<double> Ke((size_t)ne * 36, s);
        if (ne) {
            k_n1_element<<<grid_for(ne, 128), 128, 0, s>>>(ne, d_p, npts, d_t, d_signs, nq, dxw.get(),
                                                                 dxw.get() + 3 * nq, tab, d_mass, d_curl, 1,
                                                                 include_mass, include_curl, Ke.get());
            SKG_LAUNCH_CHECK("n1_element_pointwise");
        }
        gather_element_matrices(pat, Ke.get(), d_values, s);
    });
}

extern "C" int skg_n1_vector_load(const skg_pattern *pat, const double *d_p, int64_t npts, const int32_t *d_t,
                                  const int8_t *d_signs, int64_t ne, int32_t nq, const double *h_X, const double *h_W,
                                  const double *d_f, double *d_out, void *stream) {
    return guarded([&] {
        require(pat != nullptr, "pattern is NULL");
        require(ne == pat->n_elements && pat->row_local == 6, "mesh does not match the pattern");
        require(nq > 0 && h_X && h_W, "quadrature rule is empty");
        require(d_p && d_t && d_signs && d_f && d_out, "mesh, load or output arrays are NULL");
        cudaStream_t s = as_stream(stream);
        std::vector<double> xw(4 * (size_t)nq);
        for (int i = 0; i < 3 * nq; ++i) xw[i] = h_X[i];
        for (int q = 0; q < nq; ++q) xw[3 * nq + q] = h_W[q];
        DevBuf<double> dxw(xw.size(), s), le((size_t)ne * 6, s);
        SKG_CUDA(cudaMemcpyAsync(dxw.get(), xw.data(), xw.size() * 8, cudaMemcpyHostToDevice, s));
        if (ne) {
            k_n1_load<<<grid_for(ne, 128), 128, 0, s>>>(ne, d_p, npts, d_t, d_signs, nq, dxw.get(), dxw.get() + 3 * nq,
                                                       d_f, le.get());
            SKG_LAUNCH_CHECK("n1_load");
        }
        gather_element_vectors(pat, le.get(), d_out, s);
    });
}

// ------------------------------------------------------------------ basis evaluation

// A global edge field at the rule's points, component-first (3, E, Q):
// values sum_a u[dof(e, a)] s_a (lam_i b_j - lam_j b_i) / det J (covariant
// Piola of the Whitney functions, b_k = det J grad lam_k), curls
// sum_a u[dof(e, a)] s_a J c_a / det J.  One thread per (element, point).
__global__ void k_n1_evaluate(int64_t ne, const double *__restrict__ p, int64_t npts, const int32_t *__restrict__ t,
                              const int32_t *__restrict__ elem_edges, const int8_t *__restrict__ signs,
                              int64_t n_edges, int nq, const double *__restrict__ Xq,
                              const double *__restrict__ coef, int want_curl, double *__restrict__ out) {
    const int64_t total = ne * nq;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const int64_t e = i / nq;
    const int q = (int)(i - e * nq);
    double J[9], b[4][3], det;
    n1_geometry(p, npts, t, ne, e, J, b, det);
    double u[6];
    for (int a = 0; a < 6; ++a) {
        const int32_t d = elem_edges[a * ne + e];
        // an edge id outside [0, n_edges) never reaches memory: the point becomes NaN
        u[a] = d >= 0 && d < n_edges ? coef[d] * (double)signs[a * ne + e] : __longlong_as_double(0x7ff8000000000000LL);
    }
    double v[3] = {0.0, 0.0, 0.0};
    if (want_curl) {
        for (int a = 0; a < 6; ++a)
            for (int r = 0; r < 3; ++r)
                v[r] += u[a] * (J[r * 3 + 0] * kRefCurl[a][0] + J[r * 3 + 1] * kRefCurl[a][1] +
                                J[r * 3 + 2] * kRefCurl[a][2]);
    } else {
        const double x = Xq[q], y = Xq[nq + q], z = Xq[2 * nq + q];
        const double lam[4] = {1.0 - x - y - z, x, y, z};
        for (int a = 0; a < 6; ++a) {
            const int k = kEdge[a][0], l = kEdge[a][1];
            for (int r = 0; r < 3; ++r) v[r] += u[a] * (lam[k] * b[l][r] - lam[l] * b[k][r]);
        }
    }
    const double inv = 1.0 / det;  // both sums carry the factor 1 / det J
    out[i] = v[0] * inv;
    out[total + i] = v[1] * inv;
    out[2 * total + i] = v[2] * inv;
}

// Points along each global edge, x = p_first + (p_second - p_first) t_q,
// component-first (3, n_edges * nq), edge-major.  Rounded as the product
// then the sum (no fused multiply-add), as the same expression on the host.
__global__ void k_edge_points(int64_t n_edges, int nq, const double *__restrict__ p, int64_t npts,
                              const int32_t *__restrict__ edges, const double *__restrict__ param,
                              double *__restrict__ out) {
    const int64_t total = n_edges * nq;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const int64_t k = i / nq;
    const int q = (int)(i - k * nq);
    const int32_t a = edges[k], b = edges[n_edges + k];
    const bool ok = a >= 0 && a < npts && b >= 0 && b < npts;
    for (int r = 0; r < 3; ++r) {
        const double first = ok ? p[r * npts + a] : __longlong_as_double(0x7ff8000000000000LL);
        const double tangent = ok ? __dsub_rn(p[r * npts + b], first) : first;
        out[r * total + i] = __dadd_rn(first, __dmul_rn(tangent, param[q]));
    }
}

// Tangential moments m_k = sum_q w_q f(x_q) . (p_second - p_first) of a
// field sampled at k_edge_points' points, one thread per edge.
__global__ void k_edge_moments(int64_t n_edges, int nq, const double *__restrict__ p, int64_t npts,
                               const int32_t *__restrict__ edges, const double *__restrict__ weights,
                               const double *__restrict__ f, double *__restrict__ out) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_edges) return;
    const int32_t a = edges[k], b = edges[n_edges + k];
    if (!(a >= 0 && a < npts && b >= 0 && b < npts)) {
        out[k] = __longlong_as_double(0x7ff8000000000000LL);
        return;
    }
    const int64_t total = n_edges * nq;
    double tangent[3];
    for (int r = 0; r < 3; ++r) tangent[r] = p[r * npts + b] - p[r * npts + a];
    double m = 0.0;
    for (int q = 0; q < nq; ++q) {
        const int64_t i = k * nq + q;
        m += weights[q] * (f[i] * tangent[0] + f[total + i] * tangent[1] + f[2 * total + i] * tangent[2]);
    }
    out[k] = m;
}

extern "C" int skg_n1_element_matrices(const double *d_p, int64_t npts, const int32_t *d_t, const int8_t *d_signs,
                                       int64_t ne, int32_t nq, const double *h_X, const double *h_W,
                                       const double *d_mass, const double *d_curl, int32_t coef_per_point,
                                       int32_t include_mass, int32_t include_curl, double *d_out, void *stream) {
    return guarded([&] {
        require(ne >= 0 && nq > 0 && h_X && h_W, "quadrature rule is empty");
        require(coef_per_point == 0 || coef_per_point == 1, "coefficient layout must be 0 (per element) or 1 (per point)");
        require(ne == 0 || (d_p && d_t && d_signs && d_out), "mesh or output arrays are NULL");
        if (ne == 0) return;
        cudaStream_t s = as_stream(stream);
        N1Table tab;
        n1_table(nq, h_X, h_W, tab);
        if (!coef_per_point) {
            k_n1_elem_fast<<<grid_for(ne, kN1Block), kN1Block, 0, s>>>(ne, 0, ne, d_p, npts, d_t, d_signs, tab,
                                                                      d_mass, d_curl, include_mass, include_curl,
                                                                      d_out);
            SKG_LAUNCH_CHECK("n1_element_matrices");
            return;
        }
        std::vector<double> xw(4 * (size_t)nq);
        for (int i = 0; i < 3 * nq; ++i) xw[i] = h_X[i];
        for (int q = 0; q < nq; ++q) xw[3 * nq + q] = h_W[q];
        DevBuf<double> dxw(xw.size(), s);
        SKG_CUDA(cudaMemcpyAsync(dxw.get(), xw.data(), xw.size() * 8, cudaMemcpyHostToDevice, s));
        k_n1_element<<<grid_for(ne, 128), 128, 0, s>>>(ne, d_p, npts, d_t, d_signs, nq, dxw.get(), dxw.get() + 3 * nq,
                                                       tab, d_mass, d_curl, 1, include_mass, include_curl, d_out);
        SKG_LAUNCH_CHECK("n1_element_matrices_pointwise");
    });
}

extern "C" int skg_n1_evaluate(const double *d_p, int64_t npts, const int32_t *d_t, const int32_t *d_elem_edges,
                               const int8_t *d_signs, int64_t ne, int64_t n_edges, int32_t nq, const double *h_X,
                               const double *d_coefficients, int32_t curl, double *d_out, void *stream) {
    return guarded([&] {
        require(ne >= 0 && n_edges >= 0 && nq > 0 && h_X, "quadrature rule is empty");
        require(ne == 0 || (d_p && d_t && d_elem_edges && d_signs && d_coefficients && d_out),
                "mesh, coefficient or output arrays are NULL");
        if (ne == 0) return;
        cudaStream_t s = as_stream(stream);
        DevBuf<double> dX(3 * (size_t)nq, s);
        SKG_CUDA(cudaMemcpyAsync(dX.get(), h_X, 3 * (size_t)nq * 8, cudaMemcpyHostToDevice, s));
        k_n1_evaluate<<<grid_for(ne * nq, 256), 256, 0, s>>>(ne, d_p, npts, d_t, d_elem_edges, d_signs, n_edges, nq,
                                                            dX.get(), d_coefficients, curl != 0, d_out);
        SKG_LAUNCH_CHECK("n1_evaluate");
    });
}

extern "C" int skg_n1_edge_points(const double *d_p, int64_t npts, const int32_t *d_edges, int64_t n_edges,
                                  int32_t nq, const double *h_param, double *d_out, void *stream) {
    return guarded([&] {
        require(n_edges >= 0 && nq > 0 && h_param, "edge rule is empty");
        require(n_edges == 0 || (d_p && d_edges && d_out), "mesh, edge or output arrays are NULL");
        if (n_edges == 0) return;
        cudaStream_t s = as_stream(stream);
        DevBuf<double> dt((size_t)nq, s);
        SKG_CUDA(cudaMemcpyAsync(dt.get(), h_param, (size_t)nq * 8, cudaMemcpyHostToDevice, s));
        k_edge_points<<<grid_for(n_edges * nq, 256), 256, 0, s>>>(n_edges, nq, d_p, npts, d_edges, dt.get(), d_out);
        SKG_LAUNCH_CHECK("edge_points");
    });
}

extern "C" int skg_n1_edge_moments(const double *d_p, int64_t npts, const int32_t *d_edges, int64_t n_edges,
                                   int32_t nq, const double *h_weights, const double *d_values, double *d_out,
                                   void *stream) {
    return guarded([&] {
        require(n_edges >= 0 && nq > 0 && h_weights, "edge rule is empty");
        require(n_edges == 0 || (d_p && d_edges && d_values && d_out), "mesh, edge, field or output arrays are NULL");
        if (n_edges == 0) return;
        cudaStream_t s = as_stream(stream);
        DevBuf<double> dw((size_t)nq, s);
        SKG_CUDA(cudaMemcpyAsync(dw.get(), h_weights, (size_t)nq * 8, cudaMemcpyHostToDevice, s));
        k_edge_moments<<<grid_for(n_edges, 256), 256, 0, s>>>(n_edges, nq, d_p, npts, d_edges, dw.get(), d_values,
                                                             d_out);
        SKG_LAUNCH_CHECK("edge_moments");
    });
}
