// Fused assembly of scalar P1/P2 diffusion on affine tetrahedra -- the hot
// path of `asm(BilinearForm, Basis)` for w.kappa * ddot(grad u, grad v) and
// dot(mul(A, grad u), grad v) (python/skfemntv/forms.py:276-374 through
// bilinear_form_assembler.cpp:79-105 / cross_bilinear_assembler.cpp:207-247).
//
// Math.  On an affine tetrahedron every P1/P2 basis gradient is a linear
// combination of the four barycentric gradients g_k = b_k / det J (b_k the
// rows of adj J, b_0 = -(b_1+b_2+b_3)):  grad N_a = sum_k c^k_a(xi) g_k with
// c^k_a = delta_ka (P1), (4 lambda_a - 1) delta_ka (P2 vertex) and
// 4 lambda_j, 4 lambda_i on the ends of P2 edge (i, j)
// (python/skfemntv/basis.py:2224-2235).  Hence
//     K_ab = sum_{k,l} G_kl T^{kl}_ab,   G_kl = b_k . A b_l / |det J|,
//     T^{kl}_ab = sum_q w_q c^k_a(xi_q) c^l_b(xi_q),
// T tabulated on the host from the caller's quadrature rule (same rule, same
// sum as the reference, reassociated).  Only (k, l) in the supports of a and
// b contribute: 1 term for vertex-vertex, 2 vertex-edge, 4 edge-edge.
//
// Passes.
//  1. element pass (thread per element): G (4x4) from coordinates and the
//     coefficient, written to a scratch array.
//  2. row pass (thread per CSR row, warp per group of up to 32 rows): the
//     thread walks its row's incidence records (element, local row, column
//     offsets) in ascending element order, evaluates row a of K_e on the fly
//     and adds it into shared-memory accumulators of the row's slots; the
//     warp then writes the group's slot range with coalesced stores.  Every
//     slot is summed by one thread in a fixed order: results are bitwise
//     reproducible, with no atomics.
//
// Precision modes.
//  SKG_FP64           FP64 end to end (FP64 pipe).
//  SKG_FP64_EMULATED  element pass and row pass in double-float (FP32 pairs,
//                     error-free transformations; ~48-bit significands) and
//                     slot sums in double-float, converted to FP64 exactly:
//                     FP64-accurate (1e-12 class) on the FP32 pipe.
//  SKG_SPLIT_FP32     double-float element pass (FP64-class G), element
//                     contraction in FP32 with split hi/lo products and FP32
//                     accumulation, double-float slot sums.
// The FP32-pair modes work in units scaled by 2^-s (s from the largest
// vertex coordinate) so FP32 range holds; a mesh or coefficient outside that
// range is detected in the element pass and re-run in FP64.
#include <algorithm>
#include <climits>
#include <mutex>
#include <string>
#include <type_traits>
#include <cmath>
#include <vector>

#include "skg_common.cuh"
#include "skg_df64.cuh"
#include "skg_rows.cuh"

namespace skg {
namespace {

struct Support {
    int sup[10][2];
};

// Barycentric support of local basis function b: P1 and P2 vertex functions
// use lambda_b; P2 edge function 4 + k uses the two end vertices of edge k
// ((0,1),(1,2),(2,0),(0,3),(1,3),(2,3)).  Compile-time so that unrolled
// loops index registers, not local memory.
__host__ __device__ constexpr int sup_lo(int b) {
    return b < 4 ? b : (b == 4 ? 0 : b == 5 ? 1 : b == 6 ? 2 : b == 7 ? 0 : b == 8 ? 1 : 2);
}
__host__ __device__ constexpr int sup_hi(int b) {
    return b < 4 ? b : (b == 4 ? 1 : b == 5 ? 2 : b == 6 ? 0 : 3);
}

// ------------------------------------------------------------ geometry

__device__ __forceinline__ bool load_vertices(const int32_t *__restrict__ t, int64_t ne, int64_t e, int64_t npts,
                                              int32_t v[4]) {
    v[0] = t[e];
    v[1] = t[ne + e];
    v[2] = t[2 * ne + e];
    v[3] = t[3 * ne + e];
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 4; ++k) ok = ok && v[k] >= 0 && v[k] < npts;
    if (!ok) v[0] = v[1] = v[2] = v[3] = 0;
    return ok;
}

__device__ __forceinline__ double load_coef(const double *__restrict__ coef, int coef_kind, int64_t ne, int64_t e,
                                            int k) {
    // coef_kind 1: (E,3,3) row-major; 2: component-first (3,3,E)
    return coef_kind == 1 ? coef[e * 9 + k] : coef[(int64_t)k * ne + e];
}

constexpr int kElemBlock = 128;
constexpr int kStagePad = 9;  // 8 x 16-byte chunks per element + 1 pad (bank-conflict-free staging)

// Writes the block's staged G rows (8 x 16 bytes per element) to global
// memory with coalesced 16-byte stores.
__device__ __forceinline__ void flush_stage(const float4 *stage, float4 *Gout, int64_t e0, int64_t ne) {
    __syncthreads();
    const int64_t rest = ne - e0;
    const int64_t nvalid = rest < kElemBlock ? rest : (int64_t)kElemBlock;
    float4 *dst = Gout + e0 * 8;
    for (int i = threadIdx.x; i < nvalid * 8; i += kElemBlock) dst[i] = stage[(i >> 3) * kStagePad + (i & 7)];
}

// Off-diagonal pair (a, b) of a coefficient whose largest diagonal entry has
// biased exponent emax, decided on the bits: same sign, finite, and at most
// 2^(emax - e + 5) units in the last place apart, e the larger biased exponent
// of the pair (at least 1).  Then |a - b| <= 2^(emax - 1070) < 1e-14 |A_dd|,
// so a pair that passes also passes the floating-point test of
// coef_symmetric; a pair that fails goes to that test.  Integer instructions
// only, in place of FP64 additions, a multiplication and comparisons on the
// FP64 pipe.
__device__ __forceinline__ bool bits_close(double a, double b, int emax) {
    const unsigned long long ia = (unsigned long long)__double_as_longlong(a);
    const unsigned long long ib = (unsigned long long)__double_as_longlong(b);
    const unsigned long long ma = ia & 0x7fffffffffffffffull, mb = ib & 0x7fffffffffffffffull;
    const int e = max(max((int)(ma >> 52), (int)(mb >> 52)), 1);
    if (((ia ^ ib) >> 63) != 0 || e == 0x7ff || emax == 0x7ff) return false;
    const unsigned long long d = ma > mb ? ma - mb : mb - ma;
    const int sh = emax - e + 5;
    if (sh < 0) return d == 0;
    return sh >= 63 || d <= (1ull << sh);
}

// A (3 x 3, row-major) symmetric to 1e-14 of its size: |A_kl - A_lk| <=
// 1e-14 (|A_00| + |A_11| + |A_22| + |A_01| + |A_02| + |A_12|) for the three
// off-diagonal pairs (a tensor built as Q D Q^T in floating point is not
// bitwise symmetric; mirroring K_ab into K_ba then changes entries by ~1e-16
// relative).  The bit test decides first; the same decision as the
// floating-point test alone.
__device__ __forceinline__ bool coef_symmetric(const double A[9]) {
    const auto bexp = [](double x) { return (int)((__double_as_longlong(x) >> 52) & 0x7ff); };
    const int emax = max(max(bexp(A[0]), bexp(A[4])), bexp(A[8]));
    if (bits_close(A[1], A[3], emax) && bits_close(A[2], A[6], emax) && bits_close(A[5], A[7], emax)) return true;
    const double scale = 1e-14 * (fabs(A[0]) + fabs(A[4]) + fabs(A[8]) + fabs(A[1]) + fabs(A[2]) + fabs(A[5]));
    return fabs(A[1] - A[3]) <= scale && fabs(A[2] - A[6]) <= scale && fabs(A[5] - A[7]) <= scale;
}

// G_kl = b_k . A b_l / |det J| of element e in FP64 (b: adjugate rows, the
// scaled barycentric gradients).  Only the block k, l >= 1 takes dot products
// (its upper triangle when A is symmetric): b_0 = -(b_1 + b_2 + b_3) gives
// G_0l = -(G_1l + G_2l + G_3l), G_k0 likewise and G_00 = -(G_01 + G_02 + G_03);
// gscale / |det J| scales the dot products of that block (6 of them when A
// is symmetric, where scaling A would take 9).  Returns the element's
// symmetry (scalar coefficient, or a tensor equal to its transpose).
__device__ __forceinline__ bool elem_g_fp64(int64_t ne, const double *__restrict__ p, int64_t npts,
                                            const int32_t *__restrict__ t, int coef_kind,
                                            const double *__restrict__ coef, int64_t e, double g[16],
                                            double gscale = 1.0) {
    int32_t v[4];
    const bool ok = load_vertices(t, ne, e, npts, v);
    double J[9];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const double x0 = p[i * npts + v[0]];
#pragma unroll
        for (int r = 0; r < 3; ++r) J[i * 3 + r] = p[i * npts + v[r + 1]] - x0;
    }
    double b[4][3];
    b[1][0] = J[4] * J[8] - J[5] * J[7];
    b[1][1] = J[2] * J[7] - J[1] * J[8];
    b[1][2] = J[1] * J[5] - J[2] * J[4];
    b[2][0] = J[5] * J[6] - J[3] * J[8];
    b[2][1] = J[0] * J[8] - J[2] * J[6];
    b[2][2] = J[2] * J[3] - J[0] * J[5];
    b[3][0] = J[3] * J[7] - J[4] * J[6];
    b[3][1] = J[1] * J[6] - J[0] * J[7];
    b[3][2] = J[0] * J[4] - J[1] * J[3];
    const double det = J[0] * b[1][0] + J[1] * b[2][0] + J[2] * b[3][0];
    const double inv = ok ? gscale / fabs(det) : __longlong_as_double(0x7ff8000000000000LL);
    bool sym = true;
    if (coef_kind == 0) {
        const double sc = (coef ? coef[e] : 1.0) * inv;
#pragma unroll
        for (int k = 1; k < 4; ++k)
#pragma unroll
            for (int l = k; l < 4; ++l) {
                const double val = sc * (b[k][0] * b[l][0] + b[k][1] * b[l][1] + b[k][2] * b[l][2]);
                g[k * 4 + l] = val;
                g[l * 4 + k] = val;
            }
    } else {
        double A[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) A[k] = load_coef(coef, coef_kind, ne, e, k);
        sym = coef_symmetric(A);
#pragma unroll
        for (int l = 1; l < 4; ++l) {
            double Ab[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) Ab[i] = A[i * 3] * b[l][0] + A[i * 3 + 1] * b[l][1] + A[i * 3 + 2] * b[l][2];
#pragma unroll
            for (int k = 1; k < 4; ++k) {
                if (k > l && sym) continue;  // mirrored below
                g[k * 4 + l] = inv * (b[k][0] * Ab[0] + b[k][1] * Ab[1] + b[k][2] * Ab[2]);
            }
        }
        if (sym) {
#pragma unroll
            for (int k = 2; k < 4; ++k)
#pragma unroll
                for (int l = 1; l < k; ++l) g[k * 4 + l] = g[l * 4 + k];
        }
    }
#pragma unroll
    for (int l = 1; l < 4; ++l) g[l] = -(g[4 + l] + g[8 + l] + g[12 + l]);
    if (sym) {
#pragma unroll
        for (int k = 1; k < 4; ++k) g[k * 4] = g[k];
    } else {
#pragma unroll
        for (int k = 1; k < 4; ++k) g[k * 4] = -(g[k * 4 + 1] + g[k * 4 + 2] + g[k * 4 + 3]);
    }
    g[0] = -(g[1] + g[2] + g[3]);
    return sym;
}

__global__ void __launch_bounds__(kElemBlock) k_elem_fp64(int64_t ne, const double *__restrict__ p, int64_t npts,
                                                          const int32_t *__restrict__ t, int coef_kind,
                                                          const double *__restrict__ coef, float4 *__restrict__ G) {
    __shared__ float4 stage[kElemBlock * kStagePad];
    const int64_t e0 = (int64_t)blockIdx.x * kElemBlock;
    const int64_t e = e0 + threadIdx.x;
    if (e < ne) {
        double g[16];
        elem_g_fp64(ne, p, npts, t, coef_kind, coef, e, g);
        double2 *st = reinterpret_cast<double2 *>(stage + threadIdx.x * kStagePad);
#pragma unroll
        for (int m = 0; m < 8; ++m) st[m] = make_double2(g[2 * m], g[2 * m + 1]);
    }
    flush_stage(stage, G, e0, ne);
}

// P2 element matrices in FP64 (the FP64 mode on row-grouped patterns): the
// element pass evaluates K_ab = sum G T over the supports once per entry,
// the 55 entries of the upper triangle only when the element's coefficient
// is symmetric to rounding (then K is), and writes the full 10 x 10 matrix; the row
// pass only adds rows.  This halves the FP64 multiply-adds of the
// row-by-row evaluation, whose rows a and b each recompute K_ab.
constexpr int kKeBlock = 128;
constexpr int kKeChunk = 25;  // entries staged per round; 4 rounds cover the 100

__host__ __device__ constexpr int tri10(int a, int b) {  // packed upper triangle, a <= b
    return a * 10 - a * (a - 1) / 2 + (b - a);
}

__global__ void __launch_bounds__(kKeBlock) k_elem_ke_fp64(int64_t ne, int64_t e_begin, int64_t e_end,
                                                           const double *__restrict__ p, int64_t npts,
                                                           const int32_t *__restrict__ t, int coef_kind,
                                                           const double *__restrict__ coef,
                                                           const double *__restrict__ Tg, double *__restrict__ Ke) {
    __shared__ double Ts[10 * 10 * 4];
    __shared__ double stage[kKeBlock * kKeChunk];
    for (int i = threadIdx.x; i < 400; i += blockDim.x) Ts[i] = Tg[i];
    __syncthreads();
    const int64_t e0 = e_begin + (int64_t)blockIdx.x * kKeBlock;
    const int64_t e = e0 + threadIdx.x;
    const bool valid = e < e_end;
    double g[16];
    bool sym = true;
    if (valid) {
        sym = elem_g_fp64(ne, p, npts, t, coef_kind, coef, e, g);
    } else {
#pragma unroll
        for (int k = 0; k < 16; ++k) g[k] = 0.0;
    }
    auto entry = [&](int a, int bb) -> double {
        const int ka0 = sup_lo(a), ka1 = sup_hi(a), kb0 = sup_lo(bb), kb1 = sup_hi(bb);
        const double *T = Ts + (a * 10 + bb) * 4;
        double v = g[ka0 * 4 + kb0] * T[0];
        if (kb1 != kb0) v += g[ka0 * 4 + kb1] * T[1];
        if (ka1 != ka0) {
            v += g[ka1 * 4 + kb0] * T[2];
            if (kb1 != kb0) v += g[ka1 * 4 + kb1] * T[3];
        }
        return v;
    };
    double U[55];
    if (sym) {
#pragma unroll
        for (int a = 0; a < 10; ++a)
#pragma unroll
            for (int bb = a; bb < 10; ++bb) U[tri10(a, bb)] = entry(a, bb);
    }
    const int nvalid = (int)(e_end - e0 < kKeBlock ? e_end - e0 : kKeBlock);
    double *st = stage + threadIdx.x * kKeChunk;
#pragma unroll
    for (int r = 0; r < 100 / kKeChunk; ++r) {
        if (sym) {
#pragma unroll
            for (int q = 0; q < kKeChunk; ++q) {
                const int k = r * kKeChunk + q, a = k / 10, bb = k % 10;
                st[q] = U[a <= bb ? tri10(a, bb) : tri10(bb, a)];
            }
        } else {
#pragma unroll
            for (int q = 0; q < kKeChunk; ++q) {
                const int k = r * kKeChunk + q;
                st[q] = entry(k / 10, k % 10);
            }
        }
        __syncthreads();
        // coalesced copy-out: element rows are 100 doubles apart
        for (int i = threadIdx.x; i < nvalid * kKeChunk; i += kKeBlock) {
            const int el = i / kKeChunk, q = i - el * kKeChunk;
            Ke[(e0 + el) * 100 + r * kKeChunk + q] = stage[el * kKeChunk + q];
        }
        __syncthreads();
    }
}

// Scale exponent s: vertex coordinates times 2^-s are at most 1 in magnitude.
// The largest |x| is found on the bit patterns (for non-negative doubles the
// integer order of the bits is the numeric order), so the scan runs on the
// integer pipes; only the winner's exponent is decoded.
__global__ void k_scale(const double *__restrict__ p, int64_t n, int *__restrict__ s_out) {
    unsigned long long m = 0;
#pragma unroll 8
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long b = (unsigned long long)__double_as_longlong(p[i]) & 0x7fffffffffffffffULL;
        if (b < 0x7ff0000000000000ULL) m = b > m ? b : m;  // finite values only
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long q = __shfl_xor_sync(0xffffffffu, m, o);
        m = q > m ? q : m;
    }
    if ((threadIdx.x & 31) == 0 && m != 0) {
        const double a = __longlong_as_double((long long)m);
        atomicMax(s_out, ilogb(a) + 1);
    }
}

// Element pass in double-float.  G (scaled by 2^-s) as 16 df64.
// G (scaled by 2^-s, and by 1/30 for the exact-rule P2 path) in double-float
// for element e; `ok` false when a value leaves the FP32 range.  Returns the
// coefficient's symmetry (to 1e-14 of its size, as elem_g_fp64).
__device__ __forceinline__ bool elem_g_df64(int64_t ne, const double *__restrict__ p, int64_t npts,
                                            const int32_t *__restrict__ t, int coef_kind,
                                            const double *__restrict__ coef, int s, bool div30, int64_t e,
                                            df64 g[16], bool &ok) {
    int32_t v[4];
    ok = load_vertices(t, ne, e, npts, v);
    df64 J[9];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const double x0 = p[i * npts + v[0]];
#pragma unroll
        for (int r = 0; r < 3; ++r) J[i * 3 + r] = df_from_double(p[i * npts + v[r + 1]] - x0, -s, ok);
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
    if (det.hi < 0.f) det = df_neg(det);
    ok = ok && det.hi > 1e-30f;
    df64 inv = df_recip(det);
    // exact-rule P2 path: G / 30 (the integer table carries 30 T)
    if (div30) inv = df_mul(inv, df64{0x1.111112p-5f, -0x1.dddddep-30f});
    // as elem_g_fp64: dot products for the block k, l >= 1 only (upper triangle
    // when symmetric), row and column 0 from b_0 = -(b_1 + b_2 + b_3)
    bool sym = true;
    if (coef_kind == 0) {
        df64 sc = inv;
        if (coef) sc = df_mul(sc, df_from_double(coef[e], 0, ok));
#pragma unroll
        for (int k = 1; k < 4; ++k)
#pragma unroll
            for (int l = k; l < 4; ++l) {
                df64 d = df_add_fast(df_add_fast(df_mul(b[k][0], b[l][0]), df_mul(b[k][1], b[l][1])),
                                     df_mul(b[k][2], b[l][2]));
                d = df_mul(sc, d);
                g[k * 4 + l] = d;
                g[l * 4 + k] = d;
            }
    } else {
        double Ad[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) Ad[k] = load_coef(coef, coef_kind, ne, e, k);
        sym = coef_symmetric(Ad);
        df64 A[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) A[k] = df_mul(inv, df_from_double(Ad[k], 0, ok));
#pragma unroll
        for (int l = 1; l < 4; ++l) {
            df64 Ab[3];
#pragma unroll
            for (int i = 0; i < 3; ++i)
                Ab[i] = df_add_fast(df_add_fast(df_mul(A[i * 3], b[l][0]), df_mul(A[i * 3 + 1], b[l][1])),
                                    df_mul(A[i * 3 + 2], b[l][2]));
#pragma unroll
            for (int k = 1; k < 4; ++k) {
                if (k > l && sym) continue;  // mirrored below
                g[k * 4 + l] =
                    df_add_fast(df_add_fast(df_mul(b[k][0], Ab[0]), df_mul(b[k][1], Ab[1])), df_mul(b[k][2], Ab[2]));
            }
        }
        if (sym) {
#pragma unroll
            for (int k = 2; k < 4; ++k)
#pragma unroll
                for (int l = 1; l < k; ++l) g[k * 4 + l] = g[l * 4 + k];
        }
    }
#pragma unroll
    for (int l = 1; l < 4; ++l) g[l] = df_neg(df_add_fast(df_add_fast(g[4 + l], g[8 + l]), g[12 + l]));
    if (sym) {
#pragma unroll
        for (int k = 1; k < 4; ++k) g[k * 4] = g[k];
    } else {
#pragma unroll
        for (int k = 1; k < 4; ++k)
            g[k * 4] = df_neg(df_add_fast(df_add_fast(g[k * 4 + 1], g[k * 4 + 2]), g[k * 4 + 3]));
    }
    g[0] = df_neg(df_add_fast(df_add_fast(g[1], g[2]), g[3]));
#pragma unroll
    for (int k = 0; k < 16; ++k) ok = ok && df_in_range(g[k]);
    return sym;
}

__global__ void __launch_bounds__(kElemBlock, 6) k_elem_df64(int64_t ne, const double *__restrict__ p, int64_t npts,
                                                             const int32_t *__restrict__ t, int coef_kind,
                                                             const double *__restrict__ coef,
                                                             const int *__restrict__ s_ptr, float4 *__restrict__ G,
                                                             int *__restrict__ range_flag, bool div30) {
    __shared__ float4 stage[kElemBlock * kStagePad];
    const int64_t e0 = (int64_t)blockIdx.x * kElemBlock;
    const int64_t e = e0 + threadIdx.x;
    if (e < ne) {
        df64 g[16];
        bool ok;
        elem_g_df64(ne, p, npts, t, coef_kind, coef, *s_ptr, div30, e, g, ok);
        float2 *st = reinterpret_cast<float2 *>(stage + threadIdx.x * kStagePad);
#pragma unroll
        for (int k = 0; k < 16; ++k) st[k] = make_float2(g[k].hi, g[k].lo);
        if (!ok) atomicExch(range_flag, 1);
    }
    flush_stage(stage, G, e0, ne);
}

// ------------------------------------------------------------ row pass

enum { MODE_FP64 = 0, MODE_SPLIT = 1, MODE_DF64 = 2 };

// (hi, lo) += v without renormalising (renormalised once at write-out)
__device__ __forceinline__ void df_acc(df64 &a, df64 v) {
    const df64 sm = two_sum(a.hi, v.hi);
    a.hi = sm.hi;
    a.lo += sm.lo + v.lo;
}


// Barycentric-support rows of G needed by local row a: g0 = G[ka0][:],
// g1 = G[ka1][:] (zero for a single-vertex support).
template <typename GT>
struct GRows {
    GT g0[4], g1[4];
};

// 16-byte vector loads of one G row (4 entries).
__device__ __forceinline__ void load_g4(const double *__restrict__ G, double out[4]) {
    const double2 x = __ldg(reinterpret_cast<const double2 *>(G));
    const double2 y = __ldg(reinterpret_cast<const double2 *>(G) + 1);
    out[0] = x.x; out[1] = x.y; out[2] = y.x; out[3] = y.y;
}
__device__ __forceinline__ void load_g4(const df64 *__restrict__ G, df64 out[4]) {
    const float4 x = __ldg(reinterpret_cast<const float4 *>(G));
    const float4 y = __ldg(reinterpret_cast<const float4 *>(G) + 1);
    out[0] = df64{x.x, x.y}; out[1] = df64{x.z, x.w}; out[2] = df64{y.x, y.y}; out[3] = df64{y.z, y.w};
}

template <int N, typename GT>
__device__ __forceinline__ void load_grows(const GT *__restrict__ Gbase, int4 rc, GRows<GT> &gr) {
    const int32_t e = rc.x / N;
    const int a = rc.x - e * N;
    const int ka0 = sup_lo(a), ka1 = sup_hi(a);
    const GT *G = Gbase + (int64_t)e * 16;
    load_g4(G + ka0 * 4, gr.g0);
    if (ka1 != ka0) {
        load_g4(G + ka1 * 4, gr.g1);
    } else {
#pragma unroll
        for (int l = 0; l < 4; ++l) gr.g1[l] = GT{};
    }
}

// Adds row a of K_e (incidence record rc, G rows gr) into the accumulators.
// The N entries are computed first, then the N accumulators (distinct slots:
// an element's columns are distinct) are loaded together, updated and stored,
// so the shared-memory round trips overlap instead of forming a chain.
template <int N, int MODE, typename GT>
__device__ __forceinline__ void add_row(int4 rc, const GRows<GT> &gr, const double *__restrict__ Td,
                                        const df64 *__restrict__ Tf, double *accd, df64 *accf, int base) {
    const int32_t e = rc.x / N;
    const int a = rc.x - e * N;
    const bool edge_a = sup_hi(a) != sup_lo(a);
    const unsigned ow[3] = {(unsigned)rc.y, (unsigned)rc.z, (unsigned)rc.w};
    int off[N];
#pragma unroll
    for (int bb = 0; bb < N; ++bb) off[bb] = base + (int)((ow[bb >> 2] >> (8 * (bb & 3))) & 0xffu);
    if constexpr (MODE == MODE_FP64) {
        double val[N];
#pragma unroll
        for (int bb = 0; bb < N; ++bb) {
            const int kb0 = sup_lo(bb), kb1 = sup_hi(bb);
            const bool edge_b = kb1 != kb0;
            const double *T = Td + (a * N + bb) * 4;
            double v = gr.g0[kb0] * T[0];
            if (edge_b) v += gr.g0[kb1] * T[1];
            if (edge_a) {
                v += gr.g1[kb0] * T[2];
                if (edge_b) v += gr.g1[kb1] * T[3];
            }
            val[bb] = v;
        }
        double acc[N];
#pragma unroll
        for (int bb = 0; bb < N; ++bb) acc[bb] = accd[off[bb]];
#pragma unroll
        for (int bb = 0; bb < N; ++bb) accd[off[bb]] = acc[bb] + val[bb];
    } else {
        df64 val[N];
#pragma unroll
        for (int bb = 0; bb < N; ++bb) {
            const int kb0 = sup_lo(bb), kb1 = sup_hi(bb);
            const bool edge_b = kb1 != kb0;
            const df64 *T = Tf + (a * N + bb) * 4;
            const df64 xs[4] = {gr.g0[kb0], gr.g0[kb1], gr.g1[kb0], gr.g1[kb1]};
            float S = 0.f, L = 0.f;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if ((q & 1) && !edge_b) continue;
                if (q >= 2 && !edge_a) continue;
                const df64 x = xs[q], y = T[q];
                const float ph = x.hi * y.hi;
                float err = fmaf(x.hi, y.hi, -ph);
                err = fmaf(x.hi, y.lo, err);
                err = fmaf(x.lo, y.hi, err);
                if constexpr (MODE == MODE_DF64) {
                    const df64 ts = two_sum(S, ph);
                    S = ts.hi;
                    L += ts.lo + err;
                } else {
                    S += ph;  // FP32 accumulation of the split products
                    L += err;
                }
            }
            val[bb] = df64{S, L};
        }
        df64 acc[N];
#pragma unroll
        for (int bb = 0; bb < N; ++bb) acc[bb] = accf[off[bb]];
#pragma unroll
        for (int bb = 0; bb < N; ++bb) {
            df_acc(acc[bb], val[bb]);
            accf[off[bb]] = acc[bb];
        }
    }
}

// ---------------------------------------------------------------- exact rule
// For a quadrature rule that integrates quadratics exactly, 30 T^{kl}_ab of
// P2 is an integer in {-1, 3, 4, 8}: with the reference tetrahedron integrals
// int l_x l_y = (1 + d_xy) / 120, int l_x = 1/24, int 1 = 1/6, the supports
// and coefficients above give
//   vertex-vertex   (4 l_a - 1)(4 l_b - 1):  4 (1 + d_ab) - 5
//   vertex-edge     (4 l_a - 1) 4 l_y:       4 (1 + d_ay) - 5
//   edge-edge       4 l_x 4 l_y:             4 (1 + d_xy)
// where x / y is the barycentric factor multiplying the support vertex.
// The host checks the caller's rule against this table; the element pass
// then stores G / 30 and the row pass multiplies by these compile-time
// integers (exact double-float scalings).
__host__ __device__ constexpr int factor_of(int a, int slot) {
    // barycentric index whose (4 lambda) multiplies support slot `slot` of
    // edge function a (slot 0 -> 4 lambda_j on vertex i, slot 1 -> 4 lambda_i on j)
    return slot == 0 ? sup_hi(a) : sup_lo(a);
}
__host__ __device__ constexpr int t30(int a, int b, int sa, int sb) {
    const bool ea = a >= 4, eb = b >= 4;
    if (!ea && !eb) return 4 * (1 + (a == b)) - 5;
    if (!ea && eb) return 4 * (1 + (a == factor_of(b, sb))) - 5;
    if (ea && !eb) return 4 * (1 + (b == factor_of(a, sa))) - 5;
    return 4 * (1 + (factor_of(a, sa) == factor_of(b, sb)));
}

// t * x for a small integer t, as an unnormalised double-float.
template <int TV>
__device__ __forceinline__ df64 df_mul_int(df64 x) {
    if constexpr (TV == 1) return x;
    else if constexpr (TV == -1) return df64{-x.hi, -x.lo};
    else if constexpr (TV == 4 || TV == 8 || TV == -4 || TV == -8) return df64{x.hi * (float)TV, x.lo * (float)TV};
    else {
        const float ph = x.hi * (float)TV;
        const float err = fmaf(x.hi, (float)TV, -ph);
        return df64{ph, fmaf(x.lo, (float)TV, err)};
    }
}

template <int MODE>
__device__ __forceinline__ void sum_term(float &S, float &L, df64 t) {
    if constexpr (MODE == MODE_DF64) {
        const df64 ts = two_sum(S, t.hi);
        S = ts.hi;
        L += ts.lo + t.lo;
    } else {
        S += t.hi;
        L += t.lo;
    }
}

template <int A, int MODE>
__device__ __forceinline__ void add_row_exact(const GRows<df64> &gr, df64 *accf, const int off[10]) {
    constexpr int ka0 = sup_lo(A), ka1 = sup_hi(A);
    constexpr bool edge_a = ka1 != ka0;
    df64 val[10];
#pragma unroll
    for (int bb = 0; bb < 10; ++bb) {
        const int kb0 = sup_lo(bb), kb1 = sup_hi(bb);
        const bool edge_b = kb1 != kb0;
        float S = 0.f, L = 0.f;
        // slot pairs (sa, sb); the integer factors fold to immediates
        switch (bb) {
#define SKG_T(BB)                                                                                   \
    case BB: {                                                                                      \
        constexpr int kb0c = sup_lo(BB), kb1c = sup_hi(BB);                                         \
        sum_term<MODE>(S, L, df_mul_int<t30(A, BB, 0, 0)>(gr.g0[kb0c]));                            \
        if constexpr (kb1c != kb0c) sum_term<MODE>(S, L, df_mul_int<t30(A, BB, 0, 1)>(gr.g0[kb1c])); \
        if constexpr (edge_a) {                                                                     \
            sum_term<MODE>(S, L, df_mul_int<t30(A, BB, 1, 0)>(gr.g1[kb0c]));                        \
            if constexpr (kb1c != kb0c) sum_term<MODE>(S, L, df_mul_int<t30(A, BB, 1, 1)>(gr.g1[kb1c])); \
        }                                                                                           \
    } break;
            SKG_T(0) SKG_T(1) SKG_T(2) SKG_T(3) SKG_T(4) SKG_T(5) SKG_T(6) SKG_T(7) SKG_T(8) SKG_T(9)
#undef SKG_T
        }
        (void)kb0; (void)kb1; (void)edge_b;
        val[bb] = df64{S, L};
    }
    df64 acc[10];
#pragma unroll
    for (int bb = 0; bb < 10; ++bb) acc[bb] = accf[off[bb]];
#pragma unroll
    for (int bb = 0; bb < 10; ++bb) {
        df_acc(acc[bb], val[bb]);
        accf[off[bb]] = acc[bb];
    }
}

// P2 rows with the exact-rule table: dispatch on the local row index so all
// T factors are compile-time constants.
template <int MODE>
__device__ __forceinline__ void add_row_p2_exact(int4 rc, const GRows<df64> &gr, df64 *accf, int base) {
    const int32_t e = rc.x / 10;
    const int a = rc.x - e * 10;
    const unsigned ow[3] = {(unsigned)rc.y, (unsigned)rc.z, (unsigned)rc.w};
    int off[10];
#pragma unroll
    for (int bb = 0; bb < 10; ++bb) off[bb] = base + (int)((ow[bb >> 2] >> (8 * (bb & 3))) & 0xffu);
    switch (a) {
        case 0: add_row_exact<0, MODE>(gr, accf, off); break;
        case 1: add_row_exact<1, MODE>(gr, accf, off); break;
        case 2: add_row_exact<2, MODE>(gr, accf, off); break;
        case 3: add_row_exact<3, MODE>(gr, accf, off); break;
        case 4: add_row_exact<4, MODE>(gr, accf, off); break;
        case 5: add_row_exact<5, MODE>(gr, accf, off); break;
        case 6: add_row_exact<6, MODE>(gr, accf, off); break;
        case 7: add_row_exact<7, MODE>(gr, accf, off); break;
        case 8: add_row_exact<8, MODE>(gr, accf, off); break;
        default: add_row_exact<9, MODE>(gr, accf, off); break;
    }
}

// Row pass, P threads per CSR row (P = 1 for short rows, 2 for long rows).
// Each warp owns one row group (<= 32 / P consecutive rows whose slots, times
// P accumulator copies, fit SLOTS in shared memory).  Thread part p of row r
// walks the row's incidence records p, p + P, p + 2P, ... (ascending element
// order), evaluates row a of K_e on the fly and adds it into accumulator copy
// p; the next record and its G rows are loaded one step ahead.  The warp
// then sums the copies in copy order and writes the group's contiguous slot
// range with coalesced stores.  Each (copy, slot) is updated by one thread in
// a fixed order: bitwise reproducible, no atomics, no block-wide barrier
// after the table load.
template <int N, int MODE, int SLOTS, int P, bool EXACT>
__global__ void __launch_bounds__(kRowWarps * 32) k_rows_group(
    int n_groups, const int2 *__restrict__ groups, const int32_t *__restrict__ indptr,
    const int32_t *__restrict__ inc_ptr, const int4 *__restrict__ rec, const void *__restrict__ Gv,
    const double *__restrict__ Tg, const int *__restrict__ s_ptr, double *__restrict__ values) {
    using GT = typename std::conditional<MODE == MODE_FP64, double, df64>::type;
    extern __shared__ __align__(16) unsigned char smem[];
    double *Td = reinterpret_cast<double *>(smem);
    df64 *Tf = reinterpret_cast<df64 *>(smem);
    unsigned char *warp_area = smem + N * N * 4 * 8;
    for (int i = threadIdx.x; i < N * N * 4; i += blockDim.x) {
        const double tv = Tg[i];
        if constexpr (MODE == MODE_FP64) {
            Td[i] = tv;
        } else {
            const float h = (float)tv;
            Tf[i] = df64{h, (float)(tv - (double)h)};
        }
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gi = blockIdx.x * kRowWarps + warp;
    if (gi >= n_groups) return;
    double *accd = reinterpret_cast<double *>(warp_area + (size_t)warp * SLOTS * 8);
    df64 *accf = reinterpret_cast<df64 *>(accd);
    const int2 grp = groups[gi];
    const int32_t s0 = indptr[grp.x];
    const int nslots = indptr[grp.y] - s0;
    for (int j = lane; j < P * nslots; j += 32) {
        if constexpr (MODE == MODE_FP64) accd[j] = 0.0;
        else accf[j] = df64{0.f, 0.f};
    }
    __syncwarp();
    const int ridx = lane / P, part = lane - (lane / P) * P;
    const int32_t r = grp.x + ridx;
    if (ridx < 32 / P && r < grp.y) {
        const int base = indptr[r] - s0 + part * nslots;
        const int32_t it1 = inc_ptr[r + 1];
        int32_t it = inc_ptr[r] + part;
        const GT *Gb = reinterpret_cast<const GT *>(Gv);
        if (it < it1) {
            int4 rc = rec[it];
            GRows<GT> cur;
            load_grows<N>(Gb, rc, cur);
            int4 rcn = it + P < it1 ? rec[it + P] : make_int4(0, 0, 0, 0);
            for (; it < it1; it += P) {
                const bool has_next = it + P < it1;
                GRows<GT> nxt;
                if (has_next) load_grows<N>(Gb, rcn, nxt);
                const int4 rcnn = it + 2 * P < it1 ? rec[it + 2 * P] : make_int4(0, 0, 0, 0);
                if constexpr (EXACT && N == 10 && MODE != MODE_FP64) add_row_p2_exact<MODE>(rc, cur, accf, base);
                else add_row<N, MODE>(rc, cur, Td, Tf, accd, accf, base);
                rc = rcn;
                rcn = rcnn;
                if (has_next) cur = nxt;
            }
        }
    }
    __syncwarp();
    if constexpr (MODE == MODE_FP64) {
        for (int j = lane; j < nslots; j += 32) {
            double v = accd[j];
#pragma unroll
            for (int c = 1; c < P; ++c) v += accd[c * nslots + j];
            values[s0 + j] = v;
        }
    } else {
        const int sc = *s_ptr;
        for (int j = lane; j < nslots; j += 32) {
            df64 v = fast_two_sum(accf[j].hi, accf[j].lo);
#pragma unroll
            for (int c = 1; c < P; ++c) v = df_add(v, fast_two_sum(accf[c * nslots + j].hi, accf[c * nslots + j].lo));
            values[s0 + j] = df_to_double(v, sc);
        }
    }
}

// ------------------------------------------- element matrices, double-float
// The double-float mode of P2 with an exact rule: the element pass evaluates
// K_ab = sum t30 G/30 (integer factors, double-float G) once per entry (upper
// triangle for a symmetric coefficient) and stores the 10 x 10 matrix as FP32
// (hi, lo) pairs; the row pass adds rows into double-float slots.

template <int I, int N, class F>
__device__ __forceinline__ void static_for(F &&f) {
    if constexpr (I < N) {
        f(std::integral_constant<int, I>{});
        static_for<I + 1, N>(f);
    }
}

template <int A, int BB, int MODE>
__device__ __forceinline__ df64 exact_entry(const df64 g[16]) {
    constexpr int ka0 = sup_lo(A), ka1 = sup_hi(A), kb0 = sup_lo(BB), kb1 = sup_hi(BB);
    float S = 0.f, L = 0.f;
    sum_term<MODE>(S, L, df_mul_int<t30(A, BB, 0, 0)>(g[ka0 * 4 + kb0]));
    if constexpr (kb1 != kb0) sum_term<MODE>(S, L, df_mul_int<t30(A, BB, 0, 1)>(g[ka0 * 4 + kb1]));
    if constexpr (ka1 != ka0) {
        sum_term<MODE>(S, L, df_mul_int<t30(A, BB, 1, 0)>(g[ka1 * 4 + kb0]));
        if constexpr (kb1 != kb0) sum_term<MODE>(S, L, df_mul_int<t30(A, BB, 1, 1)>(g[ka1 * 4 + kb1]));
    }
    return fast_two_sum(S, L);
}

// exact_entry for a symmetric G (the upper triangle, a <= b), with fewer
// terms where G's symmetry and zero row sums allow (as shared_entry does in
// FP64): an edge's diagonal entry as 8 (G_ii + G_jj + G_ij) (3 terms instead
// of 4), an entry of two edges sharing a vertex s as 8 G_na,nb - 4 G_s,n (na,
// nb their other ends, n the fourth vertex: 2 terms instead of 4).
template <int A, int BB, int MODE>
__device__ __forceinline__ df64 exact_entry_sym(const df64 g[16]) {
    if constexpr (A >= 4 && BB >= 4) {
        constexpr int i = sup_lo(A), j = sup_hi(A), lb = sup_lo(BB), hb = sup_hi(BB);
        if constexpr (A == BB) {
            float S = 0.f, L = 0.f;
            sum_term<MODE>(S, L, df_mul_int<8>(g[i * 4 + i]));
            sum_term<MODE>(S, L, df_mul_int<8>(g[j * 4 + j]));
            sum_term<MODE>(S, L, df_mul_int<8>(g[i * 4 + j]));
            return fast_two_sum(S, L);
        } else if constexpr (i == lb || i == hb || j == lb || j == hb) {
            constexpr int sv = (i == lb || i == hb) ? i : j;
            constexpr int na = sv == i ? j : i, nb = (lb == sv) ? hb : lb, n = 6 - sv - na - nb;
            float S = 0.f, L = 0.f;
            sum_term<MODE>(S, L, df_mul_int<8>(g[na * 4 + nb]));
            sum_term<MODE>(S, L, df_mul_int<-4>(g[sv * 4 + n]));
            return fast_two_sum(S, L);
        }
    }
    return exact_entry<A, BB, MODE>(g);
}

// FP64 entry K_ab = sum t30 G (G carrying the 1/30) with compile-time integer
// factors: -1 terms become additions, a vertex-edge entry one FMA.
template <int A, int BB>
__device__ __forceinline__ double exact_entry_fp64(const double g[16]) {
    constexpr int ka0 = sup_lo(A), ka1 = sup_hi(A), kb0 = sup_lo(BB), kb1 = sup_hi(BB);
    constexpr double t00 = t30(A, BB, 0, 0), t01 = t30(A, BB, 0, 1), t10 = t30(A, BB, 1, 0), t11 = t30(A, BB, 1, 1);
    double v = t00 * g[ka0 * 4 + kb0];
    if constexpr (kb1 != kb0) v += t01 * g[ka0 * 4 + kb1];
    if constexpr (ka1 != ka0) {
        v += t10 * g[ka1 * 4 + kb0];
        if constexpr (kb1 != kb0) v += t11 * g[ka1 * 4 + kb1];
    }
    return v;
}

// The 55 entries of a symmetric element matrix with fewer FP64 instructions
// than one exact_entry_fp64 per entry (about 55 against 112).  With S_v(b) =
// G_v,lo(b) + G_v,hi(b) (vertex v, edge b), the integer table gives
//   vertex a, vertex b:      3 G_aa (a = b), -G_ab
//   vertex a, edge b:        -S_a(b) (a not on b), 3 G_a,hi - G_a,lo (a = lo(b)), 3 G_a,lo - G_a,hi (a = hi(b))
//   edge a = (i, j), edge b: 4 (S_i(b) + S_j(b) + X), X = G_ii + G_jj (a = b; with G symmetric that is
//                            8 (G_ii + G_jj + G_ij), two additions), X = G_(other end of a),(other end of b)
//                            (one shared vertex s, other ends na, nb, fourth vertex n; with G's zero row
//                            sums that is 4 (2 G_na,nb - G_s,n), one addition), X = 0 (disjoint)
// (t30 = 4 (1 + d) - 5 on vertex functions, 4 (1 + d) on edge pairs), so only
// the 12 sums S_v(b) with v off edge b are formed.  The sign flips and the
// factors 2, 4 and 8 act on the bits (integer instructions): exact, provided
// every sum stays a normal number below the overflow threshold, which
// shared_entries_ok checks on G first.
__device__ __forceinline__ double neg_bits(double x) {
    return __hiloint2double(__double2hiint(x) ^ (int)0x80000000, __double2loint(x));
}
__device__ __forceinline__ double times4_bits(double x) {  // zero stays zero
    const int hi = __double2hiint(x);
    return __hiloint2double(hi + ((hi & 0x7ff00000) ? 0x00200000 : 0), __double2loint(x));
}
__device__ __forceinline__ double times2_bits(double x) {  // zero stays zero
    const int hi = __double2hiint(x);
    return __hiloint2double(hi + ((hi & 0x7ff00000) ? 0x00100000 : 0), __double2loint(x));
}
__device__ __forceinline__ double times8_bits(double x) {  // zero stays zero
    const int hi = __double2hiint(x);
    return __hiloint2double(hi + ((hi & 0x7ff00000) ? 0x00300000 : 0), __double2loint(x));
}

// Every nonzero G entry with a biased exponent in [64, 2032]: then any sum of
// up to six of them is zero or a normal number (a multiple of the smallest
// entry's unit in the last place, above 2^-1022) and four or eight times it
// is finite.
__device__ __forceinline__ bool shared_entries_ok(const double g[16]) {
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        const int hi = __double2hiint(g[k]), lo = __double2loint(g[k]);
        const int ex = (hi >> 20) & 0x7ff;
        ok = ok && (((hi & 0x7fffffff) | lo) == 0 || (ex >= 64 && ex <= 2032));
    }
    return ok;
}

template <int A, int BB>
__device__ __forceinline__ double shared_entry(const double g[16], const double S[4][6]) {
    if constexpr (A < 4 && BB < 4) {
        if constexpr (A == BB) return 3.0 * g[A * 4 + A];
        else return neg_bits(g[A * 4 + BB]);
    } else if constexpr (A < 4) {
        constexpr int lo = sup_lo(BB), hi = sup_hi(BB);
        if constexpr (A != lo && A != hi) return neg_bits(S[A][BB - 4]);
        else if constexpr (A == lo) return fma(3.0, g[A * 4 + hi], -g[A * 4 + lo]);
        else return fma(3.0, g[A * 4 + lo], -g[A * 4 + hi]);
    } else {
        constexpr int i = sup_lo(A), j = sup_hi(A), lb = sup_lo(BB), hb = sup_hi(BB);
        if constexpr (A == BB) {
            // 4 (S_i + S_j + g_ii + g_jj) over edge (i, j) = 8 (g_ii + g_jj + g_ij): g is symmetric here
            return times8_bits((g[i * 4 + i] + g[j * 4 + j]) + g[i * 4 + j]);
        }
        if constexpr (i == lb || i == hb || j == lb || j == hb) {
            // shared vertex sv, other ends na (of a) and nb (of b), fourth vertex n: with the zero row sum
            // G_sv,sv + G_sv,na + G_sv,nb + G_sv,n = 0 the entry is 4 (2 G_na,nb - G_sv,n)
            constexpr int sv = (i == lb || i == hb) ? i : j;
            constexpr int na = sv == i ? j : i, nb = (lb == sv) ? hb : lb, n = 6 - sv - na - nb;
            return times4_bits(times2_bits(g[na * 4 + nb]) - g[sv * 4 + n]);
        } else {
            return times4_bits(S[i][BB - 4] + S[j][BB - 4]);
        }
    }
}

__device__ __forceinline__ void shared_entries(const double g[16], double U[55]) {
    double S[4][6];  // S_v(b) for vertex v off edge b only (the others are not used)
    static_for<0, 24>([&](auto kk) {
        constexpr int k = decltype(kk)::value, v = k / 6, e = k % 6;
        if constexpr (v != sup_lo(4 + e) && v != sup_hi(4 + e))
            S[v][e] = g[v * 4 + sup_lo(4 + e)] + g[v * 4 + sup_hi(4 + e)];
    });
    static_for<0, 100>([&](auto kk) {
        constexpr int k = decltype(kk)::value, A = k / 10, BB = k % 10;
        if constexpr (A <= BB) U[tri10(A, BB)] = shared_entry<A, BB>(g, S);
    });
}

// k_elem_ke_fp64 for a rule exact on quadratics (the 4-point and the 11-point
// Keast rule): the entries from the integer table with compile-time factors
// (about 30 FP64 instructions per element fewer than the table read from
// shared memory); same staging and coalesced stores.
__global__ void __launch_bounds__(kKeBlock) k_elem_ke_fp64_exact(int64_t ne, int64_t e_begin, int64_t e_end,
                                                                 const double *__restrict__ p, int64_t npts,
                                                                 const int32_t *__restrict__ t, int coef_kind,
                                                                 const double *__restrict__ coef,
                                                                 double *__restrict__ Ke) {
    __shared__ double stage[kKeBlock * kKeChunk];
    const int64_t e0 = e_begin + (int64_t)blockIdx.x * kKeBlock;
    const int64_t e = e0 + threadIdx.x;
    double g[16];
    bool sym = true;
    if (e < e_end) {
        sym = elem_g_fp64(ne, p, npts, t, coef_kind, coef, e, g, 1.0 / 30.0);
    } else {
#pragma unroll
        for (int k = 0; k < 16; ++k) g[k] = 0.0;
    }
    double U[55];
    if (sym) {
        if (shared_entries_ok(g)) {
            shared_entries(g, U);
        } else {
            static_for<0, 100>([&](auto kk) {
                constexpr int k = decltype(kk)::value, A = k / 10, BB = k % 10;
                if constexpr (A <= BB) U[tri10(A, BB)] = exact_entry_fp64<A, BB>(g);
            });
        }
    }
    const int nvalid = (int)(e_end - e0 < kKeBlock ? e_end - e0 : kKeBlock);
    double *st = stage + threadIdx.x * kKeChunk;
    static_for<0, 100 / kKeChunk>([&](auto rr) {
        constexpr int r = decltype(rr)::value;
        if (sym) {
            static_for<0, kKeChunk>([&](auto qq) {
                constexpr int q = decltype(qq)::value, k = r * kKeChunk + q, A = k / 10, BB = k % 10;
                st[q] = U[A <= BB ? tri10(A, BB) : tri10(BB, A)];
            });
        } else {
            static_for<0, kKeChunk>([&](auto qq) {
                constexpr int q = decltype(qq)::value, k = r * kKeChunk + q, A = k / 10, BB = k % 10;
                st[q] = exact_entry_fp64<A, BB>(g);
            });
        }
        __syncthreads();
        // coalesced copy-out: element rows are 100 doubles apart
        for (int i = threadIdx.x; i < nvalid * kKeChunk; i += kKeBlock) {
            const int el = i / kKeChunk, q = i - el * kKeChunk;
            Ke[(e0 + el) * 100 + r * kKeChunk + q] = stage[el * kKeChunk + q];
        }
        __syncthreads();
    });
}

// Tile `tile` (kKeBlock elements) of k_elem_ke_df64; `stage` kKeBlock *
// kKeChunk pairs of shared memory.
template <int MODE>
__device__ __forceinline__ void elem_ke_df64_tile(int64_t tile, int64_t ne, const double *__restrict__ p,
                                                  int64_t npts, const int32_t *__restrict__ t, int coef_kind,
                                                  const double *__restrict__ coef, const int *__restrict__ s_ptr,
                                                  float2 *__restrict__ Ke, int *__restrict__ range_flag,
                                                  float2 *stage) {
    const int64_t e0 = tile * kKeBlock;
    const int64_t e = e0 + threadIdx.x;
    const bool valid = e < ne;
    df64 g[16];
    bool ok = true, sym = true;
    if (valid) {
        sym = elem_g_df64(ne, p, npts, t, coef_kind, coef, *s_ptr, true, e, g, ok);
        if (!ok) atomicExch(range_flag, 1);
    } else {
#pragma unroll
        for (int k = 0; k < 16; ++k) g[k] = df64{0.f, 0.f};
    }
    df64 U[55];
    if (sym) {  // the same entries as k_elem_ke_df64_packed gives a symmetric element
        static_for<0, 100>([&](auto kk) {
            constexpr int k = decltype(kk)::value, A = k / 10, BB = k % 10;
            if constexpr (A <= BB) U[tri10(A, BB)] = exact_entry_sym<A, BB, MODE>(g);
        });
    }
    const int nvalid = (int)(ne - e0 < kKeBlock ? ne - e0 : kKeBlock);
    float2 *st = stage + threadIdx.x * kKeChunk;
    static_for<0, 100 / kKeChunk>([&](auto rr) {
        constexpr int r = decltype(rr)::value;
        if (sym) {
            static_for<0, kKeChunk>([&](auto qq) {
                constexpr int q = decltype(qq)::value, k = r * kKeChunk + q, A = k / 10, BB = k % 10;
                const df64 v = U[A <= BB ? tri10(A, BB) : tri10(BB, A)];
                st[q] = make_float2(v.hi, v.lo);
            });
        } else {
            static_for<0, kKeChunk>([&](auto qq) {
                constexpr int q = decltype(qq)::value, k = r * kKeChunk + q;
                const df64 v = exact_entry<k / 10, k % 10, MODE>(g);
                st[q] = make_float2(v.hi, v.lo);
            });
        }
        __syncthreads();
        for (int i = threadIdx.x; i < nvalid * kKeChunk; i += kKeBlock) {
            const int el = i / kKeChunk, q = i - el * kKeChunk;
            Ke[(e0 + el) * 100 + r * kKeChunk + q] = stage[el * kKeChunk + q];
        }
        __syncthreads();
    });
}

// The blocks walk the tiles (grid-stride); with `only` non-NULL they
// assemble only the tiles with only[tile] set.
template <int MODE>
__global__ void __launch_bounds__(kKeBlock, 3) k_elem_ke_df64(int64_t ne, const double *__restrict__ p, int64_t npts,
                                                           const int32_t *__restrict__ t, int coef_kind,
                                                           const double *__restrict__ coef,
                                                           const int *__restrict__ s_ptr, float2 *__restrict__ Ke,
                                                           int *__restrict__ range_flag,
                                                           const uint8_t *__restrict__ only = nullptr) {
    __shared__ float2 stage[kKeBlock * kKeChunk];
    __shared__ uint8_t flag[kKeBlock];
    const int64_t n_tiles = (ne + kKeBlock - 1) / kKeBlock;
    if (!only) {
        for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x)
            elem_ke_df64_tile<MODE>(tile, ne, p, npts, t, coef_kind, coef, s_ptr, Ke, range_flag, stage);
        return;
    }
    // kKeBlock flags per round, read by the block at once
    for (int64_t base = (int64_t)blockIdx.x * kKeBlock; base < n_tiles; base += (int64_t)gridDim.x * kKeBlock) {
        flag[threadIdx.x] = base + threadIdx.x < n_tiles ? only[base + threadIdx.x] : 0;
        if (!__syncthreads_or(flag[threadIdx.x])) continue;
        for (int j = 0; j < kKeBlock; ++j)
            if (flag[j])
                elem_ke_df64_tile<MODE>(base + j, ne, p, npts, t, coef_kind, coef, s_ptr, Ke, range_flag, stage);
        __syncthreads();  // flags of the next round
    }
}

// Element matrices of SKG_SPLIT_FP32 (P2, exact rule): G in double-float, each
// entry's integer-factor terms summed in FP32 with split products
// (exact_entry<MODE_SPLIT>), the entry rounded to FP32.  Each entry goes to
// shared memory as it is computed (the packed upper triangle of a symmetric
// matrix, mirrored by the copy-out; every entry, in two rounds of five rows,
// when a tile holds a nonsymmetric coefficient), so no entry array is held
// in registers: enough warps to hide the coordinate and coefficient loads.
__global__ void __launch_bounds__(kKeBlock) k_elem_ke_split(int64_t ne, const double *__restrict__ p, int64_t npts,
                                                            const int32_t *__restrict__ t, int coef_kind,
                                                            const double *__restrict__ coef,
                                                            const int *__restrict__ s_ptr, float *__restrict__ Ke,
                                                            int *__restrict__ range_flag) {
    constexpr int kPacked = 55, kHalf = 51;  // odd strides: conflict-free per-thread stores
    __shared__ float stage[kKeBlock * kPacked];
    const int64_t e0 = (int64_t)blockIdx.x * kKeBlock;
    const int64_t e = e0 + threadIdx.x;
    df64 g[16];
    bool ok = true, sym = true;
    if (e < ne) {
        sym = elem_g_df64(ne, p, npts, t, coef_kind, coef, *s_ptr, true, e, g, ok);
        if (!ok) atomicExch(range_flag, 1);
    } else {
#pragma unroll
        for (int k = 0; k < 16; ++k) g[k] = df64{0.f, 0.f};
    }
    const int nvalid = (int)(ne - e0 < kKeBlock ? ne - e0 : kKeBlock);
    if (__syncthreads_and(sym)) {
        float *st = stage + threadIdx.x * kPacked;
        static_for<0, 100>([&](auto kk) {
            constexpr int k = decltype(kk)::value, A = k / 10, BB = k % 10;
            if constexpr (A <= BB) {
                const df64 v = exact_entry_sym<A, BB, MODE_SPLIT>(g);
                st[tri10(A, BB)] = v.hi + v.lo;
            }
        });
        __syncthreads();
        for (int i = threadIdx.x; i < nvalid * 100; i += kKeBlock) {
            const int el = i / 100, k = i - el * 100, a = k / 10, b = k - a * 10;
            Ke[(e0 + el) * 100 + k] = stage[el * kPacked + (a <= b ? tri10(a, b) : tri10(b, a))];
        }
    } else {
        float *st = stage + threadIdx.x * kHalf;
        static_for<0, 2>([&](auto rr) {
            constexpr int r = decltype(rr)::value;
            static_for<0, 50>([&](auto qq) {
                constexpr int q = decltype(qq)::value, k = r * 50 + q;
                const df64 v = exact_entry<k / 10, k % 10, MODE_SPLIT>(g);
                st[q] = v.hi + v.lo;
            });
            __syncthreads();
            for (int i = threadIdx.x; i < nvalid * 50; i += kKeBlock) {
                const int el = i / 50, q = i - el * 50;
                Ke[(e0 + el) * 100 + r * 50 + q] = stage[el * kHalf + q];
            }
            __syncthreads();
        });
    }
}

// SKG_FP64_EMULATED element matrices with a symmetric coefficient: each of
// the 55 distinct entries is stored to shared memory as it is computed
// (packed upper triangle, mirrored by the copy-out) instead of being held in
// registers until its row is staged as in k_elem_ke_df64: 64 registers
// against 168, so more warps per SM (0.53 -> 0.41 ms at 64^3).  A tile with a
// nonsymmetric coefficient is flagged in `redo` and left to k_elem_ke_df64.
template <typename T>
__device__ __forceinline__ void copy_packed(const T *stage, int nvalid, int64_t e0, T *__restrict__ Ke) {
    for (int i = threadIdx.x; i < nvalid * 100; i += kKeBlock) {
        const int el = i / 100, k = i - el * 100, a = k / 10, b = k - a * 10;
        Ke[(e0 + el) * 100 + k] = stage[el * 55 + (a <= b ? tri10(a, b) : tri10(b, a))];
    }
}

__global__ void __launch_bounds__(kKeBlock) k_elem_ke_df64_packed(int64_t ne, const double *__restrict__ p,
                                                                  int64_t npts, const int32_t *__restrict__ t,
                                                                  int coef_kind, const double *__restrict__ coef,
                                                                  const int *__restrict__ s_ptr,
                                                                  float2 *__restrict__ Ke,
                                                                  int *__restrict__ range_flag,
                                                                  uint8_t *__restrict__ redo) {
    extern __shared__ __align__(16) unsigned char smem[];
    float2 *stage = reinterpret_cast<float2 *>(smem);  // kKeBlock x 55
    const int64_t e0 = (int64_t)blockIdx.x * kKeBlock;
    const int64_t e = e0 + threadIdx.x;
    df64 g[16];
    bool ok = true, sym = true;
    if (e < ne) {
        sym = elem_g_df64(ne, p, npts, t, coef_kind, coef, *s_ptr, true, e, g, ok);
        if (!ok) atomicExch(range_flag, 1);
    } else {
#pragma unroll
        for (int k = 0; k < 16; ++k) g[k] = df64{0.f, 0.f};
    }
    if (!__syncthreads_and(sym)) {  // a nonsymmetric coefficient: k_elem_ke_df64 redoes this tile
        if (threadIdx.x == 0) redo[blockIdx.x] = 1;
        return;
    }
    float2 *st = stage + threadIdx.x * 55;
    static_for<0, 100>([&](auto kk) {
        constexpr int k = decltype(kk)::value, A = k / 10, BB = k % 10;
        if constexpr (A <= BB) {
            const df64 v = exact_entry_sym<A, BB, MODE_DF64>(g);
            st[tri10(A, BB)] = make_float2(v.hi, v.lo);
        }
    });
    __syncthreads();
    copy_packed(stage, (int)(ne - e0 < kKeBlock ? ne - e0 : kKeBlock), e0, Ke);
}

constexpr int kPackedSmem = kKeBlock * 55 * 8;  // 56,320 bytes


// Row pass over double-float element matrices: rows of 10 (hi, lo) pairs added
// into double-float slots, converted to FP64 at write-out.
template <int SLOTS, int P>
__global__ void __launch_bounds__(kRowWarps * 32) k_rows_ke_df(int n_groups, const int2 *__restrict__ groups,
                                                              const int32_t *__restrict__ indptr,
                                                              const int32_t *__restrict__ inc_ptr,
                                                              const int4 *__restrict__ rec,
                                                              const float2 *__restrict__ Ke,
                                                              const int *__restrict__ s_ptr,
                                                              double *__restrict__ values) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gi = blockIdx.x * kRowWarps + warp;
    if (gi >= n_groups) return;
    df64 *acc = reinterpret_cast<df64 *>(smem + (size_t)warp * SLOTS * 8);
    const int2 grp = groups[gi];
    const int32_t s0 = indptr[grp.x];
    const int nslots = indptr[grp.y] - s0;
    for (int j = lane; j < P * nslots; j += 32) acc[j] = df64{0.f, 0.f};
    __syncwarp();
    const int ridx = lane / P, part = lane - (lane / P) * P;
    const int32_t r = grp.x + ridx;
    if (ridx < 32 / P && r < grp.y) {
        const int base = indptr[r] - s0 + part * nslots;
        const int32_t it1 = inc_ptr[r + 1];
        int32_t it = inc_ptr[r] + part;
        if (it < it1) {
            // records two incidences ahead of the rows they address, rows one
            int4 rc = rec[it];
            int4 rcn = it + P < it1 ? rec[it + P] : make_int4(0, 0, 0, 0);
            float4 cur[5];
            {
                const float4 *src = reinterpret_cast<const float4 *>(Ke + (int64_t)rc.x * 10);
#pragma unroll
                for (int q = 0; q < 5; ++q) cur[q] = __ldg(src + q);
            }
            bool first = true;
            for (; it < it1; it += P) {
                const bool has_next = it + P < it1;
                float4 nxt[5];
                if (has_next) {
                    const float4 *src = reinterpret_cast<const float4 *>(Ke + (int64_t)rcn.x * 10);
#pragma unroll
                    for (int q = 0; q < 5; ++q) nxt[q] = __ldg(src + q);
                }
                const int4 rcnn = it + 2 * P < it1 ? rec[it + 2 * P] : make_int4(0, 0, 0, 0);
                const unsigned ow[3] = {(unsigned)rc.y, (unsigned)rc.z, (unsigned)rc.w};
                int off[10];
#pragma unroll
                for (int bb = 0; bb < 10; ++bb) off[bb] = base + (int)((ow[bb >> 2] >> (8 * (bb & 3))) & 0xffu);
                if (first) {  // the part's first incidence: its row initialises the slots
#pragma unroll
                    for (int q = 0; q < 5; ++q) {
                        acc[off[2 * q]] = df64{cur[q].x, cur[q].y};
                        acc[off[2 * q + 1]] = df64{cur[q].z, cur[q].w};
                    }
                    first = false;
                } else {
                    df64 a[10];
#pragma unroll
                    for (int bb = 0; bb < 10; ++bb) a[bb] = acc[off[bb]];
#pragma unroll
                    for (int q = 0; q < 5; ++q) {
                        df_acc(a[2 * q], df64{cur[q].x, cur[q].y});
                        df_acc(a[2 * q + 1], df64{cur[q].z, cur[q].w});
                    }
#pragma unroll
                    for (int bb = 0; bb < 10; ++bb) acc[off[bb]] = a[bb];
                }
                if (has_next) {
                    rc = rcn;
                    rcn = rcnn;
#pragma unroll
                    for (int q = 0; q < 5; ++q) cur[q] = nxt[q];
                }
            }
        }
    }
    __syncwarp();
    const int sc = *s_ptr;
    for (int j = lane; j < nslots; j += 32) {
        df64 v = fast_two_sum(acc[j].hi, acc[j].lo);
#pragma unroll
        for (int c = 1; c < P; ++c) v = df_add(v, fast_two_sum(acc[c * nslots + j].hi, acc[c * nslots + j].lo));
        values[s0 + j] = df_to_double(v, sc);
    }
}

template <int SLOTS, int P>
void launch_ke_df_class(int n_groups, const int2 *groups, const skg_pattern *pat, const float2 *Ke, const int *s_ptr,
                        double *values, cudaStream_t s) {
    if (n_groups == 0) return;
    const size_t smem = (size_t)kRowWarps * SLOTS * 8;
    if (smem > 48 * 1024)
        SKG_CUDA(cudaFuncSetAttribute(k_rows_ke_df<SLOTS, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const unsigned grid = (unsigned)((n_groups + kRowWarps - 1) / kRowWarps);
    k_rows_ke_df<SLOTS, P><<<grid, kRowWarps * 32, smem, s>>>(n_groups, groups, pat->indptr.get(), pat->inc_ptr.get(),
                                                              pat->rec.get(), Ke, s_ptr, values);
    SKG_LAUNCH_CHECK("rows_ke_df");
}

// Row pass over FP32 element matrices (SKG_SPLIT_FP32): rows of 10 floats
// added into double-float slots, converted to FP64 at write-out; otherwise as
// k_rows_ke_df (40-byte rows: half the element-matrix bytes).
template <int SLOTS, int P>
__global__ void __launch_bounds__(kRowWarps * 32) k_rows_ke_f32(int n_groups, const int2 *__restrict__ groups,
                                                               const int32_t *__restrict__ indptr,
                                                               const int32_t *__restrict__ inc_ptr,
                                                               const int4 *__restrict__ rec,
                                                               const float *__restrict__ Ke,
                                                               const int *__restrict__ s_ptr,
                                                               double *__restrict__ values) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gi = blockIdx.x * kRowWarps + warp;
    if (gi >= n_groups) return;
    df64 *acc = reinterpret_cast<df64 *>(smem + (size_t)warp * SLOTS * 8);
    const int2 grp = groups[gi];
    const int32_t s0 = indptr[grp.x];
    const int nslots = indptr[grp.y] - s0;
    for (int j = lane; j < P * nslots; j += 32) acc[j] = df64{0.f, 0.f};
    __syncwarp();
    const int ridx = lane / P, part = lane - (lane / P) * P;
    const int32_t r = grp.x + ridx;
    if (ridx < 32 / P && r < grp.y) {
        const int base = indptr[r] - s0 + part * nslots;
        const int32_t it1 = inc_ptr[r + 1];
        int32_t it = inc_ptr[r] + part;
        if (it < it1) {
            // records two incidences ahead of the rows they address, rows one
            int4 rc = rec[it];
            int4 rcn = it + P < it1 ? rec[it + P] : make_int4(0, 0, 0, 0);
            float2 cur[5];
            {
                const float2 *src = reinterpret_cast<const float2 *>(Ke + (int64_t)rc.x * 10);
#pragma unroll
                for (int q = 0; q < 5; ++q) cur[q] = __ldg(src + q);
            }
            bool first = true;
            for (; it < it1; it += P) {
                const bool has_next = it + P < it1;
                float2 nxt[5];
                if (has_next) {
                    const float2 *src = reinterpret_cast<const float2 *>(Ke + (int64_t)rcn.x * 10);
#pragma unroll
                    for (int q = 0; q < 5; ++q) nxt[q] = __ldg(src + q);
                }
                const int4 rcnn = it + 2 * P < it1 ? rec[it + 2 * P] : make_int4(0, 0, 0, 0);
                const unsigned ow[3] = {(unsigned)rc.y, (unsigned)rc.z, (unsigned)rc.w};
                int off[10];
#pragma unroll
                for (int bb = 0; bb < 10; ++bb) off[bb] = base + (int)((ow[bb >> 2] >> (8 * (bb & 3))) & 0xffu);
                if (first) {  // the part's first incidence: its row initialises the slots
#pragma unroll
                    for (int q = 0; q < 5; ++q) {
                        acc[off[2 * q]] = df64{cur[q].x, 0.f};
                        acc[off[2 * q + 1]] = df64{cur[q].y, 0.f};
                    }
                    first = false;
                } else {
                    df64 a[10];
#pragma unroll
                    for (int bb = 0; bb < 10; ++bb) a[bb] = acc[off[bb]];
#pragma unroll
                    for (int q = 0; q < 5; ++q) {
                        df_acc(a[2 * q], df64{cur[q].x, 0.f});
                        df_acc(a[2 * q + 1], df64{cur[q].y, 0.f});
                    }
#pragma unroll
                    for (int bb = 0; bb < 10; ++bb) acc[off[bb]] = a[bb];
                }
                if (has_next) {
                    rc = rcn;
                    rcn = rcnn;
#pragma unroll
                    for (int q = 0; q < 5; ++q) cur[q] = nxt[q];
                }
            }
        }
    }
    __syncwarp();
    const int sc = *s_ptr;
    for (int j = lane; j < nslots; j += 32) {
        df64 v = fast_two_sum(acc[j].hi, acc[j].lo);
#pragma unroll
        for (int c = 1; c < P; ++c) v = df_add(v, fast_two_sum(acc[c * nslots + j].hi, acc[c * nslots + j].lo));
        values[s0 + j] = df_to_double(v, sc);
    }
}

template <int SLOTS, int P>
void launch_ke_f32_class(int n_groups, const int2 *groups, const skg_pattern *pat, const float *Ke, const int *s_ptr,
                         double *values, cudaStream_t s) {
    if (n_groups == 0) return;
    const size_t smem = (size_t)kRowWarps * SLOTS * 8;
    if (smem > 48 * 1024)
        SKG_CUDA(cudaFuncSetAttribute(k_rows_ke_f32<SLOTS, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const unsigned grid = (unsigned)((n_groups + kRowWarps - 1) / kRowWarps);
    k_rows_ke_f32<SLOTS, P><<<grid, kRowWarps * 32, smem, s>>>(n_groups, groups, pat->indptr.get(), pat->inc_ptr.get(),
                                                               pat->rec.get(), Ke, s_ptr, values);
    SKG_LAUNCH_CHECK("rows_ke_f32");
}

// Fallback row pass (patterns without row blocks): thread per row, global
// accumulation, FP64.
template <int N>
__global__ void k_rows_global(int64_t n_rows, const int32_t *__restrict__ indptr, const int32_t *__restrict__ indices,
                              const int32_t *__restrict__ inc_ptr, const int32_t *__restrict__ inc,
                              const int32_t *__restrict__ dofs, const double *__restrict__ G,
                              const double *__restrict__ Tg, Support sp, double *__restrict__ values) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rows) return;
    const int32_t rb = indptr[r], rn = indptr[r + 1] - rb;
    for (int k = 0; k < rn; ++k) values[rb + k] = 0.;
    const int32_t *cols = indices + rb;
    for (int32_t it = inc_ptr[r]; it < inc_ptr[r + 1]; ++it) {
        const int32_t item = inc[it];
        const int64_t e = item / N;
        const int a = item - (int)(e * N);
        const double *g = G + e * 16;
        const int ka0 = sp.sup[a][0], ka1 = sp.sup[a][1];
        for (int bb = 0; bb < N; ++bb) {
            const int kb0 = sp.sup[bb][0], kb1 = sp.sup[bb][1];
            const double *T = Tg + (a * N + bb) * 4;
            double val = g[ka0 * 4 + kb0] * T[0];
            if (kb1 != kb0) val += g[ka0 * 4 + kb1] * T[1];
            if (ka1 != ka0) {
                val += g[ka1 * 4 + kb0] * T[2];
                if (kb1 != kb0) val += g[ka1 * 4 + kb1] * T[3];
            }
            const int32_t col = dofs[e * N + bb];
            const int pos = lower_bound_i32(cols, rn, col);
            if (pos < rn && cols[pos] == col) values[rb + pos] += val;
        }
    }
}

// Host: T^{kl}_{ab} from the quadrature rule, compacted to the supports.
void affine_table(int nodes, int nq, const double *X, const double *W, std::vector<double> &T, Support &sp) {
    static const int edges[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
    for (int a = 0; a < 10; ++a) sp.sup[a][0] = sp.sup[a][1] = 0;
    for (int a = 0; a < nodes; ++a) {
        if (a < 4) { sp.sup[a][0] = a; sp.sup[a][1] = a; }
        else { sp.sup[a][0] = edges[a - 4][0]; sp.sup[a][1] = edges[a - 4][1]; }
    }
    auto coeff = [&](int a, int slot, int q) -> double {
        const double x = X[q], y = X[nq + q], z = X[2 * nq + q];
        const double lam[4] = {1.0 - x - y - z, x, y, z};
        if (nodes == 4) return slot == 0 ? 1.0 : 0.0;
        if (a < 4) return slot == 0 ? 4.0 * lam[a] - 1.0 : 0.0;
        const int i = edges[a - 4][0], j = edges[a - 4][1];
        return slot == 0 ? 4.0 * lam[j] : 4.0 * lam[i];
    };
    T.assign((size_t)nodes * nodes * 4, 0.0);
    for (int a = 0; a < nodes; ++a)
        for (int b = 0; b < nodes; ++b)
            for (int u = 0; u < 2; ++u)
                for (int v = 0; v < 2; ++v) {
                    if (u == 1 && sp.sup[a][1] == sp.sup[a][0]) continue;
                    if (v == 1 && sp.sup[b][1] == sp.sup[b][0]) continue;
                    double acc = 0.0;
                    for (int q = 0; q < nq; ++q) acc += W[q] * coeff(a, u, q) * coeff(b, v, q);
                    T[((size_t)(a * nodes + b)) * 4 + u * 2 + v] = acc;
                }
}

template <int N, int MODE, int SLOTS, int P, bool EXACT>
void launch_group_class(int n_groups, const int2 *groups, const skg_pattern *pat, const void *G, const double *Tg,
                        const int *s_ptr, double *values, cudaStream_t s) {
    if (n_groups == 0) return;
    const size_t smem = (size_t)N * N * 4 * 8 + (size_t)kRowWarps * SLOTS * 8;
    if (smem > 48 * 1024)
        SKG_CUDA(cudaFuncSetAttribute(k_rows_group<N, MODE, SLOTS, P, EXACT>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const unsigned grid = (unsigned)((n_groups + kRowWarps - 1) / kRowWarps);
    k_rows_group<N, MODE, SLOTS, P, EXACT><<<grid, kRowWarps * 32, smem, s>>>(n_groups, groups, pat->indptr.get(),
                                                                      pat->inc_ptr.get(), pat->rec.get(), G, Tg, s_ptr,
                                                                      values);
    SKG_LAUNCH_CHECK("rows_group");
}

template <int N, int MODE, bool EXACT = false>
void launch_rows_groups(const skg_pattern *pat, const void *G, const double *Tg, const int *s_ptr, double *values,
                        cudaStream_t s, const GroupSet &gs) {
    launch_group_class<N, MODE, kGroupSlotsSmall, 1, EXACT>(gs.n_small, gs.small, pat, G, Tg, s_ptr, values, s);
    launch_group_class<N, MODE, kGroupSlotsLarge, 2, EXACT>(gs.n_large, gs.large, pat, G, Tg, s_ptr, values, s);
}

template <int N, int MODE, bool EXACT = false>
void launch_rows_groups(const skg_pattern *pat, const void *G, const double *Tg, const int *s_ptr, double *values,
                        cudaStream_t s) {
    launch_rows_groups<N, MODE, EXACT>(pat, G, Tg, s_ptr, values, s, all_groups(pat));
}

// True when the caller's rule reproduces the exact P2 table (30 T integer).
bool p2_rule_is_exact(const std::vector<double> &T) {
    for (int a = 0; a < 10; ++a)
        for (int b = 0; b < 10; ++b)
            for (int sa = 0; sa < 2; ++sa)
                for (int sb = 0; sb < 2; ++sb) {
                    const bool used = (sa == 0 || sup_hi(a) != sup_lo(a)) && (sb == 0 || sup_hi(b) != sup_lo(b));
                    const double want = used ? t30(a, b, sa, sb) / 30.0 : 0.0;
                    if (std::fabs(T[(a * 10 + b) * 4 + sa * 2 + sb] - want) > 1e-13) return false;
                }
    return true;
}

}  // namespace

void launch_scale_exponent(const double *d_p, int64_t n, int *d_s, cudaStream_t stream) {
    k_scale<<<2 * kSmCount, 256, 0, stream>>>(d_p, n, d_s);
    SKG_LAUNCH_CHECK("scale");
}

// Shared by the C ABI entry points below.
// h_values (optional, page-locked host): the values also go there, copied in
// row chunks overlapping the row pass (run_row_pass).
void affine_assemble(const skg_pattern *pat, const double *d_p, int64_t npts, const int32_t *d_t, int32_t nodes,
                     int64_t ne, int32_t nq, const double *h_X, const double *h_W, int32_t coef_kind,
                     const double *d_coef, int32_t precision, double *d_values, cudaStream_t s, cudaEvent_t *ev,
                     double *h_values) {
    require(pat != nullptr, "pattern is NULL");
    require(nodes == 4 || nodes == 10, "affine assembly supports P1 (4) and P2 (10) tetrahedra");
    require(ne == pat->n_elements && pat->row_local == nodes && pat->col_local == nodes,
            "mesh does not match the pattern");
    require(coef_kind == 0 || ((coef_kind == 1 || coef_kind == 2) && (d_coef || ne == 0)), "invalid coefficient kind");
    require(precision == SKG_FP64 || precision == SKG_SPLIT_FP32 || precision == SKG_FP64_EMULATED,
            "invalid precision");
    require(nq > 0 && h_X && h_W, "quadrature rule is empty");
    require(ne == 0 || (d_p && d_t), "mesh arrays are NULL");
    std::vector<double> T;
    Support sp{};
    affine_table(nodes, nq, h_X, h_W, T, sp);
    const double *Tg = device_table(T.data(), T.size(), s);
    DevBuf<double> G((size_t)ne * 16, s);  // 16 doubles or 16 df64 pairs per element
    const bool blocked = pat->max_row_len > 0;
    const bool exact = nodes == 10 && blocked && precision != SKG_FP64 && p2_rule_is_exact(T);
    int mode = precision == SKG_FP64 ? MODE_FP64 : precision == SKG_SPLIT_FP32 ? MODE_SPLIT : MODE_DF64;
    if (!blocked) mode = MODE_FP64;
    DevBuf<int> misc(2, s);  // [0] scale exponent, [1] range flag
    if (mode != MODE_FP64 && exact) {
        // P2, exact rule, FP32 pairs: element matrices (double-float entries
        // for SKG_FP64_EMULATED, FP32 entries summed in FP32 for
        // SKG_SPLIT_FP32), then the row sums in double-float slots
        const int init[2] = {INT_MIN, 0};
        SKG_CUDA(cudaMemcpyAsync(misc.get(), init, sizeof(init), cudaMemcpyHostToDevice, s));
        k_scale<<<2 * kSmCount, 256, 0, s>>>(d_p, 3 * npts, misc.get());
        SKG_LAUNCH_CHECK("scale");
        DevBuf<float2> Kf(mode == MODE_DF64 ? (size_t)ne * 100 : 0, s);
        DevBuf<float> Kh(mode == MODE_SPLIT ? (size_t)ne * 100 : 0, s);
        DevBuf<uint8_t> redo(mode == MODE_DF64 ? (size_t)grid_for(ne, kKeBlock) : 0, s);  // tiles left to k_elem_ke_df64
        if (ev) SKG_CUDA(cudaEventRecord(ev[0], s));
        if (ne) {
            if (mode == MODE_DF64) {
                const unsigned tiles = grid_for(ne, kKeBlock);
                SKG_CUDA(cudaMemsetAsync(redo.get(), 0, tiles, s));
                SKG_CUDA(cudaFuncSetAttribute(k_elem_ke_df64_packed, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              kPackedSmem));
                k_elem_ke_df64_packed<<<tiles, kKeBlock, kPackedSmem, s>>>(
                    ne, d_p, npts, d_t, coef_kind, d_coef, misc.get(), Kf.get(), misc.get() + 1, redo.get());
                SKG_LAUNCH_CHECK("elem_ke_df64_packed");
                k_elem_ke_df64<MODE_DF64><<<std::min<unsigned>((tiles + kKeBlock - 1) / kKeBlock, 2 * kSmCount),
                                            kKeBlock, 0, s>>>(
                    ne, d_p, npts, d_t, coef_kind, d_coef, misc.get(), Kf.get(), misc.get() + 1, redo.get());
            }
            else
                k_elem_ke_split<<<grid_for(ne, kKeBlock), kKeBlock, 0, s>>>(ne, d_p, npts, d_t, coef_kind, d_coef,
                                                                             misc.get(), Kh.get(), misc.get() + 1);
            SKG_LAUNCH_CHECK("elem_ke_df64");
        }
        int h_misc[2];
        SKG_CUDA(cudaMemcpyAsync(h_misc, misc.get(), sizeof(h_misc), cudaMemcpyDeviceToHost, s));
        SKG_CUDA(cudaStreamSynchronize(s));
        if (h_misc[1] == 0 && h_misc[0] != INT_MIN) {
            if (ev) SKG_CUDA(cudaEventRecord(ev[1], s));
            run_row_pass(pat, d_values, h_values, s, [&](const GroupSet &gs, cudaStream_t st) {
                if (mode == MODE_DF64) {
                    launch_ke_df_class<kGroupSlotsSmall, 1>(gs.n_small, gs.small, pat, Kf.get(), misc.get(), d_values,
                                                            st);
                    launch_ke_df_class<kGroupSlotsLarge, 2>(gs.n_large, gs.large, pat, Kf.get(), misc.get(), d_values,
                                                            st);
                } else {
                    launch_ke_f32_class<kGroupSlotsSmall, 1>(gs.n_small, gs.small, pat, Kh.get(), misc.get(),
                                                             d_values, st);
                    launch_ke_f32_class<kGroupSlotsLarge, 2>(gs.n_large, gs.large, pat, Kh.get(), misc.get(),
                                                             d_values, st);
                }
            });
            if (ev) SKG_CUDA(cudaEventRecord(ev[2], s));
            return;
        }
        mode = MODE_FP64;  // out of FP32 range: FP64 instead
    }
    if (mode != MODE_FP64) {
        const int init[2] = {INT_MIN, 0};
        SKG_CUDA(cudaMemcpyAsync(misc.get(), init, sizeof(init), cudaMemcpyHostToDevice, s));
        k_scale<<<2 * kSmCount, 256, 0, s>>>(d_p, 3 * npts, misc.get());
        SKG_LAUNCH_CHECK("scale");
        if (ev) SKG_CUDA(cudaEventRecord(ev[0], s));
        if (ne) {
            k_elem_df64<<<grid_for(ne, kElemBlock), kElemBlock, 0, s>>>(ne, d_p, npts, d_t, coef_kind, d_coef,
                                                                       misc.get(), reinterpret_cast<float4 *>(G.get()),
                                                                       misc.get() + 1, exact);
            SKG_LAUNCH_CHECK("elem_df64");
        }
        int h_misc[2];
        SKG_CUDA(cudaMemcpyAsync(h_misc, misc.get(), sizeof(h_misc), cudaMemcpyDeviceToHost, s));
        SKG_CUDA(cudaStreamSynchronize(s));
        if (h_misc[1] != 0 || h_misc[0] == INT_MIN) mode = MODE_FP64;  // out of FP32 range: FP64 instead
    }
    if (mode == MODE_FP64 && nodes == 10 && blocked) {
        // FP64 P2: element matrices, then row sums
        // (with a host output the two passes interleave, see run_passes)
        const bool exact_fp64 = p2_rule_is_exact(T);
        DevBuf<double> Ke((size_t)ne * 100, s);
        if (ev) SKG_CUDA(cudaEventRecord(ev[0], s));
        run_passes(
            pat, ne, d_values, h_values, s,
            [&](int64_t e0, int64_t e1) {
                if (exact_fp64)
                    k_elem_ke_fp64_exact<<<grid_for(e1 - e0, kKeBlock), kKeBlock, 0, s>>>(ne, e0, e1, d_p, npts, d_t,
                                                                                       coef_kind, d_coef, Ke.get());
                else
                    k_elem_ke_fp64<<<grid_for(e1 - e0, kKeBlock), kKeBlock, 0, s>>>(ne, e0, e1, d_p, npts, d_t,
                                                                                 coef_kind, d_coef, Tg, Ke.get());
                SKG_LAUNCH_CHECK("elem_ke_fp64");
                if (ev) SKG_CUDA(cudaEventRecord(ev[1], s));
            },
            [&](const GroupSet &gs, cudaStream_t st) { add_element_rows<10>(pat, Ke.get(), d_values, st, gs); });
        if (ev) SKG_CUDA(cudaEventRecord(ev[2], s));
        return;
    }
    if (mode == MODE_FP64) {
        if (ev) SKG_CUDA(cudaEventRecord(ev[0], s));
        if (ne) {
            k_elem_fp64<<<grid_for(ne, kElemBlock), kElemBlock, 0, s>>>(ne, d_p, npts, d_t, coef_kind, d_coef,
                                                                       reinterpret_cast<float4 *>(G.get()));
            SKG_LAUNCH_CHECK("elem_fp64");
        }
    }
    if (ev) SKG_CUDA(cudaEventRecord(ev[1], s));
    if (!blocked) {
        const unsigned grid = grid_for(pat->n_rows, 128);
        if (nodes == 4)
            k_rows_global<4><<<grid, 128, 0, s>>>(pat->n_rows, pat->indptr.get(), pat->indices.get(),
                                                  pat->inc_ptr.get(), pat->inc.get(), pat->col_dofs.get(), G.get(),
                                                  Tg, sp, d_values);
        else
            k_rows_global<10><<<grid, 128, 0, s>>>(pat->n_rows, pat->indptr.get(), pat->indices.get(),
                                                   pat->inc_ptr.get(), pat->inc.get(), pat->col_dofs.get(), G.get(),
                                                   Tg, sp, d_values);
        SKG_LAUNCH_CHECK("rows_global");
        if (h_values && pat->nnz)
            SKG_CUDA(cudaMemcpyAsync(h_values, d_values, (size_t)pat->nnz * sizeof(double), cudaMemcpyDeviceToHost, s));
    } else {
        const int *sp_ptr = misc.get();
        run_row_pass(pat, d_values, h_values, s, [&](const GroupSet &gs, cudaStream_t st) {
#define SKG_ROWS(NN, MM) launch_rows_groups<NN, MM>(pat, G.get(), Tg, sp_ptr, d_values, st, gs)
            if (nodes == 4) {
                if (mode == MODE_FP64) SKG_ROWS(4, MODE_FP64);
                else if (mode == MODE_SPLIT) SKG_ROWS(4, MODE_SPLIT);
                else SKG_ROWS(4, MODE_DF64);
            } else {
                if (mode == MODE_FP64) SKG_ROWS(10, MODE_FP64);
                else if (mode == MODE_SPLIT) {
                    if (exact) launch_rows_groups<10, MODE_SPLIT, true>(pat, G.get(), Tg, sp_ptr, d_values, st, gs);
                    else SKG_ROWS(10, MODE_SPLIT);
                } else {
                    SKG_ROWS(10, MODE_DF64);
                }
            }
        });
#undef SKG_ROWS
    }
    if (ev) SKG_CUDA(cudaEventRecord(ev[2], s));
}

namespace {

// ------------------------------------------------ P1 forms, per-element coefficients
// Scalar or vector (CC components) P1 element matrices of the value, gradient,
// symmetric-gradient and divergence kinds of bilinear_form_assembler.cpp:79-105
// when every coefficient is constant on each element.  The barycentric
// gradients are constant on an affine tetrahedron, so the point sums collapse
// to the rule's weight sum sw = sum_q w_q and its mass table
// M_ab = sum_q w_q N_a(x_q) N_b(x_q):
//   K_(a,c),(b,d) = sw / |det J| [ s/2 (B_a,d B_b,c + d_cd B_a.B_b) + dv B_a,c B_b,d + d_cd g B_a.B_b ]
//                 + d_cd v |det J| M_ab
// with B the adjugate rows (det J times the barycentric gradients).  Every
// kind gives a symmetric matrix, so only the blocks b >= a are evaluated,
// each written with its transpose into the thread's element matrix in shared
// memory; the block then stores all matrices coalesced.  About 260 FP64
// instructions per vector element, a fifth of the tabulated path, and no
// per-point data is read.
struct P1FormsConst {
    double sw;
    double mass[16];
    double cst[4];  // value, gradient, symmetric gradient, divergence when the array is NULL
};

template <int CC, int BLK>
__global__ void __launch_bounds__(BLK) k_p1_forms_ke(int64_t ne, int64_t e_begin, int64_t e_end,
                                                     const double *__restrict__ p, int64_t npts,
                                                     const int32_t *__restrict__ t,
                                                     const double *__restrict__ cv, const double *__restrict__ cg,
                                                     const double *__restrict__ cs, const double *__restrict__ cd,
                                                     P1FormsConst fc, double *__restrict__ Ke) {
    constexpr int L = 4 * CC, LL = L * L, LP = LL + 1;
    extern __shared__ double stage[];  // BLK x LP
    const int64_t e0 = e_begin + (int64_t)blockIdx.x * BLK;
    const int64_t e = e0 + threadIdx.x;
    const int nvalid = (int)(e_end - e0 < BLK ? e_end - e0 : BLK);
    double *st = stage + threadIdx.x * LP;
    if (e < e_end) {
        int32_t v[4];
        const bool ok = load_vertices(t, ne, e, npts, v);
        double J[9];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const double x0 = p[i * npts + v[0]];
#pragma unroll
            for (int r = 0; r < 3; ++r) J[i * 3 + r] = p[i * npts + v[r + 1]] - x0;
        }
        double b[4][3];
        b[1][0] = J[4] * J[8] - J[5] * J[7];
        b[1][1] = J[2] * J[7] - J[1] * J[8];
        b[1][2] = J[1] * J[5] - J[2] * J[4];
        b[2][0] = J[5] * J[6] - J[3] * J[8];
        b[2][1] = J[0] * J[8] - J[2] * J[6];
        b[2][2] = J[2] * J[3] - J[0] * J[5];
        b[3][0] = J[3] * J[7] - J[4] * J[6];
        b[3][1] = J[1] * J[6] - J[0] * J[7];
        b[3][2] = J[0] * J[4] - J[1] * J[3];
        const double ad = fabs(J[0] * b[1][0] + J[1] * b[2][0] + J[2] * b[3][0]);
#pragma unroll
        for (int i = 0; i < 3; ++i) b[0][i] = -(b[1][i] + b[2][i] + b[3][i]);
        const double inv = ok ? fc.sw / ad : __longlong_as_double(0x7ff8000000000000LL);
        const double vm = (cv ? cv[e] : fc.cst[0]) * ad;
        const double hs = 0.5 * (cs ? cs[e] : fc.cst[2]) * inv;
        const double dv = (cd ? cd[e] : fc.cst[3]) * inv;
        const double dg = (cg ? cg[e] : fc.cst[1]) * inv + hs;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            double sa[CC], da[CC], ta[CC];  // (s/2) B_a, dv B_a and their sum (entries c == d)
#pragma unroll
            for (int c = 0; c < CC; ++c) {
                sa[c] = hs * b[a][c];
                da[c] = dv * b[a][c];
                ta[c] = sa[c] + da[c];
            }
#pragma unroll
            for (int bb = a; bb < 4; ++bb) {
                const double gg = b[a][0] * b[bb][0] + b[a][1] * b[bb][1] + b[a][2] * b[bb][2];
                const double diag = dg * gg + vm * fc.mass[a * 4 + bb];
#pragma unroll
                for (int c = 0; c < CC; ++c)
#pragma unroll
                    for (int d = 0; d < CC; ++d) {
                        if (bb == a && d < c) continue;  // diagonal block: symmetric in (c, d)
                        const double val =
                            c == d ? diag + ta[c] * b[bb][c] : sa[d] * b[bb][c] + da[c] * b[bb][d];
                        st[(a * CC + c) * L + bb * CC + d] = val;
                        if (bb != a || c != d) st[(bb * CC + d) * L + a * CC + c] = val;
                    }
            }
        }
    }
    __syncthreads();
    for (int x = threadIdx.x; x < nvalid * LL; x += BLK) {
        const int el = x / LL, k = x - el * LL;
        Ke[(e0 + el) * (int64_t)LL + k] = stage[el * LP + k];
    }
}

template <int CC, int BLK>
void launch_p1_forms(int64_t ne, int64_t e0, int64_t e1, const double *d_p, int64_t npts, const int32_t *d_t,
                     const double *const coef[4], const P1FormsConst &fc, double *Ke, cudaStream_t s) {
    if (e1 <= e0) return;
    const int smem = BLK * (16 * CC * CC + 1) * 8;
    if (smem > 48 * 1024)
        SKG_CUDA(cudaFuncSetAttribute(k_p1_forms_ke<CC, BLK>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    k_p1_forms_ke<CC, BLK><<<grid_for(e1 - e0, BLK), BLK, smem, s>>>(ne, e0, e1, d_p, npts, d_t, coef[0], coef[1],
                                                                     coef[2], coef[3], fc, Ke);
    SKG_LAUNCH_CHECK("p1_forms_ke");
}

}  // namespace

void p1_forms_assemble(const skg_pattern *pat, const double *d_p, int64_t npts, const int32_t *d_t, int64_t ne,
                       int comp, int nq, const double *h_X, const double *h_W, const double *const coef[4],
                       const double cst[4], double *d_values, double *h_values, cudaStream_t s) {
    require(pat != nullptr, "pattern is NULL");
    require(comp == 1 || comp == 3, "P1 forms take 1 or 3 components");
    require(ne == pat->n_elements && pat->row_local == 4 * comp && pat->col_local == 4 * comp,
            "mesh does not match the pattern");
    require(nq > 0 && h_X && h_W, "quadrature rule is empty");
    require(ne == 0 || (d_p && d_t), "mesh arrays are NULL");
    require(pat->nnz == 0 || d_values, "output is NULL");
    require(pat->max_row_len > 0, "pattern has no row groups");
    P1FormsConst fc{};
    for (int q = 0; q < nq; ++q) {
        const double x = h_X[q], y = h_X[nq + q], z = h_X[2 * nq + q], w = h_W[q];
        const double N[4] = {1.0 - x - y - z, x, y, z};
        fc.sw += w;
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b) fc.mass[a * 4 + b] += w * N[a] * N[b];
    }
    for (int k = 0; k < 4; ++k) fc.cst[k] = coef[k] ? 0.0 : cst[k];
    if (ne == 0) {
        if (pat->nnz) SKG_CUDA(cudaMemsetAsync(d_values, 0, (size_t)pat->nnz * sizeof(double), s));
        if (h_values && pat->nnz)
            SKG_CUDA(cudaMemcpyAsync(h_values, d_values, (size_t)pat->nnz * sizeof(double), cudaMemcpyDeviceToHost, s));
        return;
    }
    const int L = 4 * comp;
    DevBuf<double> Ke((size_t)ne * L * L, s);
    run_passes(
        pat, ne, d_values, h_values, s,
        [&](int64_t e0, int64_t e1) {
            if (comp == 3) launch_p1_forms<3, 64>(ne, e0, e1, d_p, npts, d_t, coef, fc, Ke.get(), s);
            else launch_p1_forms<1, 128>(ne, e0, e1, d_p, npts, d_t, coef, fc, Ke.get(), s);
        },
        [&](const GroupSet &gs, cudaStream_t st) {
            if (comp == 3) add_element_rows<12>(pat, Ke.get(), d_values, st, gs);
            else add_element_rows<4>(pat, Ke.get(), d_values, st, gs);
        });
}

}  // namespace skg

using namespace skg;

extern "C" int skg_h1_assemble_affine(const skg_pattern *pat, const double *d_p, int64_t npts, const int32_t *d_t,
                                      int32_t nodes, int64_t ne, int32_t nq, const double *h_X, const double *h_W,
                                      int32_t coef_kind, const double *d_coef, int32_t precision, double *d_values,
                                      void *stream) {
    return guarded([&] {
        affine_assemble(pat, d_p, npts, d_t, nodes, ne, nq, h_X, h_W, coef_kind, d_coef, precision, d_values,
                        as_stream(stream), nullptr, nullptr);
    });
}

extern "C" int skg_p1_assemble_affine_forms(const skg_pattern *pat, const double *d_p, int64_t npts,
                                            const int32_t *d_t, int64_t ne, int32_t comp, int32_t nq,
                                            const double *h_X, const double *h_W, const double *d_value,
                                            const double *d_gradient, const double *d_symgrad,
                                            const double *d_div, double c_value, double c_gradient,
                                            double c_symgrad, double c_div, double *d_values, double *h_values,
                                            void *stream) {
    return guarded([&] {
        const double *coef[4] = {d_value, d_gradient, d_symgrad, d_div};
        const double cst[4] = {c_value, c_gradient, c_symgrad, c_div};
        p1_forms_assemble(pat, d_p, npts, d_t, ne, comp, nq, h_X, h_W, coef, cst, d_values, h_values,
                          as_stream(stream));
    });
}

extern "C" int skg_h1_assemble_affine_host(const skg_pattern *pat, const double *d_p, int64_t npts,
                                           const int32_t *d_t, int32_t nodes, int64_t ne, int32_t nq,
                                           const double *h_X, const double *h_W, int32_t coef_kind,
                                           const double *d_coef, int32_t precision, double *d_values,
                                           double *h_values, void *stream) {
    return guarded([&] {
        require(h_values != nullptr, "host output is NULL");
        affine_assemble(pat, d_p, npts, d_t, nodes, ne, nq, h_X, h_W, coef_kind, d_coef, precision, d_values,
                        as_stream(stream), nullptr, h_values);
    });
}

extern "C" int skg_h1_assemble_affine_profiled(const skg_pattern *pat, const double *d_p, int64_t npts,
                                               const int32_t *d_t, int32_t nodes, int64_t ne, int32_t nq,
                                               const double *h_X, const double *h_W, int32_t coef_kind,
                                               const double *d_coef, int32_t precision, double *d_values,
                                               float *h_kernel_ms, void *stream) {
    return guarded([&] {
        require(h_kernel_ms != nullptr, "timing output is NULL");
        cudaStream_t s = as_stream(stream);
        cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
        try {
            for (auto &e : ev) SKG_CUDA(cudaEventCreate(&e));
            affine_assemble(pat, d_p, npts, d_t, nodes, ne, nq, h_X, h_W, coef_kind, d_coef, precision, d_values, s,
                            ev, nullptr);
            SKG_CUDA(cudaEventSynchronize(ev[2]));
            SKG_CUDA(cudaEventElapsedTime(&h_kernel_ms[0], ev[0], ev[1]));
            SKG_CUDA(cudaEventElapsedTime(&h_kernel_ms[1], ev[1], ev[2]));
        } catch (...) {
            for (auto &e : ev)
                if (e) cudaEventDestroy(e);
            throw;
        }
        for (auto &e : ev) cudaEventDestroy(e);
    });
}

// ----------------------------------------------------------------------------
// Allocation-free variant of skg_h1_assemble_affine.
//
// Some callers cannot let a library call cudaMalloc: applications that hand
// all device memory to their own pool allocator at start-up and forbid other
// allocations, and time-stepping solvers that re-assemble inside a loop where
// a cudaMalloc / cudaFree (which may synchronise the device) is not allowed.
// This entry point computes exactly what skg_h1_assemble_affine computes, with
// the same kernels, but its scratch (per-element G, the quadrature table, the
// scale exponent and the range flag) lives in one file-scope device array of
// fixed size instead of stream-ordered allocations.  The array is part of the
// library's device image, so every GPU on which the library is loaded holds it
// (kNoAllocBytes) until the process exits.
namespace skg {
namespace {

constexpr int64_t kNoAllocMaxElements = 262144;  // SKG_NOALLOC_MAX_ELEMENTS
constexpr size_t kNoAllocGBytes = (size_t)kNoAllocMaxElements * 16 * 8;
constexpr size_t kNoAllocTBytes = 10 * 10 * 4 * 8;
constexpr size_t kNoAllocBytes = kNoAllocGBytes + kNoAllocTBytes + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kNoAllocMaxDevices = 64;
unsigned char *g_noalloc_base[kNoAllocMaxDevices] = {};
std::mutex g_noalloc_mutex;

// Device address of the scratch array on the current device, looked up once
// per device (host code cannot use the symbol itself: on the host its name
// denotes a shadow variable, not device memory).
unsigned char *noalloc_base() {
    int dev = 0;
    SKG_CUDA(cudaGetDevice(&dev));
    require(dev >= 0 && dev < kNoAllocMaxDevices, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_base[dev]) {
        void *ptr = nullptr;
        SKG_CUDA(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
        g_noalloc_base[dev] = static_cast<unsigned char *>(ptr);
    }
    return g_noalloc_base[dev];
}

// The quadrature table T of affine_table, written into a caller array (no
// host heap either).
void affine_table_fixed(int nodes, int nq, const double *X, const double *W, double T[10 * 10 * 4]) {
    for (int i = 0; i < 10 * 10 * 4; ++i) T[i] = 0.0;
    auto coeff = [&](int a, int slot, int q) -> double {
        const double x = X[q], y = X[nq + q], z = X[2 * nq + q];
        const double lam[4] = {1.0 - x - y - z, x, y, z};
        if (nodes == 4) return slot == 0 ? 1.0 : 0.0;
        if (a < 4) return slot == 0 ? 4.0 * lam[a] - 1.0 : 0.0;
        return slot == 0 ? 4.0 * lam[sup_hi(a)] : 4.0 * lam[sup_lo(a)];
    };
    for (int a = 0; a < nodes; ++a)
        for (int b = 0; b < nodes; ++b)
            for (int u = 0; u < 2; ++u)
                for (int v = 0; v < 2; ++v) {
                    if (u == 1 && sup_hi(a) == sup_lo(a)) continue;
                    if (v == 1 && sup_hi(b) == sup_lo(b)) continue;
                    double acc = 0.0;
                    for (int q = 0; q < nq; ++q) acc += W[q] * coeff(a, u, q) * coeff(b, v, q);
                    T[(a * nodes + b) * 4 + u * 2 + v] = acc;
                }
}

bool p2_table_is_exact(const double *T) {
    for (int a = 0; a < 10; ++a)
        for (int b = 0; b < 10; ++b)
            for (int sa = 0; sa < 2; ++sa)
                for (int sb = 0; sb < 2; ++sb) {
                    const bool used = (sa == 0 || sup_hi(a) != sup_lo(a)) && (sb == 0 || sup_hi(b) != sup_lo(b));
                    const double want = used ? t30(a, b, sa, sb) / 30.0 : 0.0;
                    if (std::fabs(T[(a * 10 + b) * 4 + sa * 2 + sb] - want) > 1e-13) return false;
                }
    return true;
}

}  // namespace
}  // namespace skg

extern "C" int skg_h1_assemble_affine_noalloc(const skg_pattern *pat, const double *d_p, int64_t npts,
                                              const int32_t *d_t, int32_t nodes, int64_t ne, int32_t nq,
                                              const double *h_X, const double *h_W, int32_t coef_kind,
                                              const double *d_coef, int32_t precision, double *d_values,
                                              void *stream) {
    return guarded([&] {
        require(pat != nullptr, "pattern is NULL");
        require(nodes == 4 || nodes == 10, "affine assembly supports P1 (4) and P2 (10) tetrahedra");
        require(ne == pat->n_elements && pat->row_local == nodes && pat->col_local == nodes,
                "mesh does not match the pattern");
        require(ne <= kNoAllocMaxElements,
                "allocation-free assembly supports at most " + std::to_string(kNoAllocMaxElements) +
                    " elements (its scratch array is fixed); got " + std::to_string(ne) +
                    ": use skg_h1_assemble_affine");
        require(coef_kind == 0 || ((coef_kind == 1 || coef_kind == 2) && (d_coef || ne == 0)), "invalid coefficient kind");
        require(precision == SKG_FP64 || precision == SKG_SPLIT_FP32 || precision == SKG_FP64_EMULATED,
                "invalid precision");
        require(nq > 0 && h_X && h_W, "quadrature rule is empty");
        require(ne == 0 || (d_p && d_t), "mesh arrays are NULL");
        cudaStream_t s = as_stream(stream);
        unsigned char *base = noalloc_base();
        double *G = reinterpret_cast<double *>(base);
        double *Tg = reinterpret_cast<double *>(base + kNoAllocGBytes);
        int *misc = reinterpret_cast<int *>(base + kNoAllocGBytes + kNoAllocTBytes);
        double T[10 * 10 * 4];
        affine_table_fixed(nodes, nq, h_X, h_W, T);
        // pageable source: the copy has read T before cudaMemcpyAsync returns
        SKG_CUDA(cudaMemcpyAsync(Tg, T, (size_t)nodes * nodes * 4 * 8, cudaMemcpyHostToDevice, s));
        const bool blocked = pat->max_row_len > 0;
        const bool exact = nodes == 10 && blocked && precision != SKG_FP64 && p2_table_is_exact(T);
        int mode = precision == SKG_FP64 ? MODE_FP64 : precision == SKG_SPLIT_FP32 ? MODE_SPLIT : MODE_DF64;
        if (!blocked) mode = MODE_FP64;
        if (mode != MODE_FP64) {
            // the array keeps the previous call's contents: reset the scale and the flag
            const int init[2] = {INT_MIN, 0};
            SKG_CUDA(cudaMemcpyAsync(misc, init, sizeof(init), cudaMemcpyHostToDevice, s));
            k_scale<<<2 * kSmCount, 256, 0, s>>>(d_p, 3 * npts, misc);
            SKG_LAUNCH_CHECK("scale");
            if (ne) {
                k_elem_df64<<<grid_for(ne, kElemBlock), kElemBlock, 0, s>>>(ne, d_p, npts, d_t, coef_kind, d_coef, misc,
                                                                           reinterpret_cast<float4 *>(G), misc + 1,
                                                                           exact);
                SKG_LAUNCH_CHECK("elem_df64");
            }
            int h_misc[2];
            SKG_CUDA(cudaMemcpyAsync(h_misc, misc, sizeof(h_misc), cudaMemcpyDeviceToHost, s));
            SKG_CUDA(cudaStreamSynchronize(s));
            if (h_misc[1] != 0 || h_misc[0] == INT_MIN) mode = MODE_FP64;
        }
        if (mode == MODE_FP64 && ne) {
            k_elem_fp64<<<grid_for(ne, kElemBlock), kElemBlock, 0, s>>>(ne, d_p, npts, d_t, coef_kind, d_coef,
                                                                       reinterpret_cast<float4 *>(G));
            SKG_LAUNCH_CHECK("elem_fp64");
        }
        if (!blocked) {
            Support sp{};
            for (int a = 0; a < 10; ++a) { sp.sup[a][0] = sup_lo(a); sp.sup[a][1] = sup_hi(a); }
            const unsigned grid = grid_for(pat->n_rows, 128);
            if (nodes == 4)
                k_rows_global<4><<<grid, 128, 0, s>>>(pat->n_rows, pat->indptr.get(), pat->indices.get(),
                                                      pat->inc_ptr.get(), pat->inc.get(), pat->col_dofs.get(), G, Tg,
                                                      sp, d_values);
            else
                k_rows_global<10><<<grid, 128, 0, s>>>(pat->n_rows, pat->indptr.get(), pat->indices.get(),
                                                       pat->inc_ptr.get(), pat->inc.get(), pat->col_dofs.get(), G, Tg,
                                                       sp, d_values);
            SKG_LAUNCH_CHECK("rows_global");
            return;
        }
        if (nodes == 4) {
            if (mode == MODE_FP64) launch_rows_groups<4, MODE_FP64>(pat, G, Tg, misc, d_values, s);
            else if (mode == MODE_SPLIT) launch_rows_groups<4, MODE_SPLIT>(pat, G, Tg, misc, d_values, s);
            else launch_rows_groups<4, MODE_DF64>(pat, G, Tg, misc, d_values, s);
        } else {
            if (mode == MODE_FP64) launch_rows_groups<10, MODE_FP64>(pat, G, Tg, misc, d_values, s);
            else if (mode == MODE_SPLIT) {
                if (exact) launch_rows_groups<10, MODE_SPLIT, true>(pat, G, Tg, misc, d_values, s);
                else launch_rows_groups<10, MODE_SPLIT>(pat, G, Tg, misc, d_values, s);
            } else {
                if (exact) launch_rows_groups<10, MODE_DF64, true>(pat, G, Tg, misc, d_values, s);
                else launch_rows_groups<10, MODE_DF64>(pat, G, Tg, misc, d_values, s);
            }
        }
    });
}
