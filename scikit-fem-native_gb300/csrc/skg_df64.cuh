// Double-float ("df64") arithmetic on the FP32 pipe: a value is the
// unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2 (about 48
// significant bits).  The operations are the classical error-free
// transformations: Knuth's TwoSum, Dekker's Fast2Sum, and the FMA-based exact
// product (p = a*b, e = fma(a, b, -p)).  GB300 runs FP32 FMA at 57x the FP64
// rate, so FP64-accurate contractions are cheaper this way than on the FP64
// pipe.
//
// Conversions between double and df64 are done with integer bit operations
// (no FP64 instructions): splitting keeps the top 24 mantissa bits in hi and
// rounds the remaining 29 bits into lo; joining reconstructs the exact double
// nearest to hi + lo.  Both apply a power-of-two scale 2^s in the exponent,
// so a mesh can be mapped into FP32 range exactly.  Values whose scaled
// exponent leaves the normal FP32 range are reported through the `range_ok`
// flag and handled by the caller (FP64 fallback).
#pragma once

#include <stdint.h>

namespace skg {

struct df64 {
    float hi, lo;
};

__device__ __forceinline__ df64 df_make(float h, float l) { return {h, l}; }

// s = a + b exactly as s + e (Knuth, any order of magnitude)
__device__ __forceinline__ df64 two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    const float e = (a - (s - bb)) + (b - bb);
    return {s, e};
}

// s = a + b exactly as s + e, requires |a| >= |b| (Dekker)
__device__ __forceinline__ df64 fast_two_sum(float a, float b) {
    const float s = a + b;
    const float e = b - (s - a);
    return {s, e};
}

// a * b exactly as p + e (FMA)
__device__ __forceinline__ df64 two_prod(float a, float b) {
    const float p = a * b;
    const float e = fmaf(a, b, -p);
    return {p, e};
}

__device__ __forceinline__ df64 df_add(df64 x, df64 y) {
    df64 s = two_sum(x.hi, y.hi);
    df64 t = two_sum(x.lo, y.lo);
    s.lo += t.hi;
    s = fast_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return fast_two_sum(s.hi, s.lo);
}

// Dekker's add: one TwoSum on the high parts, low parts added plainly.  Its
// error is bounded relative to the operands (as for an FP64 addition), which
// is all a geometric contraction needs; 11 instructions instead of 20.
__device__ __forceinline__ df64 df_add_fast(df64 x, df64 y) {
    df64 s = two_sum(x.hi, y.hi);
    s.lo += x.lo + y.lo;
    return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ df64 df_neg(df64 x) { return {-x.hi, -x.lo}; }

__device__ __forceinline__ df64 df_sub(df64 x, df64 y) { return df_add(x, df_neg(y)); }

__device__ __forceinline__ df64 df_mul(df64 x, df64 y) {
    df64 p = two_prod(x.hi, y.hi);
    p.lo = fmaf(x.hi, y.lo, p.lo);
    p.lo = fmaf(x.lo, y.hi, p.lo);
    return fast_two_sum(p.hi, p.lo);
}

// acc + x * y
__device__ __forceinline__ df64 df_fma(df64 x, df64 y, df64 acc) { return df_add(acc, df_mul(x, y)); }

// |x| inside the range the double-float paths accept (or zero)
__device__ __forceinline__ bool df_in_range(df64 x) {
    const float a = fabsf(x.hi);
    return a == 0.f || (a > 1e-30f && a < 1e30f);
}

// Scale exponent s of the vertex coordinates p (n doubles): |p| * 2^-s <= 1.
// *d_s must hold INT_MIN before the launch (it stays INT_MIN when every
// coordinate is zero or not finite).
void launch_scale_exponent(const double *d_p, int64_t n, int *d_s, cudaStream_t stream);

// 1 / x: float estimate refined by one Newton step in df64
__device__ __forceinline__ df64 df_recip(df64 x) {
    const float r = 1.0f / x.hi;
    // e = 1 - x * r (df64), r' = r + r * e
    df64 xr = df_mul(x, df64{r, 0.f});
    df64 e = df_sub(df64{1.f, 0.f}, xr);
    return df_add(df64{r, 0.f}, df_mul(df64{r, 0.f}, e));
}

// ---------------------------------------------------------------- conversions

// double -> df64 scaled by 2^s (exact up to rounding of the low 29 bits).
__device__ __forceinline__ df64 df_from_double(double d, int s, bool &range_ok) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const unsigned sign = (unsigned)(b >> 63) << 31;
    const int ex = (int)((b >> 52) & 0x7ff);
    if (ex == 0) {  // zero (subnormal inputs are flushed to zero)
        if ((b & 0x000fffffffffffffULL) != 0) range_ok = false;
        return {__uint_as_float(sign), 0.f};
    }
    if (ex == 0x7ff) {
        range_ok = false;
        return {__uint_as_float(sign | 0x7fc00000u), 0.f};
    }
    const int fe = ex - 1023 + 127 + s;  // float biased exponent of hi
    if (fe < 30 || fe > 253) {
        range_ok = false;
        return {0.f, 0.f};
    }
    const unsigned long long m = b & 0x000fffffffffffffULL;  // 52 fraction bits
    const float hi = __uint_as_float(sign | ((unsigned)fe << 23) | (unsigned)(m >> 29));
    const unsigned rest = (unsigned)(m & 0x1fffffffULL);    // low 29 bits, weight 2^(e-52)
    float lo = 0.f;
    if (rest) {
        // rest * 2^(fe-127-52): convert the integer, then shift its exponent
        const float r = __uint2float_rn(rest);
        const unsigned rb = __float_as_uint(r);
        const int re = (int)((rb >> 23) & 0xff) + (fe - 127 - 52);
        if (re >= 1) lo = __uint_as_float(sign | ((unsigned)re << 23) | (rb & 0x7fffffu));
    }
    return {hi, lo};
}

// float -> double bits scaled by 2^s (exact)
__device__ __forceinline__ unsigned long long float_to_double_bits(float f, int s) {
    const unsigned b = __float_as_uint(f);
    const unsigned long long sign = (unsigned long long)(b >> 31) << 63;
    const int fe = (int)((b >> 23) & 0xff);
    if (fe == 0) return sign;  // zero (FP32 subnormals do not occur in range-checked data)
    const unsigned long long ex = (unsigned long long)(fe - 127 + 1023 + s);
    return sign | (ex << 52) | ((unsigned long long)(b & 0x7fffffu) << 29);
}

// Nearest double to (hi + lo) * 2^s, where |lo| <= ulp(hi): the exact sum has
// at most 49 significant bits, so it is assembled in a 64-bit integer.
__device__ __forceinline__ double df_to_double(df64 x, int s) {
    if (x.lo == 0.f || x.hi == 0.f) {
        const float f = x.hi != 0.f ? x.hi : x.lo;
        return __longlong_as_double((long long)float_to_double_bits(f, s));
    }
    const unsigned hb = __float_as_uint(x.hi), lb = __float_as_uint(x.lo);
    const int he = (int)((hb >> 23) & 0xff), le = (int)((lb >> 23) & 0xff);
    const long long hm = (long long)((hb & 0x7fffffu) | 0x800000u);
    long long lm = (long long)((lb & 0x7fffffu) | (le ? 0x800000u : 0u));
    const int d = he - le;  // >= 23 when |lo| <= ulp(hi)/2
    if (d < 0 || d > 80) return __longlong_as_double((long long)float_to_double_bits(x.hi, s));
    if ((hb >> 31) != (lb >> 31)) lm = -lm;
    // integer M with hi at bits D..D+23 and lo aligned below it (bits shifted
    // out of lo become a sticky bit far below the double rounding position)
    const int D = d < 38 ? d : 38;
    const int sh_lo = d - D;
    long long lo_part = lm >> sh_lo;
    const bool inexact = sh_lo > 0 && (lm & ((1LL << sh_lo) - 1)) != 0;
    long long M = (hm << D) + lo_part;  // > 0 since |lo| < |hi|
    if (inexact) M |= 1;
    const int base_e = le + sh_lo;  // biased float exponent of bit 0 of M (+23 mantissa offset)
    // normalise M to 53 bits with round-to-nearest-even
    const int lz = __clzll(M);
    const int top = 63 - lz;  // position of leading bit
    int e2 = base_e - 127 - 23 + top;  // unbiased exponent of the result
    unsigned long long mant;
    if (top > 52) {
        const int sh = top - 52;
        const unsigned long long um = (unsigned long long)M;
        const unsigned long long half = 1ULL << (sh - 1);
        const unsigned long long rem = um & ((1ULL << sh) - 1);
        mant = um >> sh;
        if (rem > half || (rem == half && (mant & 1))) {
            ++mant;
            if (mant >> 53) { mant >>= 1; ++e2; }
        }
    } else {
        mant = (unsigned long long)M << (52 - top);
    }
    const unsigned long long sign = (unsigned long long)(hb >> 31) << 63;
    const unsigned long long bits = sign | ((unsigned long long)(e2 + 1023 + s) << 52) | (mant & 0x000fffffffffffffULL);
    return __longlong_as_double((long long)bits);
}

}  // namespace skg
