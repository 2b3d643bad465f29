// df64.cuh -- double-float ("df64") arithmetic for the J/K kernels.
//
// GB300 runs FP32 at about 60 times its FP64 rate (128 FP32 lanes per SM and
// clock against roughly two FP64 FMAs), so the per-thread J/K kernels that
// need more than FP32 accuracy can carry each real number as an unevaluated
// sum hi + lo of two floats and do all their arithmetic on the FP32 pipe.
// The operations are the classical error-free transformations (Dekker,
// "A floating-point technique for extending the available precision",
// Numer. Math. 18 (1971); Knuth's two-sum, TAOCP vol. 2 sec. 4.2.2; the
// FMA-based exact product), combined the way the "sloppy" double-double
// operations of Hida, Li & Bailey's QD library are (ARITH-15, 2001):
//   two_sum(a, b):      s = a + b, e = (a - (s - bb)) + (b - bb), bb = s - a   (exact)
//   fast_two_sum(s, e): h = s + e, l = e - (h - s)                            (|s| >= |e|)
//   product:            p = a.hi b.hi, e = fma(a.hi, b.hi, -p) + a.hi b.lo + a.lo b.hi
// Each result carries about 46 significant bits (relative error near 2^-46
// of the operands' magnitude for sums), against 53 for FP64 and 24 for FP32;
// the exponent range is FP32's, which covers every quantity of these kernels
// (the FP32 kernels evaluate the same quantities).  The intrinsics __fadd_rn,
// __fsub_rn, __fmul_rn and __fmaf_rn keep the compiler from contracting or
// reordering the transformations.
#pragma once

#include "sq_common.cuh"

namespace sq {

struct dfl {
    float hi, lo;
    dfl() = default;
    __host__ __device__ constexpr dfl(float h, float l) : hi(h), lo(l) {}
    // exact for |x| < 2^24
    __host__ __device__ constexpr explicit dfl(int x) : hi((float)x), lo(0.0f) {}
    __host__ __device__ constexpr explicit dfl(float x) : hi(x), lo(0.0f) {}
    // nearest double-float of a double (constants; folded at compile time)
    __host__ __device__ constexpr explicit dfl(double x) : hi((float)x), lo((float)(x - (double)(float)x)) {}
};

// h + l = s + e exactly when |s| >= |e| (Dekker's fast two-sum).
__device__ __forceinline__ dfl df_fast(float s, float e) {
    const float h = __fadd_rn(s, e);
    return dfl(h, __fsub_rn(e, __fsub_rn(h, s)));
}

// s + e = a + b exactly, any magnitudes (Knuth's two-sum).
__device__ __forceinline__ dfl df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return dfl(s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb)));
}

__device__ __forceinline__ dfl operator-(dfl a) { return dfl(-a.hi, -a.lo); }

__device__ __forceinline__ dfl operator+(dfl a, dfl b) {
    const dfl s = df_two_sum(a.hi, b.hi);
    return df_fast(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ dfl operator-(dfl a, dfl b) { return a + (-b); }

__device__ __forceinline__ dfl operator*(dfl a, dfl b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return df_fast(p, e);
}

// double-float times float
__device__ __forceinline__ dfl df_mul(dfl a, float b) {
    const float p = __fmul_rn(a.hi, b);
    float e = __fmaf_rn(a.hi, b, -p);
    e = __fmaf_rn(a.lo, b, e);
    return df_fast(p, e);
}

// The double-float fma below would hide the FP64 and FP32 ones from
// unqualified calls inside namespace sq.
using ::fma;
using ::fmaf;

// a b + c with one rounding of the product's error term into the sum.
__device__ __forceinline__ dfl fma(dfl a, dfl b, dfl c) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    const dfl s = df_two_sum(p, c.hi);
    return df_fast(s.hi, __fadd_rn(s.lo, __fadd_rn(e, c.lo)));
}

__device__ __forceinline__ dfl &operator+=(dfl &a, dfl b) { return a = a + b; }
__device__ __forceinline__ dfl &operator*=(dfl &a, dfl b) { return a = a * b; }

// a + x for a float x (adds an FP32 partial sum into a double-float one).
__device__ __forceinline__ dfl df_add(dfl a, float x) {
    const dfl s = df_two_sum(a.hi, x);
    return df_fast(s.hi, __fadd_rn(s.lo, a.lo));
}

// x^{-1/2}: the FP32 estimate y0 refined by one Newton step carried to second
// order, y = y0 (1 + e/2 + 3e^2/8) with e = 1 - x y0^2.  e is formed from the
// exact products x.hi y0 and (x.hi y0) y0 (1 - q is exact for q near 1), so it
// is accurate to FP32 relative precision; the correction y0 (e/2 + 3e^2/8)
// (about 2^-22 of y0) then needs only FP32 arithmetic.  Error O(e^3).
__device__ __forceinline__ dfl rsqrt_df(dfl x) {
    const float y0 = rsqrtf(x.hi);
    const float p = __fmul_rn(x.hi, y0);
    float pe = __fmaf_rn(x.hi, y0, -p);
    pe = __fmaf_rn(x.lo, y0, pe);
    const float q = __fmul_rn(p, y0);
    float qe = __fmaf_rn(p, y0, -q);
    qe = __fmaf_rn(pe, y0, qe);
    const float e = __fsub_rn(__fsub_rn(1.0f, q), qe);
    const float corr = __fmul_rn(y0, __fmul_rn(e, __fmaf_rn(0.375f, e, 0.5f)));
    return df_fast(y0, corr);
}

__device__ __forceinline__ dfl df_load(const dfl *p) {
    const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
    return dfl(v.x, v.y);
}

// Sum of the two parts in FP64 (conversions on the integer pipe).
__device__ __forceinline__ double df_to_double(dfl x) { return f2d_bits(x.hi) + f2d_bits(x.lo); }

}  // namespace sq
