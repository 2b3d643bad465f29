// boys.cuh -- Boys function F_m(T) = int_0^1 t^{2m} exp(-T t^2) dt on the device.
//
// Method (tabulated Taylor expansion + downward recursion, as in Gill, Johnson
// & Pople, Int. J. Quantum Chem. 40, 745 (1991)):
//   * a grid T_k = k/16 (k < SQ_BOYS_NGRID) holds F_m(T_k) for m < 15 and
//     exp(-T_k), built once by the series F_m(T) = e^{-T} sum_i (2T)^i /
//     ((2m+1)(2m+3)...(2m+2i+1)) with compensated summation, and the scaled
//     Taylor coefficients F_{m+j}(T_k)/j!, exp(-T_k)/j!;
//   * for T < 36, F_m(T) = sum_j [F_{m+j}(T_k)/j!] (-d)^j, d = T - T_k,
//     |d| <= 1/32 (7 terms in FP64: truncation < 6e-15 relative; 5 in FP32:
//     < 3e-10, so the always-positive remainder adds no FP32-sized bias),
//     a Horner chain of FMAs only;
//     for m_max >= 2 only F_{m_max} is expanded and the lower orders follow
//     from the stable downward recursion (2m+1) F_m = 2T F_{m+1} + e^{-T},
//     with e^{-T} = e^{-T_k} e^{-d} from the same grid;
//   * for T >= 36, F_0 = sqrt(pi/T)/2 (erfc(6) < 3e-17) and the upward
//     recursion F_{m+1} = (2m+1)/(2T) F_m (the e^{-T} term is below 3e-18).
//
// The reference evaluates F_n by its own piecewise formula
// (slowquant/molecularintegrals/integralfunctions.py:74-97: erf for n = 0, a
// series to 1e-12 absolute for 1e-10 < z <= 25, the large-z asymptote beyond);
// both agree with the exact function to ~1e-12, far below the 1e-10 parity
// tolerance on integrals.
#pragma once

#include "df64.cuh"
#include "sq_common.cuh"

namespace sq {

constexpr int kBoysTaylor64 = 7;
constexpr int kBoysTaylor32 = 5;
constexpr double kSqrtPiHalf = 0.88622692545275801365;  // sqrt(pi)/2

// Grid point of T (T >= 0, T < 36) computed on the FP32 / integer pipes, and
// d = T - k/16 exactly: k/16 is built from the bit pattern of 2^48 + k/16
// (a double with ulp 2^-4), so no FP64 conversion instruction is needed.
__device__ __forceinline__ double boys_offset(double T, float Tf, int &k) {
    k = __float2int_rn(Tf * (float)SQ_BOYS_STEP_INV);
    const double kd16 = __longlong_as_double(0x42F0000000000000LL + (long long)k) - 281474976710656.0;
    return T - kd16;
}

// Horner sum_j c[j] x^j of the 7 scaled Taylor coefficients of one grid row.
__device__ __forceinline__ double taylor7(const double *__restrict__ row, double x) {
    const double2 c01 = __ldg(reinterpret_cast<const double2 *>(row));
    const double2 c23 = __ldg(reinterpret_cast<const double2 *>(row + 2));
    const double2 c45 = __ldg(reinterpret_cast<const double2 *>(row + 4));
    const double c6 = __ldg(row + 6);
    double f = fma(c6, x, c45.y);
    f = fma(f, x, c45.x);
    f = fma(f, x, c23.y);
    f = fma(f, x, c23.x);
    f = fma(f, x, c01.y);
    return fma(f, x, c01.x);
}


// FP64: F[0..M] at T >= 0.  tab: the FP64 table (SQ_BOYS_TAB64_SIZE doubles).
template <int M>
__device__ __forceinline__ void boys64(double T, const double *__restrict__ tab, double (&F)[M + 1]) {
    static_assert(M + kBoysTaylor64 <= SQ_BOYS_NCOL - 1, "Boys table too narrow for this order");
    const float Tf = d2f_bits(T);
    if (Tf < (float)SQ_BOYS_TMAX) {
        int k;
        const double md = -boys_offset(T, Tf, k);
        const double *tay = tab + SQ_BOYS_TAY64_OFF + k * 8;
        if constexpr (M <= 1) {
#pragma unroll
            for (int m = 0; m <= M; ++m) F[m] = taylor7(tay + m * SQ_BOYS_NGRID * 8, md);
        } else {
            F[M] = taylor7(tay + M * SQ_BOYS_NGRID * 8, md);
            const double e = taylor7(tay + 15 * SQ_BOYS_NGRID * 8, md);
            const double T2 = T + T;
#pragma unroll
            for (int m = M - 1; m >= 0; --m) F[m] = fma(T2, F[m + 1], e) * (1.0 / (2 * m + 1));
        }
    } else {
        const double r = rsqrt(T);
        F[0] = kSqrtPiHalf * r;
        if constexpr (M >= 1) {
            const double h = 0.5 * r * r;  // 1/(2T)
#pragma unroll
            for (int m = 0; m < M; ++m) F[m + 1] = F[m] * ((2 * m + 1) * h);
        }
    }
}

// Taylor sum of one double-float row (SQ_BOYS_DF_OFF) at md = T_k - T:
// coefficients 4-6 in FP32 (their terms are below 4e-8 of the sum for
// |md| <= 1/32, so FP32 rounding there stays near 2^-48 of the result), 0-3
// in double-float.
__device__ __forceinline__ dfl taylor_df(const float4 *__restrict__ row, dfl md) {
    const float4 a = __ldg(row), b = __ldg(row + 1), c = __ldg(row + 2);
    const float g = __fmaf_rn(__fmaf_rn(c.z, md.hi, c.y), md.hi, c.x);
    dfl f = fma(dfl(g), md, dfl(b.z, b.w));
    f = fma(f, md, dfl(b.x, b.y));
    f = fma(f, md, dfl(a.z, a.w));
    return fma(f, md, dfl(a.x, a.y));
}

// Double-float F[0..M] at T >= 0 (the df64 J/K kernels), the scheme of boys64
// on the FP32 pipe.  tab: the double-float rows (float4 view of
// table32 + SQ_BOYS_DF_OFF).  md = T_k - T is exact in its high part
// (k/16 and T.hi are within a factor of two of each other for k >= 1).
template <int M>
__device__ __forceinline__ void boys_df(dfl T, const float4 *__restrict__ tab, dfl (&F)[M + 1]) {
    static_assert(M + kBoysTaylor64 <= SQ_BOYS_NCOL - 1, "Boys table too narrow for this order");
    if (T.hi < (float)SQ_BOYS_TMAX) {
        const int k = __float2int_rn(__fmul_rn(T.hi, (float)SQ_BOYS_STEP_INV));
        const dfl md = df_two_sum(__fsub_rn(__fmul_rn((float)k, 1.0f / SQ_BOYS_STEP_INV), T.hi), -T.lo);
        const float4 *tay = tab + (long long)k * 3;
        if constexpr (M <= 1) {
#pragma unroll
            for (int m = 0; m <= M; ++m) F[m] = taylor_df(tay + m * SQ_BOYS_NGRID * 3, md);
        } else {
            F[M] = taylor_df(tay + M * SQ_BOYS_NGRID * 3, md);
            const dfl e = taylor_df(tay + 15 * SQ_BOYS_NGRID * 3, md);
            const dfl T2(__fadd_rn(T.hi, T.hi), __fadd_rn(T.lo, T.lo));
#pragma unroll
            for (int m = M - 1; m >= 0; --m) F[m] = fma(T2, F[m + 1], e) * dfl(1.0 / (2 * m + 1));
        }
    } else {
        const dfl r = rsqrt_df(T);
        F[0] = dfl(kSqrtPiHalf) * r;
        if constexpr (M >= 1) {
            const dfl r2 = r * r;
            const dfl h(__fmul_rn(0.5f, r2.hi), __fmul_rn(0.5f, r2.lo));  // 1/(2T)
#pragma unroll
            for (int m = 0; m < M; ++m) F[m + 1] = df_mul(F[m] * h, (float)(2 * m + 1));
        }
    }
}

// The two blocks of the FP32 Taylor table an order-M evaluation reads (in
// shared memory): coefficients 0-3 of each grid row as a float4, and the
// fifth coefficient.  For M <= 1 the blocks are those of orders 0 and 1; for
// M >= 2, block 0 is order M and block 1 the exp block.
struct Boys32Blocks {
    const float4 *c0, *c1;
    const float *e0, *e1;
};

// 5-term Taylor sum at md = -(T - T_k).  Five terms, not four: the remainder
// of a truncated expansion of F_m is F_{m+n}(xi) d^n / n! > 0 whatever the
// sign of d (every derivative of order n of F_m is (-1)^n F_{m+n}), so a
// 4-term sum is biased low by up to 4e-8 relative at |d| <= 1/32 -- a
// coherent bias that the energy accumulates over millions of FP32 primitive
// quartets; the fifth term brings it to 2.5e-10.
__device__ __forceinline__ float taylor5(float4 c, float e, float md) {
    return fmaf(fmaf(fmaf(fmaf(e, md, c.w), md, c.z), md, c.y), md, c.x);
}

// FP32 Boys from the table blocks tb; truncation < 3e-10 relative for T < 36.
template <int M>
__device__ __forceinline__ void boys32(float T, const Boys32Blocks &tb, float (&F)[M + 1]) {
    if (T < (float)SQ_BOYS_TMAX) {
        const int k = __float2int_rn(T * (float)SQ_BOYS_STEP_INV);
        const float md = k * (1.0f / SQ_BOYS_STEP_INV) - T;
        F[M <= 1 ? 0 : M] = taylor5(tb.c0[k], tb.e0[k], md);
        if constexpr (M == 1) {
            F[1] = taylor5(tb.c1[k], tb.e1[k], md);
        } else if constexpr (M >= 2) {
            const float e = taylor5(tb.c1[k], tb.e1[k], md);
            const float T2 = T + T;
#pragma unroll
            for (int m = M - 1; m >= 0; --m) F[m] = fmaf(T2, F[m + 1], e) * (1.0f / (2 * m + 1));
        }
    } else {
        const float r = rsqrtf(T);
        F[0] = (float)kSqrtPiHalf * r;
        if constexpr (M >= 1) {
            const float h = 0.5f * r * r;
#pragma unroll
            for (int m = 0; m < M; ++m) F[m + 1] = F[m] * ((2 * m + 1) * h);
        }
    }
}

// Mixed Boys for FP32 quartets: F_M and e^{-T} from the FP32 table (Taylor,
// FP32), then the downward recursion (2m+1) F_m = 2T F_{m+1} + e^{-T} in FP64;
// the results are handed back as FP32.  M <= 1 needs no recursion (each order
// has its own FP32 expansion), so those classes stay entirely in FP32.
template <int M>
__device__ __forceinline__ void boys_mixed(float T, const Boys32Blocks &tb, float (&F)[M + 1]) {
    if constexpr (M <= 1) {
        boys32<M>(T, tb, F);
    } else {
        if (T < (float)SQ_BOYS_TMAX) {
            const int k = __float2int_rn(T * (float)SQ_BOYS_STEP_INV);
            const float md = k * (1.0f / SQ_BOYS_STEP_INV) - T;
            const float f = taylor5(tb.c0[k], tb.e0[k], md);
            const float e = taylor5(tb.c1[k], tb.e1[k], md);
            F[M] = f;
            const double T2 = f2d_bits(T + T), ed = f2d_bits(e);
            double fd = f2d_bits(f);
#pragma unroll
            for (int m = M - 1; m >= 0; --m) {
                fd = fma(T2, fd, ed) * (1.0 / (2 * m + 1));
                F[m] = d2f_bits(fd);
            }
        } else {
            boys32<M>(T, tb, F);
        }
    }
}

// Blocks of the FP32 Taylor table used by an order-M evaluation.
template <int M>
__host__ __device__ constexpr int boys32_block(int which) {
    return M <= 1 ? which : (which == 0 ? M : 15);
}

// Runtime-order FP64 Boys (used by the one-electron kernel and the test hook):
// F[0..m_max], m_max < SQ_BOYS_NCOL - kBoysTaylor64 + 1.
__device__ inline void boys64_rt(int m_max, double T, const double *__restrict__ tab, double *F) {
    if (T < SQ_BOYS_TMAX) {
        const int k = __double2int_rn(T * SQ_BOYS_STEP_INV);
        const double d = T - k * (1.0 / SQ_BOYS_STEP_INV);
        const double *row = tab + k * SQ_BOYS_NCOL;
        double md[kBoysTaylor64];
        for (int j = 1; j < kBoysTaylor64; ++j) md[j] = -d / j;
        double f = row[m_max + kBoysTaylor64 - 1];
        for (int j = kBoysTaylor64 - 1; j >= 1; --j) f = fma(f, md[j], row[m_max + j - 1]);
        F[m_max] = f;
        double e = 1.0;
        for (int j = kBoysTaylor64 - 1; j >= 1; --j) e = fma(e, md[j], 1.0);
        e *= row[SQ_BOYS_NCOL - 1];
        for (int m = m_max - 1; m >= 0; --m) F[m] = fma(T + T, F[m + 1], e) / (2 * m + 1);
    } else {
        const double r = rsqrt(T);
        F[0] = kSqrtPiHalf * r;
        const double h = 0.5 * r * r;
        for (int m = 0; m < m_max; ++m) F[m + 1] = F[m] * ((2 * m + 1) * h);
    }
}

// High-order FP64 Boys F_m(T), m <= 16, from the grid at SQ_BOYS_HI64_OFF
// (the classes with f shells reach m = 12): the same 7-term Taylor expansion
// about the nearest grid point, each order on its own; beyond
// SQ_BOYS_HI_TMAX (60) the asymptote F_m = sqrt(pi/T)/2 prod_{j<m} (2j+1)/(2T),
// whose neglected term is below 2e-13 relative for m <= 13 there.
__device__ __forceinline__ double boys_hi(int m, double T, const double *__restrict__ tab64) {
    if (T < SQ_BOYS_HI_TMAX) {
        const int k = __double2int_rn(T * SQ_BOYS_STEP_INV);
        const double d = T - k * (1.0 / SQ_BOYS_STEP_INV);
        const double *row = tab64 + SQ_BOYS_HI64_OFF + k * SQ_BOYS_HI_NCOL + m;
        double f = __ldg(row + kBoysTaylor64 - 1);
#pragma unroll
        for (int j = kBoysTaylor64 - 1; j >= 1; --j) f = fma(f, -d * (1.0 / j), __ldg(row + j - 1));
        return f;
    }
    const double r = rsqrt(T);
    double f = kSqrtPiHalf * r;
    const double h = 0.5 * r * r;
    for (int j = 0; j < m; ++j) f *= (2 * j + 1) * h;
    return f;
}

// Reference-compatible Boys function: the piecewise formula of
// slowquant/molecularintegrals/integralfunctions.py:74-97 restated term for
// term (erf form for n = 0, large-z asymptote for z > 25, zero-z limit, and
// the series sum (2z)^i / (2n+2i+1)!! stopped when a term changes the
// unscaled sum by less than 1e-12).  Its truncation differs from the exact
// function by up to ~1e-5 relative for high orders at small z, which moves
// some integrals by ~1e-10; the dense-tensor and Schwarz outputs use it so
// that they reproduce the reference's arrays, the direct Fock build uses the
// accurate tabulated function above.
__device__ inline double factorial2_ref(double number) {
    double out = 1.0;
    if (number > 0) {
        const int n = (int)(number + 1) / 2;
        for (int i = 0; i < n; ++i) out = out * (number - 2 * i);
    }
    return out;
}

__device__ inline double boys_reference(int n, double z) {
    const double pi = 3.141592653589793;
    if (n == 0 && z < 1e-10) return 1.0;
    if (n == 0) return sqrt(pi / (4.0 * z)) * erf(sqrt(z));
    if (z > 25) return factorial2_ref(2 * n - 1) / pow(2.0, n + 1.0) * sqrt(pi / pow(z, 2.0 * n + 1.0));
    if (z < 1e-10) return 1.0 / (2.0 * n + 1.0);
    double F = 0.0;
    for (int i = 0; i < 1000; ++i) {
        double Fcheck = F;
        F += pow(2.0 * z, (double)i) / factorial2_ref(2 * n + 2 * i + 1);
        Fcheck -= F;
        if (fabs(Fcheck) < 1e-12) break;
    }
    return F * exp(-z) * factorial2_ref(2 * n - 1);
}

}  // namespace sq
