// boys.cuh -- Boys function F_m(T) = int_0^1 t^{2m} exp(-T t^2) dt on the device.
//
// Method (tabulated Taylor expansion + downward recursion, as in Gill, Johnson
// & Pople, Int. J. Quantum Chem. 40, 745 (1991)):
//   * a grid T_k = k/16 (k < SQ_BOYS_NGRID) holds F_m(T_k) for m < 15 and
//     exp(-T_k), built once by the series F_m(T) = e^{-T} sum_i (2T)^i /
//     ((2m+1)(2m+3)...(2m+2i+1)) with compensated summation;
//   * for T < 36, F_m(T) = sum_j F_{m+j}(T_k) (-d)^j / j!, d = T - T_k,
//     |d| <= 1/32 (7 terms in FP64: truncation < 6e-15 relative; 4 in FP32);
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

#include "sq_common.cuh"

namespace sq {

constexpr int kBoysTaylor64 = 7;
constexpr int kBoysTaylor32 = 4;
constexpr double kSqrtPiHalf = 0.88622692545275801365;  // sqrt(pi)/2

// FP64: F[0..M] at T >= 0.  tab: SQ_BOYS_NGRID x SQ_BOYS_NCOL doubles.
template <int M>
__device__ __forceinline__ void boys64(double T, const double *__restrict__ tab, double (&F)[M + 1]) {
    static_assert(M + kBoysTaylor64 <= SQ_BOYS_NCOL - 1, "Boys table too narrow for this order");
    if (T < SQ_BOYS_TMAX) {
        const int k = __double2int_rn(T * SQ_BOYS_STEP_INV);
        const double d = T - k * (1.0 / SQ_BOYS_STEP_INV);
        const double *row = tab + k * SQ_BOYS_NCOL;
        // md[j] = -d / j
        double md[kBoysTaylor64];
#pragma unroll
        for (int j = 1; j < kBoysTaylor64; ++j) md[j] = -d * (1.0 / j);
        if constexpr (M <= 1) {
#pragma unroll
            for (int m = 0; m <= M; ++m) {
                double f = __ldg(row + m + kBoysTaylor64 - 1);
#pragma unroll
                for (int j = kBoysTaylor64 - 1; j >= 1; --j) f = fma(f, md[j], __ldg(row + m + j - 1));
                F[m] = f;
            }
        } else {
            double f = __ldg(row + M + kBoysTaylor64 - 1);
#pragma unroll
            for (int j = kBoysTaylor64 - 1; j >= 1; --j) f = fma(f, md[j], __ldg(row + M + j - 1));
            F[M] = f;
            double e = 1.0;
#pragma unroll
            for (int j = kBoysTaylor64 - 1; j >= 1; --j) e = fma(e, md[j], 1.0);
            e *= __ldg(row + SQ_BOYS_NCOL - 1);
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

// FP32 Boys from the FP32 copy of the grid.
template <int M>
__device__ __forceinline__ void boys32(float T, const float *__restrict__ tab, float (&F)[M + 1]) {
    if (T < (float)SQ_BOYS_TMAX) {
        const int k = __float2int_rn(T * (float)SQ_BOYS_STEP_INV);
        const float d = T - k * (1.0f / SQ_BOYS_STEP_INV);
        const float *row = tab + k * SQ_BOYS_NCOL;
        float md[kBoysTaylor32];
#pragma unroll
        for (int j = 1; j < kBoysTaylor32; ++j) md[j] = -d * (1.0f / j);
        if constexpr (M <= 1) {
#pragma unroll
            for (int m = 0; m <= M; ++m) {
                float f = __ldg(row + m + kBoysTaylor32 - 1);
#pragma unroll
                for (int j = kBoysTaylor32 - 1; j >= 1; --j) f = fmaf(f, md[j], __ldg(row + m + j - 1));
                F[m] = f;
            }
        } else {
            float f = __ldg(row + M + kBoysTaylor32 - 1);
#pragma unroll
            for (int j = kBoysTaylor32 - 1; j >= 1; --j) f = fmaf(f, md[j], __ldg(row + M + j - 1));
            F[M] = f;
            float e = 1.0f;
#pragma unroll
            for (int j = kBoysTaylor32 - 1; j >= 1; --j) e = fmaf(e, md[j], 1.0f);
            e *= __ldg(row + SQ_BOYS_NCOL - 1);
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
