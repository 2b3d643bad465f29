// eri.cuh -- McMurchie-Davidson shell-quartet kernels, one template per
// quartet class (LA LB | LC LD), one thread per contracted shell quartet.
//
// For every primitive quartet (bra pair ij, ket pair kl) the thread forms
//   R_{tuv}(alpha, P-Q), t+u+v <= L,  scaled by 2 pi^{5/2} U_ij U_kl / sqrt(p+q)
// (Boys function + the Hermite Coulomb recurrences of
// slowquant/molecularintegrals/integralfunctions.py:100-148), contracts it with
// the ket's Hermite coefficients into W[tuv][cd] (summed over ket primitive
// pairs), and once per bra primitive pair contracts W with the bra's Hermite
// coefficients into the contracted block (ab|cd).  This is the arithmetic of
// electron_repulsion_integral (slowquant/molecularintegrals/electronrepulsion.py:
// 107-297) reordered so that the contraction over ket primitives happens in
// Hermite space; normalisation and contraction coefficients are folded into
// the pair data.
//
// Epilogues: MODE_DENSE scatters the block to the eight index permutations of
// a dense tensor (electronrepulsion.py:72-103); MODE_SCHWARZ stores
// sqrt(max(block)) for diagonal quartets (electronrepulsion.py:300-339);
// MODE_JK digests the block into Coulomb / exchange accumulators with the
// 8-fold permutational weights (hartreefock_in_memory.py:55-56 without the
// stored tensor).
#pragma once

#include <type_traits>

#include "boys.cuh"
#include "df64.cuh"
#include "sq_common.cuh"

namespace sq {

enum { MODE_DENSE = 0, MODE_SCHWARZ = 1, MODE_JK = 2 };
enum { BOYS_FP64 = 0, BOYS_FP32 = 1, BOYS_REF = 2 };

struct EriArgs {
    sq_basis basis;
    sq_pairs pairs;
    sq_slots slots;   // J/K and dense lists hold slot ids
    int use_slots;    // 0: quartet entries are pair ids (Schwarz lists)
    const int2 *quartets;
    long long nq;
    const double *tab64;
    const float *tab32;
    const double *D;
    const float *D32;
    double *Jacc;
    double *Kacc;
    double *V;
    double *q;
    int cfg_threads;        // 0: built-in launch shape
    long long cfg_blocks;
    int nd;                 // J/K: densities digested per integral (0 or 1: one)
    long long dstride;      // elements between consecutive densities / accumulators
    float prim_tau;         // SQ_FP64_PRIM / SQ_DF64 launches: primitive quartets with q_ij q_kl < prim_tau run in FP32
    const float *Ddf;       // SQ_DF64: the density as (hi, lo) float pairs
};

template <typename R>
constexpr bool is_df = std::is_same<R, dfl>::value;

constexpr double kTwoPi52 = 34.98683665524972;  // 2 pi^{5/2}

template <typename R>
__device__ __forceinline__ const R *herm_ptr(const sq_pairs &pr) {
    if constexpr (std::is_same<R, double>::value)
        return pr.herm;
    else
        return pr.herm32;
}
template <typename R>
__device__ __forceinline__ const R *prim_ptr(const sq_pairs &pr) {
    if constexpr (std::is_same<R, double>::value)
        return pr.prim;
    else
        return pr.prim32;
}

template <typename R>
__device__ __forceinline__ const R *slot_prim_ptr(const sq_slots &sl) {
    if constexpr (std::is_same<R, double>::value)
        return sl.prim;
    else
        return sl.prim32;
}
template <typename R>
__device__ __forceinline__ const R *slot_herm_ptr(const sq_slots &sl) {
    if constexpr (std::is_same<R, double>::value)
        return sl.herm;
    else if constexpr (is_df<R>)
        return reinterpret_cast<const dfl *>(sl.hermdf);
    else
        return sl.herm32;
}

// x^{-1/2} in FP64 with few FP64 instructions (the FP64 pipe bounds these
// kernels; the FP32 and integer pipes are idle): an FP32 estimate y0 (about 23
// correct bits, conversions on the integer pipe) refined by one step of
// Newton's iteration for f(y) = y^{-2} - x carried to second order,
//   e = 1 - x y0^2,   y = y0 (1 + e/2 + 3 e^2 / 8),
// whose error is O(e^3), below the FP64 rounding for |e| < 1e-6.  Five FP64
// operations.  x must be a positive normal double in the FP32 range.
__device__ __forceinline__ double rsqrt_f64(double x) {
    const double y0 = f2d_bits(rsqrtf(d2f_bits(x)));
    const double e = fma(-x * y0, y0, 1.0);
    const double y0e = y0 * e;
    return fma(y0e, fma(0.375, e, 0.5), y0);
}

template <typename R>
__device__ __forceinline__ R rsqrt_r(R x) {
    if constexpr (std::is_same<R, double>::value)
        return rsqrt_f64(x);
    else if constexpr (is_df<R>)
        return rsqrt_df(x);
    else
        return rsqrtf(x);
}

// Scaled R^{(0)}_{tuv} table for t+u+v <= L from Fs[n] = pref (-2 alpha)^n F_n.
template <int L, typename R>
__device__ __forceinline__ void hermite_r(const R (&Fs)[L + 1], R X, R Y, R Z, R (&out)[L + 1][L + 1][L + 1]) {
    R cur[L + 1][L + 1][L + 1];
    cur[0][0][0] = Fs[L];
#pragma unroll
    for (int n = L - 1; n >= 0; --n) {
        R nxt[L + 1][L + 1][L + 1];
        nxt[0][0][0] = Fs[n];
        const int top = L - n;
#pragma unroll
        for (int t = 0; t <= top; ++t)
#pragma unroll
            for (int u = 0; u <= top - t; ++u)
#pragma unroll
                for (int v = 0; v <= top - t - u; ++v) {
                    if (t + u + v == 0) continue;
                    R val;
                    if (t > 0) {
                        val = X * cur[t - 1][u][v];
                        if (t > 1) val = fma(R(t - 1), cur[t - 2][u][v], val);
                    } else if (u > 0) {
                        val = Y * cur[0][u - 1][v];
                        if (u > 1) val = fma(R(u - 1), cur[0][u - 2][v], val);
                    } else {
                        val = Z * cur[0][0][v - 1];
                        if (v > 1) val = fma(R(v - 1), cur[0][0][v - 2], val);
                    }
                    nxt[t][u][v] = val;
                }
#pragma unroll
        for (int t = 0; t <= top; ++t)
#pragma unroll
            for (int u = 0; u <= top - t; ++u)
#pragma unroll
                for (int v = 0; v <= top - t - u; ++v) cur[t][u][v] = nxt[t][u][v];
    }
#pragma unroll
    for (int t = 0; t <= L; ++t)
#pragma unroll
        for (int u = 0; u <= L - t; ++u)
#pragma unroll
            for (int v = 0; v <= L - t - u; ++v) out[t][u][v] = cur[t][u][v];
}

template <typename T>
__device__ __forceinline__ T gload(const T *p) {
    if constexpr (is_df<T>)
        return df_load(p);
    else
        return __ldg(p);
}

// Per-slot descriptor (sq_slots::desc): primitive-pair layout of the slot and
// what the J/K epilogue needs to index the n x n matrices.
struct SlotDesc {
    int npp, pbase, pstride, hbase;
    int oa, ob;   // first basis function of shells a, b (molecule-local)
    int pairf;    // pair index, bit 30 set when a == b
    int ld;       // leading dimension of the molecule's matrices
};

__device__ __forceinline__ SlotDesc load_desc(const int *desc, int s) {
    const int4 *d = reinterpret_cast<const int4 *>(desc) + 2 * (long long)s;
    const int4 x = __ldg(d), y = __ldg(d + 1);
    return SlotDesc{x.x, x.y, x.z, x.w, y.x, y.y, y.z, y.w};
}

// The primitive half of a descriptor and, separately, its epilogue half (oa,
// ob, pairf, ld), for kernels that load the latter only after the primitive
// loops to keep it out of their registers.
__device__ __forceinline__ SlotDesc load_desc_prims(const int *desc, int s) {
    const int4 x = __ldg(reinterpret_cast<const int4 *>(desc) + 2 * (long long)s);
    return SlotDesc{x.x, x.y, x.z, x.w, 0, 0, 0, 0};
}

__device__ __forceinline__ void load_desc_epilogue(const int *desc, int s, SlotDesc &d) {
    const int4 y = __ldg(reinterpret_cast<const int4 *>(desc) + 2 * (long long)s + 1);
    d.oa = y.x;
    d.ob = y.y;
    d.pairf = y.z;
    d.ld = y.w;
}

// Fields of one primitive pair of the slot layout: exponent sum, centre, U.
template <typename R>
struct PrimPair {
    R p, x, y, z, u;
};

// FP64 and double-float read the field-major arrays (five coalesced loads),
// FP32 the packed copy (one 16-byte load plus one 4-byte load).
template <typename R>
__device__ __forceinline__ PrimPair<R> load_prim(const sq_slots &sl, long long idx) {
    if constexpr (std::is_same<R, double>::value) {
        const long long NPP = sl.npp_total;
        return PrimPair<R>{__ldg(sl.prim + idx), __ldg(sl.prim + NPP + idx), __ldg(sl.prim + 2 * NPP + idx),
                           __ldg(sl.prim + 3 * NPP + idx), __ldg(sl.prim + 4 * NPP + idx)};
    } else if constexpr (is_df<R>) {
        const long long NPP = sl.npp_total;
        const dfl *pd = reinterpret_cast<const dfl *>(sl.primdf);
        return PrimPair<R>{df_load(pd + idx), df_load(pd + NPP + idx), df_load(pd + 2 * NPP + idx),
                           df_load(pd + 3 * NPP + idx), df_load(pd + 4 * NPP + idx)};
    } else {
        const float4 a = __ldg(reinterpret_cast<const float4 *>(sl.prim32v) + 2 * idx);
        return PrimPair<R>{a.x, a.y, a.z, a.w, __ldg(sl.prim32v + 8 * idx + 4)};
    }
}

// W[tuv][cd] of one bra primitive pair (exponent sum p, centre P) summed
// over the ket primitive pairs k0 <= k < k1 of slot kd, in precision R:
//   W[tuv][cd] += sum_k U_k / sqrt(p+q) sum_{tau nu phi} (-1)^{tau+nu+phi} E^{cd}_{tau nu phi}(k) R_{t+tau,u+nu,v+phi}
template <int LA, int LB, int LC, int LD, typename R, int BOYS>
__device__ __forceinline__ void ket_loop(const EriArgs &args, R p, R Px, R Py, R Pz, const SlotDesc &kd, int k0, int k1,
                                         const Boys32Blocks &tb,
                                         R (&W)[LA + LB + 1][LA + LB + 1][LA + LB + 1][ncart(LC) * ncart(LD)]) {
    constexpr int NC = ncart(LC), ND = ncart(LD);
    constexpr int LAB = LA + LB, LCD = LC + LD, L = LAB + LCD;
    constexpr int EK = herm_size(LC, LD);
    constexpr bool KET_S = (LCD == 0);
    const sq_slots &sl = args.slots;
    const R *hk = slot_herm_ptr<R>(sl) + kd.hbase;
    const int pk = kd.pbase, sk = kd.pstride;
    for (int k = k0; k < k1; ++k) {
        const PrimPair<R> kt = load_prim<R>(sl, pk + (long long)k * sk);
        const R q = kt.p;
        const R X = Px - kt.x;
        const R Y = Py - kt.y;
        const R Z = Pz - kt.z;
        const R Uk = kt.u;
        const R r = rsqrt_r(p + q);
        const R alpha = p * q * (r * r);
        const R T = alpha * (X * X + Y * Y + Z * Z);
        R F[L + 1];
        if constexpr (std::is_same<R, double>::value) {
            boys64<L>(T, args.tab64, F);
        } else if constexpr (is_df<R>) {
            boys_df<L>(T, reinterpret_cast<const float4 *>(args.tab32 + SQ_BOYS_DF_OFF), F);
        } else if constexpr (BOYS == BOYS_FP64) {
            boys_mixed<L>(T, tb, F);
        } else {
            boys32<L>(T, tb, F);
        }
        R fac = Uk * r;
        if constexpr (L == 0) {
            W[0][0][0][0] = fma(F[0], fac, W[0][0][0][0]);
        } else {
            R Fs[L + 1];
            const R m2a = R(-2) * alpha;
#pragma unroll
            for (int n = 0; n <= L; ++n) {
                Fs[n] = F[n] * fac;
                if (n < L) fac *= m2a;
            }
            R Rt[L + 1][L + 1][L + 1];
            hermite_r<L, R>(Fs, X, Y, Z, Rt);
            if constexpr (KET_S) {
#pragma unroll
                for (int t = 0; t <= LAB; ++t)
#pragma unroll
                    for (int u = 0; u <= LAB - t; ++u)
#pragma unroll
                        for (int v = 0; v <= LAB - t - u; ++v) W[t][u][v][0] += Rt[t][u][v];
            } else {
                const R *ek = hk + (long long)k * EK * sk;
#pragma unroll
                for (int c = 0; c < NC; ++c)
#pragma unroll
                    for (int d = 0; d < ND; ++d) {
                        const int cx = cart_x(LC, c) + cart_x(LD, d);
                        const int cy = cart_y(LC, c) + cart_y(LD, d);
                        const int cz = cart_z(LC, c) + cart_z(LD, d);
                        const int off = herm_offset(LC, LD, c, d);
#pragma unroll
                        for (int tau = 0; tau <= cx; ++tau)
#pragma unroll
                            for (int nu = 0; nu <= cy; ++nu)
#pragma unroll
                                for (int phi = 0; phi <= cz; ++phi) {
                                    R e = gload(ek + (long long)(off + (tau * (cy + 1) + nu) * (cz + 1) + phi) * sk);
                                    if ((tau + nu + phi) & 1) e = -e;
#pragma unroll
                                    for (int t = 0; t <= LAB; ++t)
#pragma unroll
                                        for (int u = 0; u <= LAB - t; ++u)
#pragma unroll
                                            for (int v = 0; v <= LAB - t - u; ++v)
                                                W[t][u][v][c * ND + d] =
                                                    fma(e, Rt[t + tau][u + nu][v + phi], W[t][u][v][c * ND + d]);
                                }
                    }
            }
        }
    }
}

template <int LA, int LB, int LC, int LD, typename R>
__device__ __forceinline__ void zero_w(R (&W)[LA + LB + 1][LA + LB + 1][LA + LB + 1][ncart(LC) * ncart(LD)]) {
    constexpr int LAB = LA + LB, NCD = ncart(LC) * ncart(LD);
#pragma unroll
    for (int t = 0; t <= LAB; ++t)
#pragma unroll
        for (int u = 0; u <= LAB - t; ++u)
#pragma unroll
            for (int v = 0; v <= LAB - t - u; ++v)
#pragma unroll
                for (int y = 0; y < NCD; ++y) W[t][u][v][y] = R(0);
}

// acc[ab][cd] += sum_tuv ub E^{ab}_{tuv}(i) W[tuv][cd] for bra primitive pair
// i (Hermite values at eb, stride sb), with the bra factor ub = 2 pi^{5/2} U_i.
template <int LA, int LB, int LC, int LD, typename R>
__device__ __forceinline__ void bra_transform(const R *eb, int sb, R ub,
                                              const R (&W)[LA + LB + 1][LA + LB + 1][LA + LB + 1][ncart(LC) * ncart(LD)],
                                              R (&acc)[ncart(LA) * ncart(LB)][ncart(LC) * ncart(LD)]) {
    constexpr int NA = ncart(LA), NB = ncart(LB), NCD = ncart(LC) * ncart(LD);
    if constexpr (LA + LB == 0) {
#pragma unroll
        for (int y = 0; y < NCD; ++y) acc[0][y] = fma(ub, W[0][0][0][y], acc[0][y]);
    } else {
#pragma unroll
        for (int a = 0; a < NA; ++a)
#pragma unroll
            for (int b = 0; b < NB; ++b) {
                const int ax = cart_x(LA, a) + cart_x(LB, b);
                const int ay = cart_y(LA, a) + cart_y(LB, b);
                const int az = cart_z(LA, a) + cart_z(LB, b);
                const int off = herm_offset(LA, LB, a, b);
#pragma unroll
                for (int t = 0; t <= ax; ++t)
#pragma unroll
                    for (int u = 0; u <= ay; ++u)
#pragma unroll
                        for (int v = 0; v <= az; ++v) {
                            const R e = ub * gload(eb + (long long)(off + (t * (ay + 1) + u) * (az + 1) + v) * sb);
#pragma unroll
                            for (int y = 0; y < NCD; ++y)
                                acc[a * NB + b][y] = fma(e, W[t][u][v][y], acc[a * NB + b][y]);
                        }
            }
    }
}

// acc += x for an FP32 partial sum x (FP64 or double-float accumulator).
__device__ __forceinline__ void add_f32(double &acc, float x) { acc += f2d_bits(x); }
__device__ __forceinline__ void add_f32(dfl &acc, float x) { acc = df_add(acc, x); }

// The same contraction of an FP32 W, each block element computed in FP32 and
// then added into the FP64 (or double-float) accumulator.
template <int LA, int LB, int LC, int LD, typename A>
__device__ __forceinline__ void bra_transform_f32_into(
    const float *eb, int sb, float ub, const float (&W)[LA + LB + 1][LA + LB + 1][LA + LB + 1][ncart(LC) * ncart(LD)],
    A (&acc)[ncart(LA) * ncart(LB)][ncart(LC) * ncart(LD)]) {
    constexpr int NA = ncart(LA), NB = ncart(LB), NCD = ncart(LC) * ncart(LD);
    if constexpr (LA + LB == 0) {
#pragma unroll
        for (int y = 0; y < NCD; ++y) add_f32(acc[0][y], ub * W[0][0][0][y]);
    } else {
#pragma unroll
        for (int a = 0; a < NA; ++a)
#pragma unroll
            for (int b = 0; b < NB; ++b) {
                const int ax = cart_x(LA, a) + cart_x(LB, b);
                const int ay = cart_y(LA, a) + cart_y(LB, b);
                const int az = cart_z(LA, a) + cart_z(LB, b);
                const int off = herm_offset(LA, LB, a, b);
                float part[NCD];
#pragma unroll
                for (int y = 0; y < NCD; ++y) part[y] = 0.0f;
#pragma unroll
                for (int t = 0; t <= ax; ++t)
#pragma unroll
                    for (int u = 0; u <= ay; ++u)
#pragma unroll
                        for (int v = 0; v <= az; ++v) {
                            const float e = ub * gload(eb + (long long)(off + (t * (ay + 1) + u) * (az + 1) + v) * sb);
#pragma unroll
                            for (int y = 0; y < NCD; ++y) part[y] = fmaf(e, W[t][u][v][y], part[y]);
                        }
#pragma unroll
                for (int y = 0; y < NCD; ++y) add_f32(acc[a * NB + b][y], part[y]);
            }
    }
}

// Contracted block of one quartet: acc[a*NB+b][c*ND+d].
//
// FP64 work per primitive quartet is what bounds these kernels on GB300, so:
// the bra factor 2 pi^{5/2} U_bra is applied once per bra primitive pair (in
// the bra transform), the Hermite coefficients of s-s pairs (exactly 1) are
// neither loaded nor multiplied, and (ss|ss) accumulates with a single FMA.
//
// SPLIT (FP64 and double-float launches): primitive-level precision.  Both slots keep
// their primitive pairs in descending primitive Schwarz factor q, so for bra
// primitive i the ket primitives with q_i q_k >= tau are a prefix [0, K_i),
// and K_i does not grow with i.  The prefix runs in FP64; the rest, whose
// primitive quartets are bounded by tau, runs in FP32 (FP64 Boys recursion,
// as in SQ_FP32 launches) and its FP32 block is added into the FP64 one.
template <int LA, int LB, int LC, int LD, typename R, int BOYS, bool SPLIT>
__device__ __forceinline__ void quartet_block(const EriArgs &args, const SlotDesc &bd, const SlotDesc &kd,
                                              const Boys32Blocks &tb,
                                              R (&acc)[ncart(LA) * ncart(LB)][ncart(LC) * ncart(LD)]) {
    static_assert(!SPLIT || std::is_same<R, double>::value || is_df<R>,
                  "primitive-level precision splits FP64 and double-float launches");
    constexpr int NAB = ncart(LA) * ncart(LB), NCD = ncart(LC) * ncart(LD);
    constexpr int LAB = LA + LB;
    constexpr int EB = herm_size(LA, LB);
    const sq_slots &sl = args.slots;
    const int nb = bd.npp, nk = kd.npp;
    const int pb = bd.pbase, sb = bd.pstride;
    const R *hb = slot_herm_ptr<R>(sl) + bd.hbase;

#pragma unroll
    for (int x = 0; x < NAB; ++x)
#pragma unroll
        for (int y = 0; y < NCD; ++y) acc[x][y] = R(0);

    int K = nk;  // FP64 ket prefix of the current bra primitive (SPLIT)
    for (int i = 0; i < nb; ++i) {
        const long long ib = pb + (long long)i * sb;
        const PrimPair<R> br = load_prim<R>(sl, ib);
        if constexpr (SPLIT) {
            if (args.prim_tau > 0.0f) {  // a zero bound keeps every primitive quartet in the accurate arithmetic
                const float thr = args.prim_tau / __ldg(sl.prim32v + 8 * ib + 5);
                while (K > 0 && __ldg(sl.prim32v + 8 * (kd.pbase + (long long)(K - 1) * kd.pstride) + 5) < thr) --K;
            }
        }
        if (!SPLIT || K > 0) {
            R W[LAB + 1][LAB + 1][LAB + 1][NCD];
            zero_w<LA, LB, LC, LD, R>(W);
            ket_loop<LA, LB, LC, LD, R, BOYS>(args, br.p, br.x, br.y, br.z, kd, 0, SPLIT ? K : nk, tb, W);
            bra_transform<LA, LB, LC, LD, R>(hb + (long long)i * EB * sb, sb, R(kTwoPi52) * br.u, W, acc);
        }
        if constexpr (SPLIT) {
            if (K < nk) {
                const float4 b4 = __ldg(reinterpret_cast<const float4 *>(sl.prim32v) + 2 * ib);
                const float ub = (float)kTwoPi52 * __ldg(sl.prim32v + 8 * ib + 4);
                float W32[LAB + 1][LAB + 1][LAB + 1][NCD];
                zero_w<LA, LB, LC, LD, float>(W32);
                ket_loop<LA, LB, LC, LD, float, BOYS_FP64>(args, b4.x, b4.y, b4.z, b4.w, kd, K, nk, tb, W32);
                bra_transform_f32_into<LA, LB, LC, LD, R>(sl.herm32 + bd.hbase + (long long)i * EB * sb, sb, ub, W32,
                                                          acc);
            }
        }
    }
}

// The six density blocks of one quartet (rows/columns of shells a, b, c, d).
template <int NA, int NB, int NC, int ND, typename R>
struct DensityBlocks {
    R ab[NA][NB], cd[NC][ND], ac[NA][NC], ad[NA][ND], bc[NB][NC], bd[NB][ND];
};

// Matrix element index of (row ra + i, column oc + j): ra = mb + oa*ld is
// the first row's offset of shell a in the molecule's block.  32-bit: the
// J/K entry points refuse matrices of 2^31 elements or more.
struct QuartetRows {
    int ra, rb, rc;      // row offsets of shells a, b, c
    int oa, ob, oc, od;  // first column of each shell
    int ld;
};

__device__ __forceinline__ QuartetRows quartet_rows(const sq_slots &sl, int P, const SlotDesc &bd, const SlotDesc &kd) {
    const int mb = sl.mbase ? (int)__ldg(sl.mbase + P) : 0;
    QuartetRows w;
    w.ld = bd.ld;
    w.oa = bd.oa;
    w.ob = bd.ob;
    w.oc = kd.oa;
    w.od = kd.ob;
    w.ra = mb + bd.oa * w.ld;
    w.rb = mb + bd.ob * w.ld;
    w.rc = mb + kd.oa * w.ld;
    return w;
}

template <int NA, int NB, int NC, int ND, typename R>
__device__ __forceinline__ void load_density(const R *D, const QuartetRows &w, DensityBlocks<NA, NB, NC, ND, R> &x) {
#pragma unroll
    for (int a = 0; a < NA; ++a)
#pragma unroll
        for (int b = 0; b < NB; ++b) x.ab[a][b] = gload(D + w.ra + a * w.ld + w.ob + b);
#pragma unroll
    for (int c = 0; c < NC; ++c)
#pragma unroll
        for (int d = 0; d < ND; ++d) x.cd[c][d] = gload(D + w.rc + c * w.ld + w.od + d);
#pragma unroll
    for (int a = 0; a < NA; ++a)
#pragma unroll
        for (int c = 0; c < NC; ++c) x.ac[a][c] = gload(D + w.ra + a * w.ld + w.oc + c);
#pragma unroll
    for (int a = 0; a < NA; ++a)
#pragma unroll
        for (int d = 0; d < ND; ++d) x.ad[a][d] = gload(D + w.ra + a * w.ld + w.od + d);
#pragma unroll
    for (int b = 0; b < NB; ++b)
#pragma unroll
        for (int c = 0; c < NC; ++c) x.bc[b][c] = gload(D + w.rb + b * w.ld + w.oc + c);
#pragma unroll
    for (int b = 0; b < NB; ++b)
#pragma unroll
        for (int d = 0; d < ND; ++d) x.bd[b][d] = gload(D + w.rb + b * w.ld + w.od + d);
}

// Digest one contracted block into Jacc/Kacc (one density):
//   Jacc[ab] += wJ sum_cd v D[cd],  Jacc[cd] += wJ sum_ab v D[ab],
//   Kacc[ac] += wK sum_bd v D[bd],  Kacc[bd] += wK v D[ac],  Kacc[ad] += wK v D[bc],  Kacc[bc] += wK v D[ad].
template <int NA, int NB, int NC, int ND, typename R>
__device__ __forceinline__ void digest_blocks(const R (&acc)[NA * NB][NC * ND], const R (&Dab)[NA][NB],
                                              const R (&Dcd)[NC][ND], const R (&Dac)[NA][NC], const R (&Dad)[NA][ND],
                                              const R (&Dbc)[NB][NC], const R (&Dbd)[NB][ND], const QuartetRows &w, R wJ,
                                              R wK, double *J, double *K) {
    R Jab[NA][NB], Jcd[NC][ND], Kac[NA][NC], Kad[NA][ND], Kbc[NB][NC], Kbd[NB][ND];
#pragma unroll
    for (int a = 0; a < NA; ++a)
#pragma unroll
        for (int b = 0; b < NB; ++b) Jab[a][b] = R(0);
#pragma unroll
    for (int c = 0; c < NC; ++c)
#pragma unroll
        for (int d = 0; d < ND; ++d) Jcd[c][d] = R(0);
#pragma unroll
    for (int a = 0; a < NA; ++a)
#pragma unroll
        for (int c = 0; c < NC; ++c) Kac[a][c] = R(0);
#pragma unroll
    for (int a = 0; a < NA; ++a)
#pragma unroll
        for (int d = 0; d < ND; ++d) Kad[a][d] = R(0);
#pragma unroll
    for (int b = 0; b < NB; ++b)
#pragma unroll
        for (int c = 0; c < NC; ++c) Kbc[b][c] = R(0);
#pragma unroll
    for (int b = 0; b < NB; ++b)
#pragma unroll
        for (int d = 0; d < ND; ++d) Kbd[b][d] = R(0);
#pragma unroll
    for (int a = 0; a < NA; ++a)
#pragma unroll
        for (int b = 0; b < NB; ++b)
#pragma unroll
            for (int c = 0; c < NC; ++c)
#pragma unroll
                for (int d = 0; d < ND; ++d) {
                    const R v = acc[a * NB + b][c * ND + d];
                    Jab[a][b] = fma(v, Dcd[c][d], Jab[a][b]);
                    Jcd[c][d] = fma(v, Dab[a][b], Jcd[c][d]);
                    Kac[a][c] = fma(v, Dbd[b][d], Kac[a][c]);
                    Kbd[b][d] = fma(v, Dac[a][c], Kbd[b][d]);
                    Kad[a][d] = fma(v, Dbc[b][c], Kad[a][d]);
                    Kbc[b][c] = fma(v, Dad[a][d], Kbc[b][c]);
                }
    auto to_d = [](R x) -> double {
        if constexpr (std::is_same<R, double>::value)
            return x;
        else if constexpr (is_df<R>)
            return df_to_double(x);
        else
            return f2d_bits(x);
    };
#pragma unroll
    for (int a = 0; a < NA; ++a)
#pragma unroll
        for (int b = 0; b < NB; ++b) atomicAdd(J + w.ra + a * w.ld + w.ob + b, to_d(wJ * Jab[a][b]));
#pragma unroll
    for (int c = 0; c < NC; ++c)
#pragma unroll
        for (int d = 0; d < ND; ++d) atomicAdd(J + w.rc + c * w.ld + w.od + d, to_d(wJ * Jcd[c][d]));
#pragma unroll
    for (int a = 0; a < NA; ++a)
#pragma unroll
        for (int c = 0; c < NC; ++c) atomicAdd(K + w.ra + a * w.ld + w.oc + c, to_d(wK * Kac[a][c]));
#pragma unroll
    for (int b = 0; b < NB; ++b)
#pragma unroll
        for (int d = 0; d < ND; ++d) atomicAdd(K + w.rb + b * w.ld + w.od + d, to_d(wK * Kbd[b][d]));
#pragma unroll
    for (int a = 0; a < NA; ++a)
#pragma unroll
        for (int d = 0; d < ND; ++d) atomicAdd(K + w.ra + a * w.ld + w.od + d, to_d(wK * Kad[a][d]));
#pragma unroll
    for (int b = 0; b < NB; ++b)
#pragma unroll
        for (int c = 0; c < NC; ++c) atomicAdd(K + w.rb + b * w.ld + w.oc + c, to_d(wK * Kbc[b][c]));
}

// Light classes: density blocks loaded before the primitive loops.
template <int NA, int NB, int NC, int ND, typename R>
__device__ __forceinline__ void digest(const R (&acc)[NA * NB][NC * ND], const DensityBlocks<NA, NB, NC, ND, R> &Dx,
                                       const QuartetRows &w, R wJ, R wK, double *J, double *K) {
    digest_blocks<NA, NB, NC, ND, R>(acc, Dx.ab, Dx.cd, Dx.ac, Dx.ad, Dx.bc, Dx.bd, w, wJ, wK, J, K);
}

// Heavy classes: density blocks loaded after the primitive loops.
template <int NA, int NB, int NC, int ND, typename R>
__device__ __forceinline__ void digest_loading(const R (&acc)[NA * NB][NC * ND], const R *D, const QuartetRows &w,
                                               R wJ, R wK, double *J, double *K) {
    DensityBlocks<NA, NB, NC, ND, R> Dx;
    load_density(D, w, Dx);
    digest<NA, NB, NC, ND, R>(acc, Dx, w, wJ, wK, J, K);
}

// Minimum resident blocks asked of ptxas: none for the light classes (their
// own register count, which keeps occupancy), one for L >= 5, whose blocks
// spill anyway: without it ptxas allocated only 32 registers to the FP64
// (dd|ds) kernel and spilled four times as much.
__host__ __device__ constexpr int kMinBlocks(int L) { return L >= 5 ? 1 : 0; }

// Per-thread J/K kernel: one contracted quartet (or sub-slot chunk) per
// thread, grid-stride over the class's quartet list.  Each quartet starts
// from its two slot descriptors.  For the light classes the whole
// descriptors and the six density blocks are loaded before the primitive
// loops, so that their latency hides behind the integral arithmetic; the
// heavy classes load the epilogue fields only after the loops.
template <int LA, int LB, int LC, int LD, typename R, int BOYS, int MODE, bool SPLIT = false>
__global__ void __launch_bounds__(128, kMinBlocks(LA + LB + LC + LD)) eri_class_kernel(const EriArgs args) {
    static_assert(MODE == MODE_JK, "per-thread kernels serve J/K launches only");
    constexpr int NA = ncart(LA), NB = ncart(LB), NC = ncart(LC), ND = ncart(LD);
    constexpr int NAB = NA * NB, NCD = NC * ND;
    constexpr int L = LA + LB + LC + LD;
    constexpr int NDENS = NAB + NCD + NA * NC + NA * ND + NB * NC + NB * ND;
    constexpr bool PREFETCH_D = NDENS <= 32;
    // FP32 launches (and the FP32 part of split FP64 launches) read the two
    // Boys Taylor blocks they need from shared memory (random rows: one smem
    // wavefront per 8 lanes instead of one L1 sector per lane).
    constexpr bool TAB32 = std::is_same<R, float>::value || SPLIT;
    __shared__ float4 s_tab[TAB32 ? 2 : 1][TAB32 ? SQ_BOYS_NGRID : 1];
    __shared__ float s_tab5[TAB32 ? 2 : 1][TAB32 ? SQ_BOYS_NGRID : 1];
    Boys32Blocks tb{nullptr, nullptr, nullptr, nullptr};
    if constexpr (TAB32) {
        const float4 *g = reinterpret_cast<const float4 *>(args.tab32 + SQ_BOYS_TAY32_OFF);
        const float *g5 = args.tab32 + SQ_BOYS_TAY32_5_OFF;
        const int blk0 = boys32_block<L>(0), blk1 = boys32_block<L>(1);
        for (int x = threadIdx.x; x < SQ_BOYS_NGRID; x += blockDim.x) {
            s_tab[0][x] = g[blk0 * SQ_BOYS_NGRID + x];
            s_tab[1][x] = g[blk1 * SQ_BOYS_NGRID + x];
            s_tab5[0][x] = g5[blk0 * SQ_BOYS_NGRID + x];
            s_tab5[1][x] = g5[blk1 * SQ_BOYS_NGRID + x];
        }
        __syncthreads();
        tb = Boys32Blocks{s_tab[0], s_tab[1], s_tab5[0], s_tab5[1]};
    }
    const int nd = args.nd > 1 ? args.nd : 1;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long qi = (long long)blockIdx.x * blockDim.x + threadIdx.x; qi < args.nq; qi += stride) {
        const int2 pq = args.quartets[qi];
        SlotDesc bd = PREFETCH_D ? load_desc(args.slots.desc, pq.x) : load_desc_prims(args.slots.desc, pq.x);
        SlotDesc kd = PREFETCH_D ? load_desc(args.slots.desc, pq.y) : load_desc_prims(args.slots.desc, pq.y);
        const R *D0;
        if constexpr (std::is_same<R, double>::value)
            D0 = args.D;
        else if constexpr (is_df<R>)
            D0 = reinterpret_cast<const dfl *>(args.Ddf);
        else
            D0 = args.D32;
        QuartetRows w;
        DensityBlocks<NA, NB, PREFETCH_D ? NC : 1, PREFETCH_D ? ND : 1, R> Dx;
        if constexpr (PREFETCH_D) {
            w = quartet_rows(args.slots, pq.x, bd, kd);
            load_density(D0, w, Dx);
        }

        R acc[NAB][NCD];
        quartet_block<LA, LB, LC, LD, R, BOYS, SPLIT>(args, bd, kd, tb, acc);
        if constexpr (!PREFETCH_D) {
            load_desc_epilogue(args.slots.desc, pq.x, bd);
            load_desc_epilogue(args.slots.desc, pq.y, kd);
            w = quartet_rows(args.slots, pq.x, bd, kd);
        }

        // Permutational weight m = 8 / 2^{[a==b] + [c==d] + [P==Q]}; J gets m/2, K gets m/4.
        float m = 8.0f;
        if ((bd.pairf >> 30) & 1) m *= 0.5f;
        if ((kd.pairf >> 30) & 1) m *= 0.5f;
        if (bd.pairf == kd.pairf) m *= 0.5f;  // sub-slots of a pair count as that pair
        const R wJ = R(0.5f * m), wK = R(0.25f * m);
        for (int di = 0; di < nd; ++di) {
            double *Jd = args.Jacc + di * args.dstride, *Kd = args.Kacc + di * args.dstride;
            if constexpr (PREFETCH_D) {
                if (di > 0) load_density(D0 + di * args.dstride, w, Dx);
                digest<NA, NB, NC, ND, R>(acc, Dx, w, wJ, wK, Jd, Kd);
            } else {
                digest_loading<NA, NB, NC, ND, R>(acc, D0 + di * args.dstride, w, wJ, wK, Jd, Kd);
            }
        }
    }
}

// Host-side launcher table entry for one quartet class.
typedef cudaError_t (*eri_launcher)(const EriArgs &args, int mode, int precision, cudaStream_t stream);

// Threads per block of a per-thread launch without an explicit shape: 128,
// or 64 / 32 when the list is too short to give every SM two blocks.  Each
// thread works through one whole quartet, so a short list of heavy quartets
// is bound by one thread's latency: spread over more SMs, its warps stop
// queueing for the same SM's FP64 (or FP32) pipe.
inline int default_threads(long long nq) {
    const long long want = 2LL * sm_count();
    for (int t = 128; t > 32; t >>= 1)
        if ((nq + t - 1) / t >= want) return t;
    return 32;
}

template <int LA, int LB, int LC, int LD>
cudaError_t launch_eri_class(const EriArgs &args, int mode, int precision, cudaStream_t stream) {
    if (args.nq <= 0) return cudaSuccess;
    const int threads = args.cfg_threads > 0 ? args.cfg_threads : default_threads(args.nq);
    long long blocks = (args.nq + threads - 1) / threads;
    // FP64: many blocks (FP64-bound, heavy-first order balances); FP32: about
    // two waves of persistent blocks so the shared Boys table is loaded rarely.
    const bool fp64 = precision == SQ_FP64 || precision == SQ_FP64_PRIM;
    const long long cap = args.cfg_threads > 0 ? args.cfg_blocks : (fp64 ? sm_count() * 16 * 8 : sm_count() * 16);
    if (blocks > cap) blocks = cap;
    (void)mode;  // per-thread kernels serve J/K launches only
    if (precision == SQ_FP64)
        eri_class_kernel<LA, LB, LC, LD, double, BOYS_FP64, MODE_JK><<<(int)blocks, threads, 0, stream>>>(args);
    else if (precision == SQ_FP64_PRIM)
        eri_class_kernel<LA, LB, LC, LD, double, BOYS_FP64, MODE_JK, true><<<(int)blocks, threads, 0, stream>>>(args);
    else if (precision == SQ_FP32)
        eri_class_kernel<LA, LB, LC, LD, float, BOYS_FP64, MODE_JK><<<(int)blocks, threads, 0, stream>>>(args);
    else
        eri_class_kernel<LA, LB, LC, LD, float, BOYS_FP32, MODE_JK><<<(int)blocks, threads, 0, stream>>>(args);
    return cudaGetLastError();
}

// FP64-only launcher (SQ_FP64) for a class whose FP32 variants have their own TU.
template <int LA, int LB, int LC, int LD>
cudaError_t launch_eri_class_f64(const EriArgs &args, int mode, int precision, cudaStream_t stream) {
    (void)mode;
    (void)precision;
    if (args.nq <= 0) return cudaSuccess;
    const int threads = args.cfg_threads > 0 ? args.cfg_threads : default_threads(args.nq);
    long long blocks = (args.nq + threads - 1) / threads;
    const long long cap = args.cfg_threads > 0 ? args.cfg_blocks : sm_count() * 16 * 8;
    if (blocks > cap) blocks = cap;
    eri_class_kernel<LA, LB, LC, LD, double, BOYS_FP64, MODE_JK><<<(int)blocks, threads, 0, stream>>>(args);
    return cudaGetLastError();
}

// Double-float launcher (SQ_DF64): every quartet of the list in double-float
// arithmetic on the FP32 pipe, with the primitive quartets below prim_tau in
// FP32 (prim_tau = 0: none) in the classes with L <= 4.  The heavier classes
// run whole in double-float: their d pairs have one primitive pair, so the
// split would move little, and without its FP32 branch the kernels compile in
// half the time.
template <int LA, int LB, int LC, int LD>
cudaError_t launch_eri_class_df(const EriArgs &args, int mode, int precision, cudaStream_t stream) {
    constexpr bool kSplit = LA + LB + LC + LD <= 4;
    (void)mode;
    (void)precision;
    if (args.nq <= 0) return cudaSuccess;
    const int threads = args.cfg_threads > 0 ? args.cfg_threads : default_threads(args.nq);
    long long blocks = (args.nq + threads - 1) / threads;
    const long long cap = args.cfg_threads > 0 ? args.cfg_blocks : sm_count() * 16 * 8;
    if (blocks > cap) blocks = cap;
    eri_class_kernel<LA, LB, LC, LD, dfl, BOYS_FP64, MODE_JK, kSplit><<<(int)blocks, threads, 0, stream>>>(args);
    return cudaGetLastError();
}

// FP32-only launcher (SQ_FP32) for the heavy classes whose full set of
// variants would take too long to compile.
template <int LA, int LB, int LC, int LD>
cudaError_t launch_eri_class_f32(const EriArgs &args, int mode, int precision, cudaStream_t stream) {
    (void)mode;
    (void)precision;
    if (args.nq <= 0) return cudaSuccess;
    const int threads = args.cfg_threads > 0 ? args.cfg_threads : default_threads(args.nq);
    long long blocks = (args.nq + threads - 1) / threads;
    const long long cap = args.cfg_threads > 0 ? args.cfg_blocks : sm_count() * 16;
    if (blocks > cap) blocks = cap;
    eri_class_kernel<LA, LB, LC, LD, float, BOYS_FP64, MODE_JK><<<(int)blocks, threads, 0, stream>>>(args);
    return cudaGetLastError();
}

}  // namespace sq
