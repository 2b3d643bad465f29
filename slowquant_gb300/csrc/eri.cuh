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
};

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
    else
        return sl.herm32;
}

template <typename R>
__device__ __forceinline__ R rsqrt_r(R x) {
    if constexpr (std::is_same<R, double>::value)
        return rsqrt(x);
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
    return __ldg(p);
}

// Contracted block of one quartet: acc[a*NB+b][c*ND+d].
//
// FP64 work per primitive quartet is what bounds these kernels on GB300, so:
// the bra factor 2 pi^{5/2} U_bra is applied once per bra primitive pair (in
// the bra transform), the Hermite coefficients of s-s pairs (exactly 1) are
// neither loaded nor multiplied, and (ss|ss) accumulates with a single FMA.
template <int LA, int LB, int LC, int LD, typename R, int BOYS>
__device__ __forceinline__ void quartet_block(const EriArgs &args, int P, int Q, const float4 *tb0,
                                              const float4 *tb1,
                                              R (&acc)[ncart(LA) * ncart(LB)][ncart(LC) * ncart(LD)]) {
    constexpr int NA = ncart(LA), NB = ncart(LB), NC = ncart(LC), ND = ncart(LD);
    constexpr int NAB = NA * NB, NCD = NC * ND;
    constexpr int LAB = LA + LB, LCD = LC + LD, L = LAB + LCD;
    constexpr int EB = herm_size(LA, LB), EK = herm_size(LC, LD);
    constexpr bool BRA_S = (LAB == 0), KET_S = (LCD == 0);

    // slot layout: field f of primitive pair i of slot s at prim[f*NPP + pbase[s] + i*pstride[s]]
    const sq_slots &sl = args.slots;
    const R *prim = slot_prim_ptr<R>(sl);
    const R *herm = slot_herm_ptr<R>(sl);
    const long long NPP = sl.npp_total;
    const int nb = gload(sl.npp + P), nk = gload(sl.npp + Q);
    const int pb = gload(sl.pbase + P), sb = gload(sl.pstride + P);
    const int pk = gload(sl.pbase + Q), sk = gload(sl.pstride + Q);
    const R *hb = herm + gload(sl.hbase + P);
    const R *hk = herm + gload(sl.hbase + Q);

#pragma unroll
    for (int x = 0; x < NAB; ++x)
#pragma unroll
        for (int y = 0; y < NCD; ++y) acc[x][y] = R(0);

    for (int i = 0; i < nb; ++i) {
        const long long ib = pb + (long long)i * sb;
        const R p = gload(prim + ib);
        const R Px = gload(prim + NPP + ib), Py = gload(prim + 2 * NPP + ib), Pz = gload(prim + 3 * NPP + ib);
        const R Ub = gload(prim + 4 * NPP + ib);
        R W[LAB + 1][LAB + 1][LAB + 1][NCD];
#pragma unroll
        for (int t = 0; t <= LAB; ++t)
#pragma unroll
            for (int u = 0; u <= LAB - t; ++u)
#pragma unroll
                for (int v = 0; v <= LAB - t - u; ++v)
#pragma unroll
                    for (int y = 0; y < NCD; ++y) W[t][u][v][y] = R(0);

        for (int k = 0; k < nk; ++k) {
            const long long ik = pk + (long long)k * sk;
            const R q = gload(prim + ik);
            const R X = Px - gload(prim + NPP + ik);
            const R Y = Py - gload(prim + 2 * NPP + ik);
            const R Z = Pz - gload(prim + 3 * NPP + ik);
            const R Uk = gload(prim + 4 * NPP + ik);
            const R r = rsqrt_r(p + q);
            const R alpha = p * q * (r * r);
            const R T = alpha * (X * X + Y * Y + Z * Z);
            R F[L + 1];
            if constexpr (std::is_same<R, double>::value) {
                boys64<L>(T, args.tab64, F);
            } else if constexpr (BOYS == BOYS_FP64) {
                boys_mixed<L>(T, tb0, tb1, F);
            } else {
                boys32<L>(T, tb0, tb1, F);
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
                    // W[tuv][cd] += sum_{tau nu phi} (-1)^{tau+nu+phi} E^{cd}_{tau nu phi} R[t+tau][u+nu][v+phi]
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
        // bra transform with the bra factor 2 pi^{5/2} U_bra
        const R ub = R(kTwoPi52) * Ub;
        if constexpr (BRA_S) {
#pragma unroll
            for (int y = 0; y < NCD; ++y) acc[0][y] = fma(ub, W[0][0][0][y], acc[0][y]);
        } else {
            const R *eb = hb + (long long)i * EB * sb;
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
}

template <int LA, int LB, int LC, int LD, typename R, int BOYS, int MODE>
__global__ void __launch_bounds__(128) eri_class_kernel(const EriArgs args) {
    constexpr int NA = ncart(LA), NB = ncart(LB), NC = ncart(LC), ND = ncart(LD);
    constexpr int NAB = NA * NB, NCD = NC * ND;
    constexpr int L = LA + LB + LC + LD;
    // FP32 launches read the two Boys Taylor blocks they need from shared memory
    // (random rows: one smem wavefront per 8 lanes instead of one L1 sector per lane).
    __shared__ float4 s_tab[std::is_same<R, float>::value ? 2 : 1][std::is_same<R, float>::value ? SQ_BOYS_NGRID : 1];
    const float4 *tb0 = nullptr, *tb1 = nullptr;
    if constexpr (std::is_same<R, float>::value) {
        const float4 *g = reinterpret_cast<const float4 *>(args.tab32 + SQ_BOYS_TAY32_OFF);
        const int blk0 = boys32_block<L>(0), blk1 = boys32_block<L>(1);
        for (int x = threadIdx.x; x < SQ_BOYS_NGRID; x += blockDim.x) {
            s_tab[0][x] = g[blk0 * SQ_BOYS_NGRID + x];
            s_tab[1][x] = g[blk1 * SQ_BOYS_NGRID + x];
        }
        __syncthreads();
        tb0 = s_tab[0];
        tb1 = s_tab[1];
    }
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long qi = (long long)blockIdx.x * blockDim.x + threadIdx.x; qi < args.nq; qi += stride) {
        const int2 pq = args.quartets[qi];
        const int P = pq.x, Q = pq.y;
        R acc[NAB][NCD];
        quartet_block<LA, LB, LC, LD, R, BOYS>(args, P, Q, tb0, tb1, acc);

        const int pairP = gload(args.slots.pair + P), pairQ = gload(args.slots.pair + Q);
        const int sa = gload(args.pairs.shells + 2 * pairP), sb = gload(args.pairs.shells + 2 * pairP + 1);
        const int sc = gload(args.pairs.shells + 2 * pairQ), sd = gload(args.pairs.shells + 2 * pairQ + 1);
        const int oa = gload(args.basis.bf_off + sa), ob = gload(args.basis.bf_off + sb);
        const int oc = gload(args.basis.bf_off + sc), od = gload(args.basis.bf_off + sd);
        const long long n = args.basis.nbf;

        if constexpr (MODE == MODE_SCHWARZ) {
            R mx = acc[0][0];
#pragma unroll
            for (int x = 0; x < NAB; ++x)
#pragma unroll
                for (int y = 0; y < NCD; ++y) mx = acc[x][y] > mx ? acc[x][y] : mx;
            args.q[P] = sqrt((double)mx);
        } else if constexpr (MODE == MODE_DENSE) {
            double *V = args.V;
#pragma unroll
            for (int a = 0; a < NA; ++a)
#pragma unroll
                for (int b = 0; b < NB; ++b)
#pragma unroll
                    for (int c = 0; c < NC; ++c)
#pragma unroll
                        for (int d = 0; d < ND; ++d) {
                            const double v = acc[a * NB + b][c * ND + d];
                            const long long A = oa + a, B = ob + b, C = oc + c, Dd = od + d;
                            V[((A * n + B) * n + C) * n + Dd] = v;
                            V[((B * n + A) * n + C) * n + Dd] = v;
                            V[((A * n + B) * n + Dd) * n + C] = v;
                            V[((B * n + A) * n + Dd) * n + C] = v;
                            V[((C * n + Dd) * n + A) * n + B] = v;
                            V[((Dd * n + C) * n + A) * n + B] = v;
                            V[((C * n + Dd) * n + B) * n + A] = v;
                            V[((Dd * n + C) * n + B) * n + A] = v;
                        }
        } else {
            // Permutational weight m = 8 / 2^{[a==b] + [c==d] + [P==Q]}; J gets m/2, K gets m/4.
            double m = 8.0;
            if (sa == sb) m *= 0.5;
            if (sc == sd) m *= 0.5;
            if (pairP == pairQ) m *= 0.5;  // sub-slots of a pair count as that pair
            const R wJ = R(0.5 * m), wK = R(0.25 * m);
            const int nd = args.nd > 1 ? args.nd : 1;
            for (int di = 0; di < nd; ++di) {
            const R *D;
            if constexpr (std::is_same<R, double>::value)
                D = args.D + di * args.dstride;
            else
                D = args.D32 + di * args.dstride;
            R Dab[NA][NB], Dcd[NC][ND], Dac[NA][NC], Dad[NA][ND], Dbc[NB][NC], Dbd[NB][ND];
            const sq_basis &bs = args.basis;
#pragma unroll
            for (int a = 0; a < NA; ++a)
#pragma unroll
                for (int b = 0; b < NB; ++b) Dab[a][b] = gload(D + mat_index(bs, sa, a, sb, b));
#pragma unroll
            for (int c = 0; c < NC; ++c)
#pragma unroll
                for (int d = 0; d < ND; ++d) Dcd[c][d] = gload(D + mat_index(bs, sc, c, sd, d));
#pragma unroll
            for (int a = 0; a < NA; ++a)
#pragma unroll
                for (int c = 0; c < NC; ++c) Dac[a][c] = gload(D + mat_index(bs, sa, a, sc, c));
#pragma unroll
            for (int a = 0; a < NA; ++a)
#pragma unroll
                for (int d = 0; d < ND; ++d) Dad[a][d] = gload(D + mat_index(bs, sa, a, sd, d));
#pragma unroll
            for (int b = 0; b < NB; ++b)
#pragma unroll
                for (int c = 0; c < NC; ++c) Dbc[b][c] = gload(D + mat_index(bs, sb, b, sc, c));
#pragma unroll
            for (int b = 0; b < NB; ++b)
#pragma unroll
                for (int d = 0; d < ND; ++d) Dbd[b][d] = gload(D + mat_index(bs, sb, b, sd, d));

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
            double *J = args.Jacc + di * args.dstride, *K = args.Kacc + di * args.dstride;
            auto to_d = [](R x) -> double {
                if constexpr (std::is_same<R, double>::value)
                    return x;
                else
                    return f2d_bits(x);
            };
#pragma unroll
            for (int a = 0; a < NA; ++a)
#pragma unroll
                for (int b = 0; b < NB; ++b) atomicAdd(J + mat_index(bs, sa, a, sb, b), to_d(wJ * Jab[a][b]));
#pragma unroll
            for (int c = 0; c < NC; ++c)
#pragma unroll
                for (int d = 0; d < ND; ++d) atomicAdd(J + mat_index(bs, sc, c, sd, d), to_d(wJ * Jcd[c][d]));
#pragma unroll
            for (int a = 0; a < NA; ++a)
#pragma unroll
                for (int c = 0; c < NC; ++c) atomicAdd(K + mat_index(bs, sa, a, sc, c), to_d(wK * Kac[a][c]));
#pragma unroll
            for (int b = 0; b < NB; ++b)
#pragma unroll
                for (int d = 0; d < ND; ++d) atomicAdd(K + mat_index(bs, sb, b, sd, d), to_d(wK * Kbd[b][d]));
#pragma unroll
            for (int a = 0; a < NA; ++a)
#pragma unroll
                for (int d = 0; d < ND; ++d) atomicAdd(K + mat_index(bs, sa, a, sd, d), to_d(wK * Kad[a][d]));
#pragma unroll
            for (int b = 0; b < NB; ++b)
#pragma unroll
                for (int c = 0; c < NC; ++c) atomicAdd(K + mat_index(bs, sb, b, sc, c), to_d(wK * Kbc[b][c]));
            }  // densities
        }
    }
}

// Host-side launcher table entry for one quartet class.
typedef cudaError_t (*eri_launcher)(const EriArgs &args, int mode, int precision, cudaStream_t stream);

template <int LA, int LB, int LC, int LD>
cudaError_t launch_eri_class(const EriArgs &args, int mode, int precision, cudaStream_t stream) {
    if (args.nq <= 0) return cudaSuccess;
    const int threads = args.cfg_threads > 0 ? args.cfg_threads : 128;
    long long blocks = (args.nq + threads - 1) / threads;
    // FP64: many blocks (FP64-bound, heavy-first order balances); FP32: about
    // two waves of persistent blocks so the shared Boys table is loaded rarely.
    const long long cap = args.cfg_threads > 0 ? args.cfg_blocks : (precision == SQ_FP64 ? sm_count() * 16 * 8 : sm_count() * 16);
    if (blocks > cap) blocks = cap;
    (void)mode;  // per-thread kernels serve J/K launches only
    if (precision == SQ_FP64)
        eri_class_kernel<LA, LB, LC, LD, double, BOYS_FP64, MODE_JK><<<(int)blocks, threads, 0, stream>>>(args);
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
    const int threads = args.cfg_threads > 0 ? args.cfg_threads : 128;
    long long blocks = (args.nq + threads - 1) / threads;
    const long long cap = args.cfg_threads > 0 ? args.cfg_blocks : sm_count() * 16 * 8;
    if (blocks > cap) blocks = cap;
    eri_class_kernel<LA, LB, LC, LD, double, BOYS_FP64, MODE_JK><<<(int)blocks, threads, 0, stream>>>(args);
    return cudaGetLastError();
}

// FP32-only launcher (SQ_FP32) for the heavy classes whose full set of
// variants would take too long to compile.
template <int LA, int LB, int LC, int LD>
cudaError_t launch_eri_class_f32(const EriArgs &args, int mode, int precision, cudaStream_t stream) {
    (void)mode;
    (void)precision;
    if (args.nq <= 0) return cudaSuccess;
    const int threads = args.cfg_threads > 0 ? args.cfg_threads : 128;
    long long blocks = (args.nq + threads - 1) / threads;
    const long long cap = args.cfg_threads > 0 ? args.cfg_blocks : sm_count() * 16;
    if (blocks > cap) blocks = cap;
    eri_class_kernel<LA, LB, LC, LD, float, BOYS_FP64, MODE_JK><<<(int)blocks, threads, 0, stream>>>(args);
    return cudaGetLastError();
}

}  // namespace sq
