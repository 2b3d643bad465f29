// grad_thread.cu -- per-thread RHF gradient kernels for the light quartet classes.
//
// Same contraction as the warp kernel in grad.cu (Gamma' with the derivative
// integrals of the two bra centres, formed on the fly), one quartet per
// thread with compile-time sizes.  The warp kernel keeps only 1-4 of its 32
// lanes busy for s/p classes whose pairs have many primitives (an (ss|ss)
// quartet of 8-primitive s shells is 4096 primitive quartets), so these
// classes run here.  LA,LB is the bra of the launch's orientation: the ket
// centres' pass runs the swapped class.
#include "boys.cuh"
#include "capi_internal.cuh"
#include "eri.cuh"

namespace sq {

// E^{ij}_t / E^{00}_0 for i <= NI-1, j <= NJ-1 (integralfunctions.py:9-71), unrolled.
template <int NI, int NJ>
__device__ __forceinline__ void ecoef_ct(double XPA, double XPB, double inv2p, double (&E)[NI][NJ][NI + NJ - 1]) {
#pragma unroll
    for (int i = 0; i < NI; ++i)
#pragma unroll
        for (int j = 0; j < NJ; ++j)
#pragma unroll
            for (int t = 0; t < NI + NJ - 1; ++t) E[i][j][t] = 0.0;
    E[0][0][0] = 1.0;
#pragma unroll
    for (int i = 0; i < NI; ++i)
#pragma unroll
        for (int j = 0; j < NJ; ++j) {
            if (i == 0 && j == 0) continue;
#pragma unroll
            for (int t = 0; t <= i + j; ++t) {
                double v = 0.0;
                if (i == 0) {
                    if (t > 0) v += inv2p * E[0][j - 1][t - 1];
                    if (t <= i + j - 1) v += XPB * E[0][j - 1][t];
                    if (t + 1 <= i + j - 1) v += (t + 1) * E[0][j - 1][t + 1];
                } else {
                    if (t > 0) v += inv2p * E[i - 1][j][t - 1];
                    if (t <= i + j - 1) v += XPA * E[i - 1][j][t];
                    if (t + 1 <= i + j - 1) v += (t + 1) * E[i - 1][j][t + 1];
                }
                E[i][j][t] = v;
            }
        }
}

template <int LA, int LB, int LC, int LD>
__global__ void __launch_bounds__(128) grad2e_thread_kernel(const EriArgs args, int swap, double *grad) {
    constexpr int NA = ncart(LA), NB = ncart(LB), NC = ncart(LC), ND = ncart(LD);
    constexpr int NAB = NA * NB, NCD = NC * ND;
    constexpr int LAB = LA + LB, L1 = LAB + LC + LD + 1, H1 = LAB + 1;  // W' reaches |tuv| = LAB + 1
    constexpr int EK = herm_size(LC, LD);
    const sq_pairs &pr = args.pairs;
    const sq_basis &bs = args.basis;
    const long long n = bs.nbf;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long qi = (long long)blockIdx.x * blockDim.x + threadIdx.x; qi < args.nq; qi += stride) {
        const int2 pq = args.quartets[qi];
        const int slotP = swap ? pq.y : pq.x, slotQ = swap ? pq.x : pq.y;
        const int P = gload(args.slots.pair + slotP), Q = gload(args.slots.pair + slotQ);
        const int sa = gload(pr.shells + 2 * P), sb = gload(pr.shells + 2 * P + 1);
        const int sc = gload(pr.shells + 2 * Q), sd = gload(pr.shells + 2 * Q + 1);
        const long long oa = gload(bs.bf_off + sa), ob = gload(bs.bf_off + sb);
        const long long oc = gload(bs.bf_off + sc), od = gload(bs.bf_off + sd);
        double m = 8.0;
        if (sa == sb) m *= 0.5;
        if (sc == sd) m *= 0.5;
        if (P == Q) m *= 0.5;
        const double *D = args.D;
        double G[NAB][NCD];
#pragma unroll
        for (int ab = 0; ab < NAB; ++ab)
#pragma unroll
            for (int cd = 0; cd < NCD; ++cd) {
                const long long A = oa + ab / NB, B = ob + ab % NB, C = oc + cd / ND, Dd = od + cd % ND;
                G[ab][cd] = 0.5 * m *
                            (gload(D + A * n + B) * gload(D + C * n + Dd) -
                             0.25 * (gload(D + A * n + C) * gload(D + B * n + Dd) +
                                     gload(D + A * n + Dd) * gload(D + B * n + C)));
            }
        const int i0 = gload(pr.pp_off + P), i1 = gload(pr.pp_off + P + 1);
        const int k0 = gload(pr.pp_off + Q), k1 = gload(pr.pp_off + Q + 1);
        const double *hk = pr.herm + gload(pr.herm_off + Q);
        const int npb = gload(bs.nprim + sb);
        const int poa = gload(bs.prim_off + sa), pob = gload(bs.prim_off + sb);
        double Ac[3], Bc[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            Ac[d] = gload(bs.center + 3 * sa + d);
            Bc[d] = gload(bs.center + 3 * sb + d);
        }
        double gacc[6] = {0, 0, 0, 0, 0, 0};
        for (int i = i0; i < i1; ++i) {
            const int loc = i - i0;
            const double al = gload(bs.exps + poa + loc / npb);
            const double be = gload(bs.exps + pob + loc % npb);
            const double p = gload(pr.prim + 8 * i + 0);
            const double Pv[3] = {gload(pr.prim + 8 * i + 1), gload(pr.prim + 8 * i + 2), gload(pr.prim + 8 * i + 3)};
            const double Ub = gload(pr.prim + 8 * i + 4);
            double W[H1 + 1][H1 + 1][H1 + 1][NCD];
#pragma unroll
            for (int t = 0; t <= H1; ++t)
#pragma unroll
                for (int u = 0; u <= H1 - t; ++u)
#pragma unroll
                    for (int v = 0; v <= H1 - t - u; ++v)
#pragma unroll
                        for (int cd = 0; cd < NCD; ++cd) W[t][u][v][cd] = 0.0;
            for (int k = k0; k < k1; ++k) {
                const double q = gload(pr.prim + 8 * k + 0);
                const double X = Pv[0] - gload(pr.prim + 8 * k + 1);
                const double Y = Pv[1] - gload(pr.prim + 8 * k + 2);
                const double Z = Pv[2] - gload(pr.prim + 8 * k + 3);
                const double Uk = gload(pr.prim + 8 * k + 4);
                const double r = rsqrt(p + q);
                const double alpha = p * q * (r * r);
                const double T = alpha * (X * X + Y * Y + Z * Z);
                double F[L1 + 1];
                boys64<L1>(T, args.tab64, F);
                double Fs[L1 + 1];
                double fac = kTwoPi52 * Ub * Uk * r;
                const double m2a = -2.0 * alpha;
#pragma unroll
                for (int j = 0; j <= L1; ++j) {
                    Fs[j] = F[j] * fac;
                    fac *= m2a;
                }
                double Rt[L1 + 1][L1 + 1][L1 + 1];
                hermite_r<L1, double>(Fs, X, Y, Z, Rt);
                // ket transform into W'[tuv][cd], |tuv| <= LAB + 1
                const double *ek = hk + (long long)(k - k0) * EK;
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
                                    double e = gload(ek + off + (tau * (cy + 1) + nu) * (cz + 1) + phi);
                                    if ((tau + nu + phi) & 1) e = -e;
#pragma unroll
                                    for (int t = 0; t <= H1; ++t)
#pragma unroll
                                        for (int u = 0; u <= H1 - t; ++u)
#pragma unroll
                                            for (int v = 0; v <= H1 - t - u; ++v)
                                                W[t][u][v][c * ND + d] =
                                                    fma(e, Rt[t + tau][u + nu][v + phi], W[t][u][v][c * ND + d]);
                                }
                    }
            }
            // derivative contraction with Gamma' over the bra components
            double E[3][LA + 2][LB + 2][LA + LB + 3];
#pragma unroll
            for (int d = 0; d < 3; ++d) ecoef_ct<LA + 2, LB + 2>(Pv[d] - Ac[d], Pv[d] - Bc[d], 0.5 / p, E[d]);
#pragma unroll
            for (int a = 0; a < NA; ++a)
#pragma unroll
                for (int b = 0; b < NB; ++b) {
                    const int a3[3] = {cart_x(LA, a), cart_y(LA, a), cart_z(LA, a)};
                    const int b3[3] = {cart_x(LB, b), cart_y(LB, b), cart_z(LB, b)};
                    const double cn = 1.0 / sqrt(dfact_odd(a3[0]) * dfact_odd(a3[1]) * dfact_odd(a3[2]) *
                                                 dfact_odd(b3[0]) * dfact_odd(b3[1]) * dfact_odd(b3[2]));
                    const int ab = a * NB + b;
                    const int t3[3] = {a3[0] + b3[0], a3[1] + b3[1], a3[2] + b3[2]};
#pragma unroll
                    for (int t = 0; t <= LAB + 1; ++t)
#pragma unroll
                        for (int u = 0; u <= LAB + 1 - t; ++u)
#pragma unroll
                            for (int v = 0; v <= LAB + 1 - t - u; ++v) {
                                if (t > t3[0] + 1 || u > t3[1] + 1 || v > t3[2] + 1) continue;
                                const int raised = (t > t3[0]) + (u > t3[1]) + (v > t3[2]);
                                if (raised > 1) continue;
                                double Yv = 0.0;
#pragma unroll
                                for (int cd = 0; cd < NCD; ++cd) Yv = fma(W[t][u][v][cd], G[ab][cd], Yv);
                                const int idx3[3] = {t, u, v};
#pragma unroll
                                for (int dir = 0; dir < 3; ++dir) {
                                    bool ok = true;
                                    double other = 1.0;
#pragma unroll
                                    for (int o = 0; o < 3; ++o) {
                                        if (o == dir) continue;
                                        if (idx3[o] > t3[o]) ok = false;
                                        else other *= E[o][a3[o]][b3[o]][idx3[o]];
                                    }
                                    if (!ok) continue;
                                    const int td = idx3[dir];
                                    double dA = 2.0 * al * E[dir][a3[dir] + 1][b3[dir]][td];
                                    if (a3[dir] > 0 && td <= a3[dir] - 1 + b3[dir])
                                        dA -= a3[dir] * E[dir][a3[dir] - 1][b3[dir]][td];
                                    double dB = 2.0 * be * E[dir][a3[dir]][b3[dir] + 1][td];
                                    if (b3[dir] > 0 && td <= a3[dir] + b3[dir] - 1)
                                        dB -= b3[dir] * E[dir][a3[dir]][b3[dir] - 1][td];
                                    const double f = cn * other * Yv;
                                    gacc[dir] = fma(dA, f, gacc[dir]);
                                    gacc[3 + dir] = fma(dB, f, gacc[3 + dir]);
                                }
                            }
                }
        }
        const int atA = gload(bs.shell_atom + sa), atB = gload(bs.shell_atom + sb);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            atomicAdd(grad + 3 * atA + c, gacc[c]);
            atomicAdd(grad + 3 * atB + c, gacc[3 + c]);
        }
    }
}

template <int LA, int LB, int LC, int LD>
cudaError_t launch_grad_thread(const EriArgs &a, int swap, double *grad, cudaStream_t s) {
    if (a.nq <= 0) return cudaSuccess;
    long long blocks = (a.nq + 127) / 128;
    if (blocks > sm_count() * 16 * 8) blocks = sm_count() * 16 * 8;
    grad2e_thread_kernel<LA, LB, LC, LD><<<(unsigned)blocks, 128, 0, s>>>(a, swap, grad);
    return cudaGetLastError();
}

// Per-thread launch of quartet class qc in the given orientation (swap: the
// ket pair is the launch's bra); cudaErrorNotSupported if the class has no
// per-thread gradient kernel.
cudaError_t launch_grad_thread_class(int qc, const EriArgs &a, int swap, double *grad, cudaStream_t s) {
    switch (qc * 2 + swap) {
        case 0 * 2 + 0:
        case 0 * 2 + 1: return launch_grad_thread<0, 0, 0, 0>(a, swap, grad, s);  // (ss|ss)
        case 1 * 2 + 0: return launch_grad_thread<1, 0, 0, 0>(a, swap, grad, s);  // (ps|ss)
        case 1 * 2 + 1: return launch_grad_thread<0, 0, 1, 0>(a, swap, grad, s);
        case 2 * 2 + 0:
        case 2 * 2 + 1: return launch_grad_thread<1, 0, 1, 0>(a, swap, grad, s);  // (ps|ps)
        case 3 * 2 + 0: return launch_grad_thread<1, 1, 0, 0>(a, swap, grad, s);  // (pp|ss)
        case 3 * 2 + 1: return launch_grad_thread<0, 0, 1, 1>(a, swap, grad, s);
        case 4 * 2 + 0: return launch_grad_thread<1, 1, 1, 0>(a, swap, grad, s);  // (pp|ps)
        case 4 * 2 + 1: return launch_grad_thread<1, 0, 1, 1>(a, swap, grad, s);
        case 6 * 2 + 0: return launch_grad_thread<2, 0, 0, 0>(a, swap, grad, s);  // (ds|ss)
        case 6 * 2 + 1: return launch_grad_thread<0, 0, 2, 0>(a, swap, grad, s);
        case 7 * 2 + 0: return launch_grad_thread<2, 0, 1, 0>(a, swap, grad, s);  // (ds|ps)
        case 7 * 2 + 1: return launch_grad_thread<1, 0, 2, 0>(a, swap, grad, s);
        case 10 * 2 + 0: return launch_grad_thread<2, 1, 0, 0>(a, swap, grad, s);  // (dp|ss)
        case 10 * 2 + 1: return launch_grad_thread<0, 0, 2, 1>(a, swap, grad, s);
        default: return cudaErrorNotSupported;
    }
}

}  // namespace sq
