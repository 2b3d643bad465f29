// grad.cu -- RHF nuclear gradient kernels (adjoint contraction on the fly).
//
// The reference has no gradients.  For converged D the RHF gradient is
//   dE/dR = sum D_ab dH_ab/dR - sum W_ab dS_ab/dR
//         + sum_{unique quartets} (m/2) sum_abcd Gamma'_abcd d(ab|cd)/dR + dV_nn/dR,
//   Gamma'_abcd = D_ab D_cd - (D_ac D_bd + D_ad D_bc)/4,  W = D F D / 2,
// with D = 2 C_occ C_occ^T (the reference's density).  Derivatives of a
// primitive Cartesian Gaussian: d/dA_x G(a) = 2 alpha G(a + 1_x) - a_x G(a - 1_x),
// so in McMurchie-Davidson form the bra overlap distribution's derivative has
// Hermite coefficients (2 alpha E^{a_x+1, b_x}_t - a_x E^{a_x-1, b_x}_t) E^{ab}_u E^{ab}_v
// and reaches t = a_x + b_x + 1; the Hermite Coulomb table is needed to L + 1.
//
// sq_grad_2e: one warp per quartet forms W'[tuv][cd] (ket transform, |tuv| <= L_ab+1),
// contracts it with Gamma' and the derivative coefficients of the bra centres,
// and runs a second time with bra and ket exchanged for the ket centres.  The
// light classes ((ss|ss), (ps|ss), (ps|ps), (pp|ss), (pp|ps), (ds|ss),
// (ds|ps), (dp|ss)) run the same contraction one quartet per thread
// (grad_thread.cu).
// Nothing is stored: each derivative integral is used once and dropped.
#include <cstdlib>

#include "boys.cuh"
#include "capi_internal.cuh"
#include "eri.cuh"

namespace sq {

constexpr int kGradL = SQ_MAX_L_GRAD;       // f
constexpr int kGradWarps = 4;               // warps per block where a class's slice fits four times
constexpr int kGHmax = nherm(4 * kGradL + 1);  // R to L + 1
constexpr int kGE = kGradL + 2;             // 1D tables with indices up to l + 1

// A warp's shared-memory slice, laid out per quartet class (offsets in doubles):
// two R buffers, W'[cd][h], Gamma'[ab][cd], the three 1D E tables, F_m.  Sizing
// it per class (instead of for (ff|ff)) lets the light classes keep many more
// warps resident; an (ff|ff) slice (186 KB) runs one warp per block.
struct GradLayout {
    int rbuf;    // entries per R buffer: nherm(L + 1)
    int W;       // offset of W'
    int G;       // offset of Gamma'
    int E;       // offset of the E tables [3][kGE][kGE][2 kGE - 1]
    int Fs;      // offset of F_m (16)
    int stride;  // doubles per warp (multiple of 2)
};
constexpr int kGEsize = 3 * kGE * kGE * (2 * kGE - 1);

// 1D expansion coefficients E^{ij}_t / E^{00}_0 (integralfunctions.py:9-71).
template <int NI, int NT>
__device__ inline void ecoef_table(double XPA, double XPB, double inv2p, int li, int lj, double (*E)[NI][NT]) {
    for (int i = 0; i <= li; ++i)
        for (int j = 0; j <= lj; ++j)
            for (int t = 0; t < NT; ++t) E[i][j][t] = 0.0;
    E[0][0][0] = 1.0;
    for (int i = 0; i <= li; ++i)
        for (int j = 0; j <= lj; ++j) {
            if (i == 0 && j == 0) continue;
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

// F_m(T) for any m <= 16: the Taylor grid while m + 6 <= 14, the high-order
// grid above (the top orders of (dd|dd) and of every f class; it is exact to
// T = 60, where the asymptote's neglected term for m = 13 is ~1e-13 relative,
// against ~6e-6 at T = 36).
__device__ inline double boys_any(int m, double T, const double *tab) {
    if (m + kBoysTaylor64 - 1 > SQ_BOYS_NCOL - 2) return boys_hi(m, T, tab);
    if (T >= SQ_BOYS_TMAX) {
        const double r = rsqrt(T);
        double f = kSqrtPiHalf * r;
        const double h = 0.5 * r * r;
        for (int j = 0; j < m; ++j) f *= (2 * j + 1) * h;
        return f;
    }
    const int kk = __double2int_rn(T * SQ_BOYS_STEP_INV);
    const double dd = T - kk * (1.0 / SQ_BOYS_STEP_INV);
    const double *row = tab + kk * SQ_BOYS_NCOL + m;
    double f = row[kBoysTaylor64 - 1];
    for (int j = kBoysTaylor64 - 1; j >= 1; --j) f = fma(f, -dd / j, row[j - 1]);
    return f;
}

cudaError_t launch_grad_thread_class(int qc, const EriArgs &a, int swap, double *grad, cudaStream_t s);
int grad_thread_enabled();

// Angular momenta of quartet class qc (bra pair class >= ket pair class).
inline void grad_class_l(int qc, int &la, int &lb, int &lc, int &ld) {
    int cb = 0;
    while ((cb + 1) * (cb + 2) / 2 <= qc) ++cb;
    const int ck = qc - cb * (cb + 1) / 2;
    la = 0;
    while ((la + 1) * (la + 2) / 2 <= cb) ++la;
    lb = cb - la * (la + 1) / 2;
    lc = 0;
    while ((lc + 1) * (lc + 2) / 2 <= ck) ++lc;
    ld = ck - lc * (lc + 1) / 2;
}

// Layout for a class in either orientation (the ket-centre pass swaps bra and ket).
inline GradLayout grad_layout(int la, int lb, int lc, int ld) {
    const int nab = ncart(la) * ncart(lb), ncd = ncart(lc) * ncart(ld);
    const int L1 = la + lb + lc + ld + 1;
    const int w1 = nherm(la + lb + 1) * ncd, w2 = nherm(lc + ld + 1) * nab;
    GradLayout g;
    g.rbuf = nherm(L1);
    g.W = 2 * g.rbuf;
    g.G = g.W + (w1 > w2 ? w1 : w2);
    g.E = g.G + nab * ncd;
    g.Fs = g.E + kGEsize;
    g.stride = (g.Fs + 16 + 1) / 2 * 2;
    return g;
}

__global__ void __launch_bounds__(32 * kGradWarps) grad2e_kernel(const EriArgs args, int swap, double *grad,
                                                                const GradLayout lay) {
    extern __shared__ __align__(16) double smem_d[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    double *wbase = smem_d + (long long)warp * lay.stride;
    double *rbuf0 = wbase, *rbuf1 = wbase + lay.rbuf;
    double *smW = wbase + lay.W, *smG = wbase + lay.G, *smFs = wbase + lay.Fs;
    double(*smE)[kGE][kGE][2 * kGE - 1] = reinterpret_cast<double(*)[kGE][kGE][2 * kGE - 1]>(wbase + lay.E);
    __shared__ int s_tuv[kGHmax];
    for (int e = threadIdx.x; e < kGHmax; e += blockDim.x) {
        int n = 0;
        while ((n + 1) * (n + 2) * (n + 3) / 6 <= e) ++n;
        int r = e - n * (n + 1) * (n + 2) / 6;
        int t = n;
        while (r >= n - t + 1) {
            r -= n - t + 1;
            --t;
        }
        const int u = n - t - r, v = n - t - u;
        s_tuv[e] = t | (u << 8) | (v << 16);
    }
    __syncthreads();

    const sq_pairs &pr = args.pairs;
    const sq_basis &bs = args.basis;
    const long long n = bs.nbf;
    const long long nwarps = (long long)gridDim.x * wpb;
    for (long long qi = (long long)blockIdx.x * wpb + warp; qi < args.nq; qi += nwarps) {
        const int2 pq = args.quartets[qi];
        const int slotP = swap ? pq.y : pq.x, slotQ = swap ? pq.x : pq.y;
        const int P = gload(args.slots.pair + slotP), Q = gload(args.slots.pair + slotQ);
        const int sa = gload(pr.shells + 2 * P), sb = gload(pr.shells + 2 * P + 1);
        const int sc = gload(pr.shells + 2 * Q), sd = gload(pr.shells + 2 * Q + 1);
        const int la = gload(bs.l + sa), lb = gload(bs.l + sb), lc = gload(bs.l + sc), ld = gload(bs.l + sd);
        const int NA = ncart(la), NB = ncart(lb), NC = ncart(lc), ND = ncart(ld);
        const int NAB = NA * NB, NCD = NC * ND;
        const int LAB = la + lb, L1 = LAB + lc + ld + 1, HAB1 = nherm(LAB + 1);
        const int EK = herm_offset_rt(lc, ld, NC, 0);
        const long long oa = gload(bs.bf_off + sa), ob = gload(bs.bf_off + sb);
        const long long oc = gload(bs.bf_off + sc), od = gload(bs.bf_off + sd);
        double m = 8.0;
        if (sa == sb) m *= 0.5;
        if (sc == sd) m *= 0.5;
        if (P == Q) m *= 0.5;
        const double *D = args.D;
        for (int x = lane; x < NAB * NCD; x += 32) {
            const int ab = x / NCD, cd = x - ab * NCD;
            const long long A = oa + ab / NB, B = ob + ab % NB, C = oc + cd / ND, Dd = od + cd % ND;
            smG[x] = 0.5 * m *
                      (gload(D + A * n + B) * gload(D + C * n + Dd) -
                       0.25 * (gload(D + A * n + C) * gload(D + B * n + Dd) + gload(D + A * n + Dd) * gload(D + B * n + C)));
        }
        const int i0 = gload(pr.pp_off + P), i1 = gload(pr.pp_off + P + 1);
        const int k0 = gload(pr.pp_off + Q), k1 = gload(pr.pp_off + Q + 1);
        const double *hk = pr.herm + gload(pr.herm_off + Q);
        const int npb = gload(bs.nprim + sb);
        const double *Ac = bs.center + 3 * sa, *Bc = bs.center + 3 * sb;
        double gacc[6] = {0, 0, 0, 0, 0, 0};
        __syncwarp();
        for (int i = i0; i < i1; ++i) {
            const int loc = i - i0;
            const double al = gload(bs.exps + gload(bs.prim_off + sa) + loc / npb);
            const double be = gload(bs.exps + gload(bs.prim_off + sb) + loc % npb);
            const double p = gload(pr.prim + 8 * i + 0);
            const double Pv[3] = {gload(pr.prim + 8 * i + 1), gload(pr.prim + 8 * i + 2), gload(pr.prim + 8 * i + 3)};
            const double Ub = gload(pr.prim + 8 * i + 4);
            if (lane < 3)
                ecoef_table<kGE, 2 * kGE - 1>(Pv[lane] - gload(Ac + lane), Pv[lane] - gload(Bc + lane), 0.5 / p, la + 1,
                                             lb + 1, smE[lane]);
            for (int w = lane; w < HAB1 * NCD; w += 32) smW[w] = 0.0;
            __syncwarp();
            for (int k = k0; k < k1; ++k) {
                const double q = gload(pr.prim + 8 * k + 0);
                const double X = Pv[0] - gload(pr.prim + 8 * k + 1);
                const double Y = Pv[1] - gload(pr.prim + 8 * k + 2);
                const double Z = Pv[2] - gload(pr.prim + 8 * k + 3);
                const double Uk = gload(pr.prim + 8 * k + 4);
                const double r = rsqrt(p + q);
                const double alpha = p * q * (r * r);
                const double T = alpha * (X * X + Y * Y + Z * Z);
                if (lane <= L1) {
                    double fac = kTwoPi52 * Ub * Uk * r;
                    for (int j = 0; j < lane; ++j) fac *= -2.0 * alpha;
                    smFs[lane] = fac * boys_any(lane, T, args.tab64);
                }
                __syncwarp();
                double *cur = rbuf0, *nxt = rbuf1;
                if (lane == 0) cur[0] = smFs[L1];
                __syncwarp();
                for (int lev = L1 - 1; lev >= 0; --lev) {
                    const int cnt = nherm(L1 - lev);
                    for (int e = lane; e < cnt; e += 32) {
                        double val;
                        if (e == 0) {
                            val = smFs[lev];
                        } else {
                            const int tuv = s_tuv[e];
                            const int t = tuv & 255, u = (tuv >> 8) & 255, v = tuv >> 16;
                            if (t > 0) {
                                val = X * cur[herm_index(t - 1, u, v)];
                                if (t > 1) val = fma((double)(t - 1), cur[herm_index(t - 2, u, v)], val);
                            } else if (u > 0) {
                                val = Y * cur[herm_index(0, u - 1, v)];
                                if (u > 1) val = fma((double)(u - 1), cur[herm_index(0, u - 2, v)], val);
                            } else {
                                val = Z * cur[herm_index(0, 0, v - 1)];
                                if (v > 1) val = fma((double)(v - 1), cur[herm_index(0, 0, v - 2)], val);
                            }
                        }
                        nxt[e] = val;
                    }
                    __syncwarp();
                    double *tmp = cur;
                    cur = nxt;
                    nxt = tmp;
                }
                // ket transform into W'[cd][h], |h| <= LAB + 1
                const double *ek = hk + (long long)(k - k0) * EK;
                for (int w = lane; w < HAB1 * NCD; w += 32) {
                    const int cd = w / HAB1, h = w - cd * HAB1;
                    const int tuv = s_tuv[h];
                    const int t = tuv & 255, u = (tuv >> 8) & 255, v = tuv >> 16;
                    int cx, cy, cz, dx, dy, dz;
                    cart_powers(lc, cd / ND, cx, cy, cz);
                    cart_powers(ld, cd % ND, dx, dy, dz);
                    cx += dx;
                    cy += dy;
                    cz += dz;
                    const double *e = ek + herm_offset_rt(lc, ld, cd / ND, cd % ND);
                    double s = 0.0;
                    for (int tau = 0; tau <= cx; ++tau)
                        for (int nu = 0; nu <= cy; ++nu)
                            for (int phi = 0; phi <= cz; ++phi) {
                                double ev = gload(e + (tau * (cy + 1) + nu) * (cz + 1) + phi);
                                if ((tau + nu + phi) & 1) ev = -ev;
                                s = fma(ev, cur[herm_index(t + tau, u + nu, v + phi)], s);
                            }
                    smW[w] += s;
                }
                __syncwarp();
            }
            // derivative contraction: lanes own bra component pairs ab
            for (int ab = lane; ab < NAB; ab += 32) {
                int ax, ay, az, bx, by, bz;
                cart_powers(la, ab / NB, ax, ay, az);
                cart_powers(lb, ab % NB, bx, by, bz);
                const double cn = 1.0 / sqrt(dfact_odd(ax) * dfact_odd(ay) * dfact_odd(az) * dfact_odd(bx) *
                                             dfact_odd(by) * dfact_odd(bz));
                // (U_bra, U_ket and 2 pi^{5/2} are already in Fs)
                const int tx = ax + bx, ty = ay + by, tz = az + bz;
                const int a3[3] = {ax, ay, az}, b3[3] = {bx, by, bz}, t3[3] = {tx, ty, tz};
                for (int t = 0; t <= tx + 1; ++t)
                    for (int u = 0; u <= ty + 1; ++u)
                        for (int v = 0; v <= tz + 1; ++v) {
                            const int raised = (t > tx) + (u > ty) + (v > tz);
                            if (raised > 1) continue;
                            const int h = herm_index(t, u, v);
                            double Yv = 0.0;
                            for (int cd = 0; cd < NCD; ++cd) Yv = fma(smW[cd * HAB1 + h], smG[ab * NCD + cd], Yv);
                            const int idx3[3] = {t, u, v};
                            for (int dir = 0; dir < 3; ++dir) {
                                // the other two directions must lie inside their unraised ranges
                                bool ok = true;
                                double other = 1.0;
                                for (int o = 0; o < 3; ++o) {
                                    if (o == dir) continue;
                                    if (idx3[o] > t3[o]) {
                                        ok = false;
                                        break;
                                    }
                                    other *= smE[o][a3[o]][b3[o]][idx3[o]];
                                }
                                if (!ok) continue;
                                const int td = idx3[dir];
                                const double (*Ed)[kGE][2 * kGE - 1] = smE[dir];
                                double dA = 2.0 * al * Ed[a3[dir] + 1][b3[dir]][td];
                                if (a3[dir] > 0 && td <= a3[dir] - 1 + b3[dir]) dA -= a3[dir] * Ed[a3[dir] - 1][b3[dir]][td];
                                double dB = 2.0 * be * Ed[a3[dir]][b3[dir] + 1][td];
                                if (b3[dir] > 0 && td <= a3[dir] + b3[dir] - 1) dB -= b3[dir] * Ed[a3[dir]][b3[dir] - 1][td];
                                const double f = cn * other * Yv;
                                gacc[dir] = fma(dA, f, gacc[dir]);
                                gacc[3 + dir] = fma(dB, f, gacc[3 + dir]);
                            }
                        }
            }
            __syncwarp();
        }
#pragma unroll
        for (int c = 0; c < 6; ++c)
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) gacc[c] += __shfl_xor_sync(0xffffffffu, gacc[c], off);
        if (lane == 0) {
            const int atA = gload(bs.shell_atom + sa), atB = gload(bs.shell_atom + sb);
            for (int c = 0; c < 3; ++c) {
                atomicAdd(grad + 3 * atA + c, gacc[c]);
                atomicAdd(grad + 3 * atB + c, gacc[3 + c]);
            }
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// One-electron derivatives, one thread per shell pair (s1 >= s2).
constexpr int kG1I = kGradL + 4;  // a + 1 + 2 for the kinetic operator
constexpr int kG1J = kGradL + 2;
constexpr int kG1R = nherm(2 * kGradL + 1);  // R^0_{tuv} to L = la + lb + 1

// R^0_{tuv}, t+u+v <= L (L <= 2 kGradL + 1), at herm_index(t, u, v).
__device__ inline void hermite_r_grad(int L, double p, const double *PC, const double *tab, double *out) {
    double F[2 * kGradL + 2];
    const double T = p * (PC[0] * PC[0] + PC[1] * PC[1] + PC[2] * PC[2]);
    for (int m = 0; m <= L; ++m) F[m] = boys_any(m, T, tab);
    double bufa[kG1R], bufb[kG1R];
    double *cur = bufa, *nxt = bufb;
#define RI(t, u, v) herm_index(t, u, v)
    double fac = 1.0;
    for (int m = 0; m <= L; ++m) {
        F[m] *= fac;
        fac *= -2.0 * p;
    }
    cur[0] = F[L];
    for (int lev = L - 1; lev >= 0; --lev) {
        const int top = L - lev;
        nxt[0] = F[lev];
        for (int t = 0; t <= top; ++t)
            for (int u = 0; u <= top - t; ++u)
                for (int v = 0; v <= top - t - u; ++v) {
                    if (t + u + v == 0) continue;
                    double val;
                    if (t > 0) {
                        val = PC[0] * cur[RI(t - 1, u, v)];
                        if (t > 1) val += (t - 1) * cur[RI(t - 2, u, v)];
                    } else if (u > 0) {
                        val = PC[1] * cur[RI(0, u - 1, v)];
                        if (u > 1) val += (u - 1) * cur[RI(0, u - 2, v)];
                    } else {
                        val = PC[2] * cur[RI(0, 0, v - 1)];
                        if (v > 1) val += (v - 1) * cur[RI(0, 0, v - 2)];
                    }
                    nxt[RI(t, u, v)] = val;
                }
        double *tmp = cur;
        cur = nxt;
        nxt = tmp;
    }
    for (int e = 0; e < nherm(L); ++e) out[e] = cur[e];
#undef RI
}

__device__ inline double comp_norm_g(int l, int c) {
    int x, y, z;
    cart_powers(l, c, x, y, z);
    return 1.0 / sqrt(dfact_odd(x) * dfact_odd(y) * dfact_odd(z));
}

// Kinetic integral of Cartesian powers a (on the first centre, exponent al) and b
// from 1D tables E[d][i][j][0] (kineticenergy.py:42-133), without the (pi/p)^{3/2} factor.
__device__ inline double kinetic_ab(const double (*E)[kG1I][kG1J][kG1I + kG1J], const int *a, const int *b, double al) {
    double e0[3], d2[3];
    for (int d = 0; d < 3; ++d) {
        e0[d] = E[d][a[d]][b[d]][0];
        d2[d] = 4 * al * al * E[d][a[d] + 2][b[d]][0] - 2 * al * (2 * a[d] + 1) * e0[d] +
                (a[d] >= 2 ? a[d] * (a[d] - 1) * E[d][a[d] - 2][b[d]][0] : 0.0);
    }
    return -0.5 * (d2[0] * e0[1] * e0[2] + e0[0] * d2[1] * e0[2] + e0[0] * e0[1] * d2[2]);
}

__device__ inline double hermite_sum(const double (*E)[kG1I][kG1J][kG1I + kG1J], const int *a, const int *b,
                                     const double *R) {
    double s = 0.0;
    for (int t = 0; t <= a[0] + b[0]; ++t)
        for (int u = 0; u <= a[1] + b[1]; ++u)
            for (int v = 0; v <= a[2] + b[2]; ++v)
                s += E[0][a[0]][b[0]][t] * E[1][a[1]][b[1]][u] * E[2][a[2]][b[2]][v] * R[herm_index(t, u, v)];
    return s;
}

__global__ void grad1e_kernel(const sq_basis basis, const double *tab, const double *Dm, const double *Wm,
                              double *grad) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const int ns = basis.nshell;
    if (idx >= ns * (ns + 1) / 2) return;
    int s1 = (int)((sqrt(8.0 * idx + 1.0) - 1.0) * 0.5);
    while ((s1 + 1) * (s1 + 2) / 2 <= idx) ++s1;
    while (s1 * (s1 + 1) / 2 > idx) --s1;
    const int s2 = idx - s1 * (s1 + 1) / 2;
    const int l1 = basis.l[s1], l2 = basis.l[s2];
    const int n1 = ncart(l1), n2 = ncart(l2);
    const int np1 = basis.nprim[s1], np2 = basis.nprim[s2];
    const double *A = basis.center + 3 * s1, *B = basis.center + 3 * s2;
    const int atA = basis.shell_atom[s1], atB = basis.shell_atom[s2];
    const long long n = basis.nbf;
    const int o1 = basis.bf_off[s1], o2 = basis.bf_off[s2];
    const double sym = (s1 == s2) ? 1.0 : 2.0;
    constexpr double pi = 3.141592653589793;
    double gA[3] = {0, 0, 0}, gB[3] = {0, 0, 0};
    double E[3][kG1I][kG1J][kG1I + kG1J];
    double R[kG1R];
    for (int i = 0; i < np1; ++i)
        for (int j = 0; j < np2; ++j) {
            const double al = basis.exps[basis.prim_off[s1] + i], be = basis.exps[basis.prim_off[s2] + j];
            const double cc = basis.coefs[basis.prim_off[s1] + i] * basis.coefs[basis.prim_off[s2] + j];
            const double p = al + be, mu = al * be / p;
            double Pc[3], AB2 = 0.0;
            for (int d = 0; d < 3; ++d) {
                Pc[d] = (al * A[d] + be * B[d]) / p;
                AB2 += (A[d] - B[d]) * (A[d] - B[d]);
            }
            const double K = exp(-mu * AB2);
            for (int d = 0; d < 3; ++d)
                ecoef_table<kG1J, kG1I + kG1J>(Pc[d] - A[d], Pc[d] - B[d], 0.5 / p, l1 + 3, l2 + 1, E[d]);
            const double ov = (pi / p) * sqrt(pi / p);
            // overlap and kinetic: d/dA, and d/dB = -d/dA (two-centre integrals)
            for (int x = 0; x < n1; ++x) {
                int a[3];
                cart_powers(l1, x, a[0], a[1], a[2]);
                for (int y = 0; y < n2; ++y) {
                    int b[3];
                    cart_powers(l2, y, b[0], b[1], b[2]);
                    const double w = sym * cc * K * comp_norm_g(l1, x) * comp_norm_g(l2, y);
                    const double Dv = Dm[(o1 + x) * n + o2 + y], Wv = Wm[(o1 + x) * n + o2 + y];
                    for (int d = 0; d < 3; ++d) {
                        int ap[3] = {a[0], a[1], a[2]};
                        ap[d] += 1;
                        double dS = 2 * al * E[0][ap[0]][b[0]][0] * E[1][ap[1]][b[1]][0] * E[2][ap[2]][b[2]][0];
                        double dT = 2 * al * kinetic_ab(E, ap, b, al);
                        if (a[d] > 0) {
                            int am[3] = {a[0], a[1], a[2]};
                            am[d] -= 1;
                            dS -= a[d] * E[0][am[0]][b[0]][0] * E[1][am[1]][b[1]][0] * E[2][am[2]][b[2]][0];
                            dT -= a[d] * kinetic_ab(E, am, b, al);
                        }
                        const double g = w * ov * (Dv * dT - Wv * dS);
                        gA[d] += g;
                        gB[d] -= g;
                    }
                }
            }
            // nuclear attraction: basis-function centres and the nucleus
            for (int at = 0; at < basis.natom; ++at) {
                double PC[3];
                for (int d = 0; d < 3; ++d) PC[d] = Pc[d] - basis.atom_xyz[3 * at + d];
                hermite_r_grad(l1 + l2 + 1, p, PC, tab, R);
                const double zf = -2.0 * pi / p * basis.atom_charge[at];
                double gC[3] = {0, 0, 0};
                for (int x = 0; x < n1; ++x) {
                    int a[3];
                    cart_powers(l1, x, a[0], a[1], a[2]);
                    for (int y = 0; y < n2; ++y) {
                        int b[3];
                        cart_powers(l2, y, b[0], b[1], b[2]);
                        const double w = sym * cc * K * comp_norm_g(l1, x) * comp_norm_g(l2, y) * zf *
                                         Dm[(o1 + x) * n + o2 + y];
                        for (int d = 0; d < 3; ++d) {
                            int ap[3] = {a[0], a[1], a[2]}, bp[3] = {b[0], b[1], b[2]};
                            ap[d] += 1;
                            bp[d] += 1;
                            double dA = 2 * al * hermite_sum(E, ap, b, R);
                            double dB = 2 * be * hermite_sum(E, a, bp, R);
                            if (a[d] > 0) {
                                int am[3] = {a[0], a[1], a[2]};
                                am[d] -= 1;
                                dA -= a[d] * hermite_sum(E, am, b, R);
                            }
                            if (b[d] > 0) {
                                int bm[3] = {b[0], b[1], b[2]};
                                bm[d] -= 1;
                                dB -= b[d] * hermite_sum(E, a, bm, R);
                            }
                            gA[d] += w * dA;
                            gB[d] += w * dB;
                            gC[d] -= w * (dA + dB);
                        }
                    }
                }
                for (int d = 0; d < 3; ++d) atomicAdd(grad + 3 * at + d, gC[d]);
            }
        }
    for (int d = 0; d < 3; ++d) {
        atomicAdd(grad + 3 * atA + d, gA[d]);
        atomicAdd(grad + 3 * atB + d, gB[d]);
    }
}

}  // namespace sq

using namespace sq;

extern "C" int sq_grad_2e(const sq_basis *basis, const sq_pairs *pairs, const sq_slots *slots,
                          const sq_quartets *quartets, const double *table64, const double *D, double *grad,
                          void *stream) {
    if (!basis || !pairs || !slots || !quartets || !table64 || !D || !grad || !basis->shell_atom)
        return set_error(SQ_ERR_ARG, "sq_grad_2e: NULL argument");
    if (basis->mat_base) return set_error(SQ_ERR_ARG, "sq_grad_2e: batched (packed) bases are not supported");
    if (quartets->nquartet == 0) return SQ_OK;
    for (int c = 0; c < SQ_MAX_QCLASS; ++c) {
        if (quartets->class_off[c + 1] <= quartets->class_off[c]) continue;
        int la, lb, lc, ld;
        grad_class_l(c, la, lb, lc, ld);
        if (la > SQ_MAX_L_GRAD || lb > SQ_MAX_L_GRAD || lc > SQ_MAX_L_GRAD || ld > SQ_MAX_L_GRAD)
            return set_error(SQ_ERR_UNSUPPORTED, "sq_grad_2e: class %d has l > %d (no gradient kernel)", c,
                             SQ_MAX_L_GRAD);
    }
    EriArgs a{};
    a.basis = *basis;
    a.pairs = *pairs;
    a.slots = *slots;
    a.use_slots = 1;
    a.tab64 = table64;
    a.D = D;
    a.quartets = reinterpret_cast<const int2 *>(quartets->pairs);
    a.nq = quartets->nquartet;
    // one launch per quartet class and orientation, each with its own shared-memory
    // layout; as many warps per block (up to four) as the opt-in shared memory holds
    int dev = 0, optin = 0;
    cudaFuncAttributes fa{};
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, grad2e_kernel);
    const long long avail = (long long)optin - (long long)fa.sharedSizeBytes;
    if (e == cudaSuccess) e = cudaFuncSetAttribute(grad2e_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)avail);
    if (e != cudaSuccess) return set_error(SQ_ERR_CUDA, "sq_grad_2e: %s", cudaGetErrorString(e));
    for (int c = 0; c < SQ_MAX_QCLASS; ++c) {
        const long long nq = quartets->class_off[c + 1] - quartets->class_off[c];
        if (nq <= 0) continue;
        int la, lb, lc, ld;
        grad_class_l(c, la, lb, lc, ld);
        const GradLayout lay = grad_layout(la, lb, lc, ld);
        a.quartets = reinterpret_cast<const int2 *>(quartets->pairs) + quartets->class_off[c];
        a.nq = nq;
        const long long slice = (long long)lay.stride * (long long)sizeof(double);
        long long wpb = avail / slice;
        if (wpb > kGradWarps) wpb = kGradWarps;
        if (wpb < 1)
            return set_error(SQ_ERR_UNSUPPORTED, "sq_grad_2e: class %d needs %lld bytes of shared memory per warp", c,
                             slice);
        const size_t sz = (size_t)(slice * wpb);
        long long blocks = (nq + wpb - 1) / wpb;
        if (blocks > sm_count() * 64) blocks = sm_count() * 64;
        for (int swap = 0; swap < 2; ++swap) {
            // light classes: one quartet per thread; the rest: one per warp
            if (grad_thread_enabled() &&
                launch_grad_thread_class(c, a, swap, grad, (cudaStream_t)stream) != cudaErrorNotSupported)
                continue;
            grad2e_kernel<<<(unsigned)blocks, (unsigned)(32 * wpb), sz, (cudaStream_t)stream>>>(a, swap, grad, lay);
        }
    }
    return check_launch("sq_grad_2e");
}

extern "C" int sq_grad_1e(const sq_basis *basis, const double *table64, const double *D, const double *W, double *grad,
                          void *stream) {
    if (!basis || !table64 || !D || !W || !grad || !basis->shell_atom)
        return set_error(SQ_ERR_ARG, "sq_grad_1e: NULL argument");
    if (basis->mat_base) return set_error(SQ_ERR_ARG, "sq_grad_1e: batched (packed) bases are not supported");
    const int np = basis->nshell * (basis->nshell + 1) / 2;
    if (np == 0) return SQ_OK;
    {
        // the kernel's E tables hold l <= SQ_MAX_L_GRAD: refuse other bases
        int *lh = (int *)malloc(sizeof(int) * basis->nshell);
        if (!lh) return set_error(SQ_ERR_ARG, "sq_grad_1e: host allocation failed");
        cudaError_t e = cudaMemcpyAsync(lh, basis->l, sizeof(int) * basis->nshell, cudaMemcpyDeviceToHost,
                                        (cudaStream_t)stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
        int lmax = 0;
        for (int s = 0; e == cudaSuccess && s < basis->nshell; ++s) lmax = lh[s] > lmax ? lh[s] : lmax;
        free(lh);
        if (e != cudaSuccess) return set_error(SQ_ERR_CUDA, "sq_grad_1e: %s", cudaGetErrorString(e));
        if (lmax > SQ_MAX_L_GRAD)
            return set_error(SQ_ERR_UNSUPPORTED, "sq_grad_1e: shell with l = %d > %d (no gradient kernel)", lmax,
                             SQ_MAX_L_GRAD);
    }
    grad1e_kernel<<<(np + 63) / 64, 64, 0, (cudaStream_t)stream>>>(*basis, table64, D, W, grad);
    return check_launch("sq_grad_1e");
}
