// prep.cu -- Boys grid, primitive-pair data, one-electron matrices and the
// small utility kernels (quartet-list expansion, Fock assembly).
#include <cstdio>

#include "boys.cuh"
#include "capi_internal.cuh"
#include "sq_common.cuh"

namespace sq {

// ---------------------------------------------------------------------------
// Boys grid: one thread per (grid point, order); compensated series sum.
// ngrid x ncol entries at out (last column exp(-T_k)); the FP32 copy is optional.
__global__ void boys_table_kernel(double *out, float *out32, int ngrid, int ncol) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= ngrid * ncol) return;
    const int k = idx / ncol, m = idx % ncol;
    const double T = k * (1.0 / SQ_BOYS_STEP_INV);
    double val;
    if (m == ncol - 1) {
        val = exp(-T);
    } else {
        // F_m(T) = e^{-T} sum_i (2T)^i / ((2m+1)(2m+3)...(2m+2i+1))
        double term = 1.0 / (2 * m + 1), sum = 0.0, comp = 0.0;
        for (int i = 0; i < 600; ++i) {
            const double y = term - comp;
            const double t = sum + y;
            comp = (t - sum) - y;
            sum = t;
            term *= (2.0 * T) / (2 * m + 2 * i + 3);
            if (term < 1e-18 * sum) break;
        }
        val = sum * exp(-T);
    }
    out[idx] = val;
    if (out32) out32[idx] = (float)val;
}

// Scaled Taylor blocks from the finished F grid: F_{m+j}(T_k)/j! (m < 15) and
// exp(-T_k)/j! (block 15).
__global__ void boys_taylor_kernel(double *tab64, float *tab32) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 16 * SQ_BOYS_NGRID * 8) return;
    const int j = idx & 7, mk = idx >> 3;
    const int m = mk / SQ_BOYS_NGRID, k = mk % SQ_BOYS_NGRID;
    double fact = 1.0;
    for (int t = 2; t <= j; ++t) fact *= t;
    double val = 0.0;
    if (j < kBoysTaylor64) {
        const int col = (m == 15) ? SQ_BOYS_NCOL - 1 : m + j;
        if (col < SQ_BOYS_NCOL) val = tab64[k * SQ_BOYS_NCOL + col] / fact;
        if (m != 15 && col >= SQ_BOYS_NCOL - 1) val = 0.0;
    }
    tab64[SQ_BOYS_TAY64_OFF + idx] = val;
    if (tab32 && j < 4) tab32[SQ_BOYS_TAY32_OFF + mk * 4 + j] = (float)val;
    if (tab32 && j == 4) tab32[SQ_BOYS_TAY32_5_OFF + mk] = (float)val;
    if (tab32) {
        // double-float row: c0..c3 as (hi, lo) pairs, c4..c6 as floats, one pad
        float *row = tab32 + SQ_BOYS_DF_OFF + (long long)mk * 12;
        const float h = (float)val;
        if (j < 4) {
            row[2 * j] = h;
            row[2 * j + 1] = (float)(val - (double)h);
        } else {
            row[4 + j] = j < kBoysTaylor64 ? h : 0.0f;
        }
    }
}

__global__ void boys_eval_kernel(int n_max, const double *z, long long nz, const double *tab, int mode,
                                 double *out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nz) return;
    double F[SQ_BOYS_HI_NCOL];
    if (mode == 1) {
        for (int m = 0; m <= n_max; ++m) F[m] = boys_reference(m, z[i]);
    } else if (mode == 2) {
        for (int m = 0; m <= n_max; ++m) F[m] = boys_hi(m, z[i], tab);
    } else {
        boys64_rt(n_max, z[i], tab, F);
    }
    for (int m = 0; m <= n_max; ++m) out[i * (n_max + 1) + m] = F[m];
}

// Double-float Boys (the df64 J/K kernels' boys_df) at FP64 arguments, for the test hook.
template <int M>
__global__ void boys_df_eval_kernel(const double *z, long long nz, const float4 *tab, double *out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nz) return;
    const double v = z[i];
    const float h = (float)v;
    dfl F[M + 1];
    boys_df<M>(dfl(h, (float)(v - (double)h)), tab, F);
    for (int m = 0; m <= M; ++m) out[i * (M + 1) + m] = (double)F[m].hi + (double)F[m].lo;
}

template <int M>
static void launch_boys_df(const double *z, long long nz, const float *table32, double *out, cudaStream_t s) {
    boys_df_eval_kernel<M><<<(unsigned)((nz + 127) / 128), 128, 0, s>>>(
        z, nz, reinterpret_cast<const float4 *>(table32 + SQ_BOYS_DF_OFF), out);
}

// ---------------------------------------------------------------------------
// Primitive-pair data.  One thread per primitive pair.
// 1D MD expansion coefficients E^{ij}_t / E^{00}_0 per Cartesian direction
// (integralfunctions.py:9-71; the common factor exp(-mu X_AB^2) of all three
// directions is kept in U).
constexpr int kEMax = 4;  // supports l <= 3 per shell
__device__ inline void ecoef_1d(double XPA, double XPB, double inv2p, int la, int lb,
                                double (&E)[kEMax][kEMax][2 * kEMax - 1]) {
    for (int i = 0; i <= la; ++i)
        for (int j = 0; j <= lb; ++j)
            for (int t = 0; t <= la + lb; ++t) E[i][j][t] = 0.0;
    E[0][0][0] = 1.0;
    for (int i = 0; i <= la; ++i)
        for (int j = 0; j <= lb; ++j) {
            if (i == 0 && j == 0) continue;
            for (int t = 0; t <= i + j; ++t) {
                double v = 0.0;
                if (i == 0) {  // increment j
                    if (t > 0) v += inv2p * E[0][j - 1][t - 1];
                    if (t <= i + j - 1) v += XPB * E[0][j - 1][t];
                    if (t + 1 <= i + j - 1) v += (t + 1) * E[0][j - 1][t + 1];
                } else {  // increment i
                    if (t > 0) v += inv2p * E[i - 1][j][t - 1];
                    if (t <= i + j - 1) v += XPA * E[i - 1][j][t];
                    if (t + 1 <= i + j - 1) v += (t + 1) * E[i - 1][j][t + 1];
                }
                E[i][j][t] = v;
            }
        }
}

__device__ inline double comp_norm(int l, int c) {
    return 1.0 / sqrt(dfact_odd(cart_x(l, c)) * dfact_odd(cart_y(l, c)) * dfact_odd(cart_z(l, c)));
}

__global__ void pair_prep_kernel(const sq_basis basis, sq_pairs pairs) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= pairs.nprimpair) return;
    // pair owning this primitive pair: largest P with pp_off[P] <= idx
    int lo = 0, hi = pairs.npair - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pairs.pp_off[mid] <= idx) lo = mid;
        else hi = mid - 1;
    }
    const int P = lo;
    const int a = pairs.shells[2 * P], b = pairs.shells[2 * P + 1];
    const int la = basis.l[a], lb = basis.l[b];
    const int local = idx - pairs.pp_off[P];
    const int nbp = basis.nprim[b];
    const int ia = local / nbp, ib = local % nbp;
    const double al = basis.exps[basis.prim_off[a] + ia], be = basis.exps[basis.prim_off[b] + ib];
    const double ca = basis.coefs[basis.prim_off[a] + ia], cb = basis.coefs[basis.prim_off[b] + ib];
    const double *A = basis.center + 3 * a, *B = basis.center + 3 * b;
    const double p = al + be, mu = al * be / p;
    double Pc[3], AB2 = 0.0;
    for (int d = 0; d < 3; ++d) {
        Pc[d] = (al * A[d] + be * B[d]) / p;
        AB2 += (A[d] - B[d]) * (A[d] - B[d]);
    }
    const double U = ca * cb * exp(-mu * AB2) / p;
    double *pd = pairs.prim + 8 * (long long)idx;
    pd[0] = p;
    pd[1] = Pc[0];
    pd[2] = Pc[1];
    pd[3] = Pc[2];
    pd[4] = U;
    pd[5] = pd[6] = pd[7] = 0.0;
    if (pairs.prim32) {
        float *pf = pairs.prim32 + 8 * (long long)idx;
        for (int x = 0; x < 8; ++x) pf[x] = (float)pd[x];
    }
    double E[3][kEMax][kEMax][2 * kEMax - 1];
    for (int d = 0; d < 3; ++d) ecoef_1d(Pc[d] - A[d], Pc[d] - B[d], 0.5 / p, la, lb, E[d]);
    const int na = ncart(la), nb = ncart(lb);
    int esize = 0;
    for (int x = 0; x < na; ++x)
        for (int y = 0; y < nb; ++y) esize += herm_terms(la, x, lb, y);
    const long long base = pairs.herm_off[P] + (long long)local * esize;
    long long o = base;
    for (int x = 0; x < na; ++x) {
        const int ax = cart_x(la, x), ay = cart_y(la, x), az = cart_z(la, x);
        const double sa = comp_norm(la, x);
        for (int y = 0; y < nb; ++y) {
            const int bx = cart_x(lb, y), by = cart_y(lb, y), bz = cart_z(lb, y);
            const double s = sa * comp_norm(lb, y);
            for (int t = 0; t <= ax + bx; ++t)
                for (int u = 0; u <= ay + by; ++u)
                    for (int v = 0; v <= az + bz; ++v) {
                        const double e = s * E[0][ax][bx][t] * E[1][ay][by][u] * E[2][az][bz][v];
                        pairs.herm[o] = e;
                        if (pairs.herm32) pairs.herm32[o] = (float)e;
                        ++o;
                    }
        }
    }
}

// ---------------------------------------------------------------------------
// One-electron matrices; one thread per shell pair (s1 >= s2).
constexpr int kE1 = 6;  // l+2 <= 5 (f shells + 2)

__device__ inline void ecoef_1d_big(double XPA, double XPB, double inv2p, int la, int lb,
                                    double (&E)[kE1][kE1][2 * kE1 - 1]) {
    for (int i = 0; i <= la; ++i)
        for (int j = 0; j <= lb; ++j)
            for (int t = 0; t <= la + lb; ++t) E[i][j][t] = 0.0;
    E[0][0][0] = 1.0;
    for (int i = 0; i <= la; ++i)
        for (int j = 0; j <= lb; ++j) {
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

// R^0_{tuv}, t+u+v <= L (L <= 6), flat index ((t*7)+u)*7+v.
__device__ inline void hermite_r_rt(int L, double p, const double *PC, const double *tab, double *out) {
    double F[SQ_BOYS_NCOL];
    const double T = p * (PC[0] * PC[0] + PC[1] * PC[1] + PC[2] * PC[2]);
    boys64_rt(L, T, tab, F);
    double cur[343], nxt[343];
#define RI(t, u, v) (((t) * 7 + (u)) * 7 + (v))
    double fac = 1.0;
    for (int n = 0; n <= L; ++n) {
        F[n] *= fac;
        fac *= -2.0 * p;
    }
    cur[0] = F[L];
    for (int n = L - 1; n >= 0; --n) {
        const int top = L - n;
        nxt[0] = F[n];
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
        for (int t = 0; t <= top; ++t)
            for (int u = 0; u <= top - t; ++u)
                for (int v = 0; v <= top - t - u; ++v) cur[RI(t, u, v)] = nxt[RI(t, u, v)];
    }
    for (int t = 0; t <= L; ++t)
        for (int u = 0; u <= L - t; ++u)
            for (int v = 0; v <= L - t - u; ++v) out[RI(t, u, v)] = cur[RI(t, u, v)];
#undef RI
}

__global__ void one_electron_kernel(const sq_basis basis, const double *tab, double *S, double *Tm, double *Vm) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const int ns = basis.nshell;
    if (idx >= ns * (ns + 1) / 2) return;
    // idx -> (s1, s2), s1 >= s2
    int s1 = (int)((sqrt(8.0 * idx + 1.0) - 1.0) * 0.5);
    while ((s1 + 1) * (s1 + 2) / 2 <= idx) ++s1;
    while (s1 * (s1 + 1) / 2 > idx) --s1;
    const int s2 = idx - s1 * (s1 + 1) / 2;
    // batch: shells of different molecules have no matrix element
    if (basis.mat_base != nullptr && basis.mat_base[s1] != basis.mat_base[s2]) return;
    const int l1 = basis.l[s1], l2 = basis.l[s2];
    const int n1 = ncart(l1), n2 = ncart(l2);
    const int np1 = basis.nprim[s1], np2 = basis.nprim[s2];
    const double *A = basis.center + 3 * s1, *B = basis.center + 3 * s2;
    double sblk[100], tblk[100], vblk[100];
    for (int x = 0; x < n1 * n2; ++x) sblk[x] = tblk[x] = vblk[x] = 0.0;
    double E[3][kE1][kE1][2 * kE1 - 1];
    double R[343];
    constexpr double pi = 3.141592653589793;
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
            for (int d = 0; d < 3; ++d) ecoef_1d_big(Pc[d] - A[d], Pc[d] - B[d], 0.5 / p, l1 + 2, l2, E[d]);
            const double sp = pi / p;
            const double ov = sp * sqrt(sp);
            for (int x = 0; x < n1; ++x) {
                const int a[3] = {cart_x(l1, x), cart_y(l1, x), cart_z(l1, x)};
                const double na = comp_norm(l1, x);
                for (int y = 0; y < n2; ++y) {
                    const int b[3] = {cart_x(l2, y), cart_y(l2, y), cart_z(l2, y)};
                    const double w = cc * K * na * comp_norm(l2, y);
                    double e0[3], d2[3];
                    for (int d = 0; d < 3; ++d) {
                        e0[d] = E[d][a[d]][b[d]][0];
                        d2[d] = 4 * al * al * E[d][a[d] + 2][b[d]][0] - 2 * al * (2 * a[d] + 1) * e0[d] +
                                (a[d] >= 2 ? a[d] * (a[d] - 1) * E[d][a[d] - 2][b[d]][0] : 0.0);
                    }
                    sblk[x * n2 + y] += w * ov * e0[0] * e0[1] * e0[2];
                    tblk[x * n2 + y] += w * (-0.5 * ov) *
                                        (d2[0] * e0[1] * e0[2] + e0[0] * d2[1] * e0[2] + e0[0] * e0[1] * d2[2]);
                }
            }
            if (Vm) {
                const int L = l1 + l2;
                const int at0 = basis.atom_begin ? basis.atom_begin[s1] : 0;
                const int at1 = basis.atom_end ? basis.atom_end[s1] : basis.natom;
                for (int at = at0; at < at1; ++at) {
                    double PC[3];
                    for (int d = 0; d < 3; ++d) PC[d] = Pc[d] - basis.atom_xyz[3 * at + d];
                    hermite_r_rt(L, p, PC, tab, R);
                    const double zf = -2.0 * pi / p * basis.atom_charge[at];
                    for (int x = 0; x < n1; ++x) {
                        const int a[3] = {cart_x(l1, x), cart_y(l1, x), cart_z(l1, x)};
                        const double na = comp_norm(l1, x);
                        for (int y = 0; y < n2; ++y) {
                            const int b[3] = {cart_x(l2, y), cart_y(l2, y), cart_z(l2, y)};
                            double acc = 0.0;
                            for (int t = 0; t <= a[0] + b[0]; ++t)
                                for (int u = 0; u <= a[1] + b[1]; ++u)
                                    for (int v = 0; v <= a[2] + b[2]; ++v)
                                        acc += E[0][a[0]][b[0]][t] * E[1][a[1]][b[1]][u] * E[2][a[2]][b[2]][v] *
                                               R[(t * 7 + u) * 7 + v];
                            vblk[x * n2 + y] += cc * K * na * comp_norm(l2, y) * zf * acc;
                        }
                    }
                }
            }
        }
    for (int x = 0; x < n1; ++x)
        for (int y = 0; y < n2; ++y) {
            const long long rc = mat_index(basis, s1, x, s2, y), cr = mat_index(basis, s2, y, s1, x);
            if (S) S[rc] = S[cr] = sblk[x * n2 + y];
            if (Tm) Tm[rc] = Tm[cr] = tblk[x * n2 + y];
            if (Vm) Vm[rc] = Vm[cr] = vblk[x * n2 + y];
        }
}

// Multipole integrals <a| (x-Cx)^ex (y-Cy)^ey (z-Cz)^ez |b> over contracted
// Cartesian shells (slowquant/molecularintegrals/multipole.py:48-135): per
// primitive pair and dimension, the Hermite multipole integrals of
// integralfunctions.py:151-183,
//   M^0_0 = sqrt(pi/p),  M^{e+1}_t = t M^e_{t-1} + X_PC M^e_t + M^e_{t+1} / (2p),
// contracted with the expansion coefficients: S = prod_d sum_{t <= min(a_d+b_d, e_d)} E^{ab}_t M^{e_d}_t.
// One shell pair per thread, both triangles written (the matrix is symmetric).
constexpr int kMultipoleMax = 16;  // highest order per Cartesian direction

__global__ void multipole_kernel(const sq_basis basis, int ex, int ey, int ez, double cx, double cy, double cz,
                                 double *M) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const int ns = basis.nshell;
    if (idx >= ns * (ns + 1) / 2) return;
    int s1 = (int)((sqrt(8.0 * idx + 1.0) - 1.0) * 0.5);
    while ((s1 + 1) * (s1 + 2) / 2 <= idx) ++s1;
    while (s1 * (s1 + 1) / 2 > idx) --s1;
    const int s2 = idx - s1 * (s1 + 1) / 2;
    if (basis.mat_base != nullptr && basis.mat_base[s1] != basis.mat_base[s2]) return;
    const int l1 = basis.l[s1], l2 = basis.l[s2];
    const int n1 = ncart(l1), n2 = ncart(l2);
    const int np1 = basis.nprim[s1], np2 = basis.nprim[s2];
    const double *A = basis.center + 3 * s1, *B = basis.center + 3 * s2;
    const double C[3] = {cx, cy, cz};
    const int eo[3] = {ex, ey, ez};
    double blk[100];
    for (int x = 0; x < n1 * n2; ++x) blk[x] = 0.0;
    double E[3][kE1][kE1][2 * kE1 - 1];
    double Mh[3][kMultipoleMax + 1];  // M^{e_d}_t, t <= e_d, of each direction
    double row[kMultipoleMax + 1], nxt[kMultipoleMax + 1];
    constexpr double pi = 3.141592653589793;
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
            for (int d = 0; d < 3; ++d) {
                ecoef_1d_big(Pc[d] - A[d], Pc[d] - B[d], 0.5 / p, l1, l2, E[d]);
                const double X = Pc[d] - C[d];
                for (int t = 0; t <= eo[d]; ++t) row[t] = 0.0;
                row[0] = sqrt(pi / p);
                for (int e = 0; e < eo[d]; ++e) {  // row holds M^e_t; build M^{e+1}_t
                    for (int t = 0; t <= e + 1; ++t) {
                        double v = X * (t <= e ? row[t] : 0.0);
                        if (t > 0) v += t * row[t - 1];
                        if (t + 1 <= e) v += (0.5 / p) * row[t + 1];
                        nxt[t] = v;
                    }
                    for (int t = 0; t <= e + 1; ++t) row[t] = nxt[t];
                }
                for (int t = 0; t <= eo[d]; ++t) Mh[d][t] = row[t];
            }
            for (int x = 0; x < n1; ++x) {
                const int a[3] = {cart_x(l1, x), cart_y(l1, x), cart_z(l1, x)};
                const double na = comp_norm(l1, x);
                for (int y = 0; y < n2; ++y) {
                    const int b[3] = {cart_x(l2, y), cart_y(l2, y), cart_z(l2, y)};
                    double prod = cc * K * na * comp_norm(l2, y);
                    for (int d = 0; d < 3; ++d) {
                        const int tmax = a[d] + b[d] < eo[d] ? a[d] + b[d] : eo[d];
                        double sdim = 0.0;
                        for (int t = 0; t <= tmax; ++t) sdim += E[d][a[d]][b[d]][t] * Mh[d][t];
                        prod *= sdim;
                    }
                    blk[x * n2 + y] += prod;
                }
            }
        }
    for (int x = 0; x < n1; ++x)
        for (int y = 0; y < n2; ++y) {
            const long long rc = mat_index(basis, s1, x, s2, y), cr = mat_index(basis, s2, y, s1, x);
            M[rc] = M[cr] = blk[x * n2 + y];
        }
}

// ---------------------------------------------------------------------------
__global__ void quartets_expand_kernel(long long ntask, const int *bra, const int *ket_start, const int *count,
                                       const long long *offset, const int *ket_list, int2 *out, long long nout) {
    const long long qi = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (qi >= nout) return;
    long long lo = 0, hi = ntask - 1;
    while (lo < hi) {
        const long long mid = (lo + hi + 1) >> 1;
        if (offset[mid] <= qi) lo = mid;
        else hi = mid - 1;
    }
    const long long k = qi - offset[lo];
    out[qi] = make_int2(bra[lo], ket_list ? ket_list[ket_start[lo] + k] : (int)(ket_start[lo] + k));
}

// Slot layout: one thread per slot copies its primitive pairs' fields and
// Hermite values from the pair (AoS) arrays.
__global__ void slots_fill_kernel(const sq_basis basis, const sq_pairs pairs, sq_slots slots) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= slots.nslot) return;
    const int P = slots.pair[s];
    const int a = pairs.shells[2 * P], b = pairs.shells[2 * P + 1];
    const int la = basis.l[a], lb = basis.l[b];
    int E = 0;
    for (int x = 0; x < ncart(la); ++x)
        for (int y = 0; y < ncart(lb); ++y) E += herm_terms(la, x, lb, y);
    const int n = slots.npp[s], stride = slots.pstride[s];
    const long long pb = slots.pbase[s], hb = slots.hbase[s], NPP = slots.npp_total;
    const long long src = pairs.pp_off[P];
    const long long hsrc = pairs.herm_off[P];
    for (int k = 0; k < n; ++k) {
        const long long dst = pb + (long long)k * stride;
        const int kk = slots.prim_src ? slots.prim_src[slots.prim_src_off[s] + k] : k;
        for (int f = 0; f < 5; ++f) {
            const double v = pairs.prim[8 * (src + kk) + f];
            slots.prim[f * NPP + dst] = v;
            if (slots.prim32) slots.prim32[f * NPP + dst] = (float)v;
            if (slots.prim32v) slots.prim32v[8 * dst + f] = (float)v;
            if (slots.primdf) {
                const float h = (float)v;
                slots.primdf[2 * (f * NPP + dst)] = h;
                slots.primdf[2 * (f * NPP + dst) + 1] = (float)(v - (double)h);
            }
        }
        if (slots.prim32v) {
            slots.prim32v[8 * dst + 5] = pairs.pq ? (float)pairs.pq[src + kk] : 0.0f;
            slots.prim32v[8 * dst + 6] = 0.0f;
            slots.prim32v[8 * dst + 7] = 0.0f;
        }
        for (int e = 0; e < E; ++e) {
            const double v = pairs.herm[hsrc + (long long)kk * E + e];
            const long long d = hb + ((long long)k * E + e) * stride;
            slots.herm[d] = v;
            if (slots.herm32) slots.herm32[d] = (float)v;
            if (slots.hermdf) {
                const float h = (float)v;
                slots.hermdf[2 * d] = h;
                slots.hermdf[2 * d + 1] = (float)(v - (double)h);
            }
        }
    }
}

// Slot descriptor (see sq_slots::desc): one thread per slot.
__global__ void slots_describe_kernel(const sq_basis basis, const sq_pairs pairs, sq_slots slots) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= slots.nslot) return;
    const int P = slots.pair[s];
    const int a = pairs.shells[2 * P], b = pairs.shells[2 * P + 1];
    int *d = slots.desc + 8 * (long long)s;
    d[0] = slots.npp[s];
    d[1] = slots.pbase[s];
    d[2] = slots.pstride[s];
    d[3] = (int)slots.hbase[s];
    d[4] = basis.bf_off[a];
    d[5] = basis.bf_off[b];
    d[6] = P | (a == b ? (1 << 30) : 0);
    d[7] = basis.mat_base == nullptr ? basis.nbf : basis.mat_ld[a];
    if (basis.mat_base != nullptr) slots.mbase[s] = basis.mat_base[a];
}

__global__ void fock_build_kernel(int nbf, const double *H, const double *Jacc, const double *Kacc, double *F,
                                  double *J, double *K) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = nbf;
    if (idx >= n * n) return;
    const long long r = idx / n, c = idx % n;
    const double j = 0.5 * (Jacc[r * n + c] + Jacc[c * n + r]);
    const double k = 0.5 * (Kacc[r * n + c] + Kacc[c * n + r]);
    if (F) F[idx] = H[idx] + j - 0.5 * k;
    if (J) J[idx] = j;
    if (K) K[idx] = k;
}

__global__ void to_float_kernel(long long n, const double *x, float *y) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = (float)x[i];
}

// x as double-float pairs: y[2i] = (float)x[i], y[2i+1] = (float)(x[i] - y[2i]).
__global__ void to_df_kernel(long long n, const double *x, float2 *y) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const double v = x[i];
        const float h = (float)v;
        y[i] = make_float2(h, (float)(v - (double)h));
    }
}

}  // namespace sq

using namespace sq;

extern "C" int sq_boys_table(double *table64, float *table32, void *stream) {
    if (!table64) return set_error(SQ_ERR_ARG, "sq_boys_table: table64 is NULL");
    const int n = SQ_BOYS_NGRID * SQ_BOYS_NCOL;
    boys_table_kernel<<<(n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(table64, table32, SQ_BOYS_NGRID,
                                                                         SQ_BOYS_NCOL);
    const int nh = SQ_BOYS_HI_NGRID * SQ_BOYS_HI_NCOL;
    boys_table_kernel<<<(nh + 127) / 128, 128, 0, (cudaStream_t)stream>>>(table64 + SQ_BOYS_HI64_OFF, nullptr,
                                                                          SQ_BOYS_HI_NGRID, SQ_BOYS_HI_NCOL);
    const int nt = 16 * SQ_BOYS_NGRID * 8;
    boys_taylor_kernel<<<(nt + 127) / 128, 128, 0, (cudaStream_t)stream>>>(table64, table32);
    return check_launch("sq_boys_table");
}

extern "C" int sq_boys(int n_max, const double *z, long long nz, const double *table64, int mode, double *out,
                       void *stream) {
    if (!z || !table64 || !out || nz < 0 || mode < 0 || mode > 2) return set_error(SQ_ERR_ARG, "sq_boys: bad argument");
    const int limit = mode == 0 ? SQ_BOYS_NCOL - 1 - kBoysTaylor64
                                : (mode == 2 ? SQ_BOYS_HI_NCOL - 1 - kBoysTaylor64 : SQ_BOYS_HI_NCOL - 2);
    if (n_max < 0 || n_max > limit) return set_error(SQ_ERR_ARG, "sq_boys: n_max %d out of range 0..%d", n_max, limit);
    if (nz == 0) return SQ_OK;
    boys_eval_kernel<<<(unsigned)((nz + 127) / 128), 128, 0, (cudaStream_t)stream>>>(n_max, z, nz, table64, mode,
                                                                                  out);
    return check_launch("sq_boys");
}

extern "C" int sq_boys_df(int n_max, const double *z, long long nz, const float *table32, double *out,
                          void *stream) {
    if (!z || !table32 || !out || nz < 0) return set_error(SQ_ERR_ARG, "sq_boys_df: bad argument");
    if (n_max < 0 || n_max > 8) return set_error(SQ_ERR_ARG, "sq_boys_df: n_max %d out of range (0..8)", n_max);
    if (nz == 0) return SQ_OK;
    cudaStream_t s = (cudaStream_t)stream;
    switch (n_max) {
        case 0: launch_boys_df<0>(z, nz, table32, out, s); break;
        case 1: launch_boys_df<1>(z, nz, table32, out, s); break;
        case 2: launch_boys_df<2>(z, nz, table32, out, s); break;
        case 3: launch_boys_df<3>(z, nz, table32, out, s); break;
        case 4: launch_boys_df<4>(z, nz, table32, out, s); break;
        case 5: launch_boys_df<5>(z, nz, table32, out, s); break;
        case 6: launch_boys_df<6>(z, nz, table32, out, s); break;
        case 7: launch_boys_df<7>(z, nz, table32, out, s); break;
        default: launch_boys_df<8>(z, nz, table32, out, s); break;
    }
    return check_launch("sq_boys_df");
}

extern "C" int sq_pair_prep(const sq_basis *basis, sq_pairs *pairs, void *stream) {
    if (!basis || !pairs || !pairs->prim || !pairs->herm || !pairs->shells || !pairs->pp_off || !pairs->herm_off)
        return set_error(SQ_ERR_ARG, "sq_pair_prep: bad argument");
    if (pairs->nprimpair <= 0) return SQ_OK;
    pair_prep_kernel<<<(pairs->nprimpair + 127) / 128, 128, 0, (cudaStream_t)stream>>>(*basis, *pairs);
    return check_launch("sq_pair_prep");
}

extern "C" int sq_one_electron(const sq_basis *basis, const double *table64, double *S, double *T, double *V,
                               void *stream) {
    if (!basis || !table64) return set_error(SQ_ERR_ARG, "sq_one_electron: bad argument");
    const int np = basis->nshell * (basis->nshell + 1) / 2;
    if (np == 0) return SQ_OK;
    one_electron_kernel<<<(np + 63) / 64, 64, 0, (cudaStream_t)stream>>>(*basis, table64, S, T, V);
    return check_launch("sq_one_electron");
}

extern "C" int sq_multipole(const sq_basis *basis, const int *order, const double *origin, double *M,
                            void *stream) {
    if (!basis || !order || !origin || !M) return set_error(SQ_ERR_ARG, "sq_multipole: NULL argument");
    for (int d = 0; d < 3; ++d)
        if (order[d] < 0 || order[d] > kMultipoleMax)
            return set_error(SQ_ERR_ARG, "sq_multipole: order %d out of range 0..%d", order[d], kMultipoleMax);
    const int np = basis->nshell * (basis->nshell + 1) / 2;
    if (np == 0) return SQ_OK;
    multipole_kernel<<<(np + 63) / 64, 64, 0, (cudaStream_t)stream>>>(*basis, order[0], order[1], order[2],
                                                                       origin[0], origin[1], origin[2], M);
    return check_launch("sq_multipole");
}

extern "C" int sq_quartets_expand(long long ntask, const int *bra, const int *ket_start, const int *count,
                                  const long long *offset, const int *ket_list, int *out_pairs, long long nout,
                                  void *stream) {
    if (ntask < 0 || nout < 0) return set_error(SQ_ERR_ARG, "sq_quartets_expand: negative size");
    if (ntask == 0 || nout == 0) return SQ_OK;
    if (!bra || !ket_start || !count || !offset || !out_pairs)
        return set_error(SQ_ERR_ARG, "sq_quartets_expand: NULL pointer");
    quartets_expand_kernel<<<(unsigned)((nout + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        ntask, bra, ket_start, count, offset, ket_list, (int2 *)out_pairs, nout);
    return check_launch("sq_quartets_expand");
}

extern "C" int sq_slots_fill(const sq_basis *basis, const sq_pairs *pairs, sq_slots *slots, void *stream) {
    if (!basis || !pairs || !slots || !slots->pair || !slots->npp || !slots->pbase || !slots->pstride ||
        !slots->hbase || !slots->prim || !slots->herm)
        return set_error(SQ_ERR_ARG, "sq_slots_fill: bad argument");
    if (slots->nslot <= 0) return SQ_OK;
    slots_fill_kernel<<<(slots->nslot + 127) / 128, 128, 0, (cudaStream_t)stream>>>(*basis, *pairs, *slots);
    return check_launch("sq_slots_fill");
}

extern "C" int sq_slots_describe(const sq_basis *basis, const sq_pairs *pairs, sq_slots *slots, void *stream) {
    if (!basis || !pairs || !slots || !slots->pair || !slots->npp || !slots->pbase || !slots->pstride ||
        !slots->hbase || !slots->desc || !pairs->shells ||
        (basis->mat_base != nullptr && (!basis->mat_ld || !slots->mbase)))
        return set_error(SQ_ERR_ARG, "sq_slots_describe: bad argument");
    if (slots->nherm_total >= (1LL << 31) || pairs->npair >= (1 << 30))
        return set_error(SQ_ERR_ARG, "sq_slots_describe: %lld Hermite values / %d pairs exceed the descriptor's "
                         "32-bit fields", slots->nherm_total, pairs->npair);
    if (slots->nslot <= 0) return SQ_OK;
    slots_describe_kernel<<<(slots->nslot + 127) / 128, 128, 0, (cudaStream_t)stream>>>(*basis, *pairs, *slots);
    return check_launch("sq_slots_describe");
}

extern "C" int sq_fock_build(int nbf, const double *H, const double *Jacc, const double *Kacc, double *F, double *J,
                             double *K, void *stream) {
    if (nbf <= 0 || !Jacc || !Kacc || (F && !H)) return set_error(SQ_ERR_ARG, "sq_fock_build: bad argument");
    const long long n2 = (long long)nbf * nbf;
    fock_build_kernel<<<(unsigned)((n2 + 255) / 256), 256, 0, (cudaStream_t)stream>>>(nbf, H, Jacc, Kacc, F, J, K);
    return check_launch("sq_fock_build");
}

namespace sq {
int to_float(long long n, const double *x, float *y, cudaStream_t stream) {
    if (n <= 0) return SQ_OK;
    to_float_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(n, x, y);
    return check_launch("to_float");
}

int to_df(long long n, const double *x, float *y, cudaStream_t stream) {
    if (n <= 0) return SQ_OK;
    to_df_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(n, x, reinterpret_cast<float2 *>(y));
    return check_launch("to_df");
}
}  // namespace sq

// ---------------------------------------------------------------------------
// Arithmetic-pipe probe: independent FMA chains, 16 per thread per iteration.
namespace sq {
template <typename T>
__global__ void fma_probe_kernel(T *out, int iters, T a, T b) {
    T x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = (T)(threadIdx.x + k);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += x[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// The same chains in double-float arithmetic (csrc/df64.cuh): one fma is two
// FP64-model FLOPs carried out by about fifteen FP32 instructions.
__global__ void fma_probe_df_kernel(float2 *out, int iters, dfl a, dfl b) {
    dfl x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = dfl((float)(threadIdx.x + k));
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
    }
    dfl s(0.0f);
#pragma unroll
    for (int k = 0; k < 8; ++k) s = s + x[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = make_float2(s.hi, s.lo);
}
}  // namespace sq

extern "C" int sq_fma_probe(int precision, int blocks, int iters, void *out, void *stream) {
    if (blocks <= 0 || iters <= 0 || !out) return set_error(SQ_ERR_ARG, "sq_fma_probe: bad argument");
    if (precision == SQ_FP64)
        sq::fma_probe_kernel<double><<<blocks, 256, 0, (cudaStream_t)stream>>>((double *)out, iters, 1.0000001, 1e-9);
    else if (precision == SQ_DF64)
        sq::fma_probe_df_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>((float2 *)out, iters, sq::dfl(1.0000001),
                                                                          sq::dfl(1e-9));
    else
        sq::fma_probe_kernel<float><<<blocks, 256, 0, (cudaStream_t)stream>>>((float *)out, iters, 1.0000001f, 1e-9f);
    return check_launch("sq_fma_probe");
}
