/*
 * sq_oracle.c -- CPU restatement of SlowQuant's molecular-integral hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: the parity tests, the
 * smoke check and the CPU-baseline leg of the benchmark call it to check (or
 * time beside) the CUDA path.  Nothing in the product library links it.
 *
 * Every routine restates the reference's arithmetic in C, with the same
 * branches and loop structure (paths relative to the SlowQuant project):
 *   factorial2                 slowquant/molecule/moleculefunctions.py:7-26
 *   boys_function              slowquant/molecularintegrals/integralfunctions.py:74-97
 *   expansion_coefficients     slowquant/molecularintegrals/integralfunctions.py:9-71
 *   hermite_coulomb_integral   slowquant/molecularintegrals/integralfunctions.py:100-148
 *   electron_repulsion_integral slowquant/molecularintegrals/electronrepulsion.py:107-297
 *   electron_repulsion_integral_driver  electronrepulsion.py:11-104
 *   get_cauchy_schwarz_matrix  electronrepulsion.py:300-339
 *   J/K einsums (direct)       slowquant/hartreefock/hartreefock_in_memory.py:55-56
 *   multipole (overlap)        slowquant/molecularintegrals/multipole.py:48-135
 *   kinetic_energy_integral    slowquant/molecularintegrals/kineticenergy.py:42-133
 *   nuclear_attraction_integral slowquant/molecularintegrals/nuclearattraction.py:47-135
 *
 * "faithful" mode reproduces the reference's hermite_coulomb_integral call with
 * angular_x = angular_y = angular_z = L (electronrepulsion.py:244-250): a full
 * (L+1)^3 x (3L+2) table with Boys values up to n = 3L.  Mode 0 builds only the
 * t+u+v <= L entries the contraction reads (same recurrences, same Boys
 * branches); R^0 entries are identical in both modes.
 *
 * Shell-quartet loops are parallelised with OpenMP (the reference is
 * single-threaded); each thread owns whole quartets.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    int nshell;
    const double *center;   /* [nshell][3] */
    const int *nprim;       /* [nshell] */
    const int *prim_off;    /* [nshell] offset into exps/coefs */
    const int *ncart;       /* [nshell] number of Cartesian components */
    const int *cart_off;    /* [nshell] offset (in components) into cart */
    const int *bf_off;      /* [nshell] first basis-function index */
    const int *norm_off;    /* [nshell] offset into norm ([ncart][nprim] row-major) */
    const double *exps;
    const double *coefs;
    const int *cart;        /* [ncart_total][3] */
    const double *norm;
    int nbf;
} sqo_basis;

/* moleculefunctions.py:7-26 */
double sqo_factorial2(double number) {
    double out = 1.0;
    if (number > 0) {
        int n = (int)(number + 1) / 2;
        for (int i = 0; i < n; i++) out = out * (number - 2 * i);
    }
    return out;
}

/*
 * Boys-function mode: 0 (default) restates the reference's piecewise formula
 * exactly; 1 evaluates the same series to full double precision (relative
 * stopping test, asymptote only beyond z = 60, where its neglected term is
 * below 2e-13 relative up to n = 13).  Mode 1 exists to measure how far the
 * reference's own truncation moves the integrals.
 */
static int g_boys_mode = 0;
void sqo_set_boys_mode(int mode) { g_boys_mode = mode; }

static double boys_exact(int n, double z) {
    const double pi = 3.141592653589793;
    if (z > 60.0) {
        double F = 0.5 * sqrt(pi / z);
        for (int m = 0; m < n; m++) F *= (2 * m + 1) / (2.0 * z);
        return F;
    }
    double term = 1.0 / (2 * n + 1), sum = 0.0;
    for (int i = 0; i < 2000; i++) {
        sum += term;
        term *= 2.0 * z / (2 * n + 2 * i + 3);
        if (term < 1e-18 * sum) break;
    }
    return sum * exp(-z);
}

/* integralfunctions.py:74-97 */
double sqo_boys(int n, double z) {
    const double pi = 3.141592653589793;
    double F;
    if (g_boys_mode == 1) return boys_exact(n, z);
    if (n == 0 && z < 1e-10) {
        F = 1.0;
    } else if (n == 0) {
        F = pow(pi / (4.0 * z), 0.5) * erf(pow(z, 0.5));
    } else if (z > 25) {
        F = sqo_factorial2(2 * n - 1) / pow(2.0, n + 1.0) * pow(pi / pow(z, 2.0 * n + 1.0), 0.5);
    } else if (z < 1e-10) {
        F = 1.0 / (2.0 * n + 1.0);
    } else {
        F = 0.0;
        const double threshold = 1e-12;
        for (int i = 0; i < 1000; i++) {
            double Fcheck = F;
            F += pow(2.0 * z, (double)i) / sqo_factorial2(2 * n + 2 * i + 1);
            Fcheck -= F;
            if (fabs(Fcheck) < threshold) break;
        }
        F *= exp(-z) * sqo_factorial2(2 * n - 1);
    }
    return F;
}

/* integralfunctions.py:9-71.  out is [la+1][lb+1][la+lb+1] row-major. */
void sqo_expansion_coefficients(double A_x, double B_x, double a, double b, int la, int lb, double *out) {
    const double X_AB = A_x - B_x;
    const double p = a + b;
    const double mu = a * b / (a + b);
    const double P_x = (a * A_x + b * B_x) / p;
    const double X_PA = P_x - A_x;
    const double X_PB = P_x - B_x;
    const int nj = lb + 1, nt = la + lb + 1;
#define EIDX(i, j, t) (((i) * nj + (j)) * nt + (t))
    for (int i = 0; i <= la; i++)
        for (int j = 0; j <= lb; j++)
            for (int t = 0; t < nt; t++) {
                double value = 0.0;
                if (i == 0 && j == 0 && t == 0) {
                    value = exp(-mu * X_AB * X_AB);
                } else if (i == 0) {
                    if (j > 0 && t > 0) value += 1 / (2 * p) * out[EIDX(i, j - 1, t - 1)];
                    if (j > 0) value += X_PB * out[EIDX(i, j - 1, t)];
                    if (j > 0 && t + 1 <= i + j) value += (t + 1) * out[EIDX(i, j - 1, t + 1)];
                } else {
                    if (i > 0 && t > 0) value += 1 / (2 * p) * out[EIDX(i - 1, j, t - 1)];
                    if (i > 0) value += X_PA * out[EIDX(i - 1, j, t)];
                    if (i > 0 && t + 1 <= i + j) value += (t + 1) * out[EIDX(i - 1, j, t + 1)];
                }
                out[EIDX(i, j, t)] = value;
            }
#undef EIDX
}

/*
 * integralfunctions.py:100-148.  Computes R^n_{tuv} for t<=ax,u<=ay,v<=az,
 * n<=ax+ay+az in a scratch table and returns R^0 in out[(ax+1)(ay+1)(az+1)].
 * With triangular != 0 only entries with t+u+v+n <= ax (ax=ay=az=L) are formed:
 * the R^0_{tuv}, t+u+v<=L, that the ERI contraction reads.
 */
static void hermite_coulomb(int ax, int ay, int az, double p, const double *PC, double *out, double *scratch,
                            int triangular) {
    const double X = PC[0], Y = PC[1], Z = PC[2];
    const double R_PC = pow(X * X + Y * Y + Z * Z, 0.5);
    const int nu = ay + 1, nv = az + 1, nn = ax + ay + az + 2;
#define RIDX(t, u, v, n) ((((t) * nu + (u)) * nv + (v)) * nn + (n))
    const size_t total = (size_t)(ax + 1) * nu * nv * nn;
    memset(scratch, 0, total * sizeof(double));
    for (int t = 0; t <= ax; t++)
        for (int u = 0; u <= ay; u++)
            for (int v = 0; v <= az; v++) {
                int nmax = ax + ay + az;
                if (triangular) {
                    if (t + u + v > ax) continue;
                    nmax = ax - (t + u + v);
                }
                for (int n = 0; n <= nmax; n++) {
                    double value = 0.0;
                    if (t == 0 && u == 0 && v == 0) {
                        value = pow(-2.0 * p, (double)n) * sqo_boys(n, p * R_PC * R_PC);
                    } else if (t == 0 && u == 0) {
                        if (v > 1) value += (v - 1) * scratch[RIDX(t, u, v - 2, n + 1)];
                        if (v > 0) value += Z * scratch[RIDX(t, u, v - 1, n + 1)];
                    } else if (t == 0) {
                        if (u > 1) value += (u - 1) * scratch[RIDX(t, u - 2, v, n + 1)];
                        if (u > 0) value += Y * scratch[RIDX(t, u - 1, v, n + 1)];
                    } else {
                        if (t > 1) value += (t - 1) * scratch[RIDX(t - 2, u, v, n + 1)];
                        if (t > 0) value += X * scratch[RIDX(t - 1, u, v, n + 1)];
                    }
                    scratch[RIDX(t, u, v, n)] = value;
                }
            }
    for (int t = 0; t <= ax; t++)
        for (int u = 0; u <= ay; u++)
            for (int v = 0; v <= az; v++) out[(t * nu + u) * nv + v] = scratch[RIDX(t, u, v, 0)];
#undef RIDX
}

void sqo_hermite_coulomb(int ax, int ay, int az, double p, const double *PC, double *out) {
    size_t total = (size_t)(ax + 1) * (ay + 1) * (az + 1) * (ax + ay + az + 2);
    double *scratch = (double *)malloc(total * sizeof(double));
    hermite_coulomb(ax, ay, az, p, PC, out, scratch, 0);
    free(scratch);
}

static int shell_lmax(const sqo_basis *B, int s) {
    int m = 0;
    for (int c = 0; c < B->ncart[s]; c++)
        for (int d = 0; d < 3; d++) {
            int v = B->cart[3 * (B->cart_off[s] + c) + d];
            if (v > m) m = v;
        }
    return m;
}

/*
 * electronrepulsion.py:107-297 for shells (s1 s2 | s3 s4).  out receives the
 * contracted block [nbf1][nbf2][nbf3][nbf4].  work must hold eri_work_size()
 * doubles.
 */
static size_t eri_work_size(const sqo_basis *B) {
    int maxL = 0, maxprim = 0;
    size_t maxcp = 0; /* largest (components x primitives) of one shell */
    for (int s = 0; s < B->nshell; s++) {
        const int l = shell_lmax(B, s);
        if (l > maxL) maxL = l;
        if (B->nprim[s] > maxprim) maxprim = B->nprim[s];
        const size_t cp = (size_t)B->ncart[s] * B->nprim[s];
        if (cp > maxcp) maxcp = cp;
    }
    size_t Lt = 4 * (size_t)maxL;
    size_t rtab = (Lt + 1) * (Lt + 1) * (Lt + 1) * (3 * Lt + 2);
    size_t rout = (Lt + 1) * (Lt + 1) * (Lt + 1);
    size_t e1 = (size_t)(maxL + 1) * (maxL + 1) * (2 * maxL + 1);
    size_t pre = (size_t)maxprim * maxprim * e1 * 3;
    size_t vprim = maxcp * maxcp * maxcp * maxcp;
    return rtab + rout + 3 * e1 + pre + vprim;
}

static void eri_block(const sqo_basis *B, int s1, int s2, int s3, int s4, double *out, double *work,
                      int faithful) {
    const double pi = 3.141592653589793;
    const int sh[4] = {s1, s2, s3, s4};
    int np[4], nb[4], lm[4];
    for (int q = 0; q < 4; q++) {
        np[q] = B->nprim[sh[q]];
        nb[q] = B->ncart[sh[q]];
        lm[q] = shell_lmax(B, sh[q]);
    }
    const double *c1 = B->center + 3 * s1, *c2 = B->center + 3 * s2, *c3 = B->center + 3 * s3,
                 *c4 = B->center + 3 * s4;
    const double *e1 = B->exps + B->prim_off[s1], *e2 = B->exps + B->prim_off[s2],
                 *e3 = B->exps + B->prim_off[s3], *e4 = B->exps + B->prim_off[s4];
    const double *k1 = B->coefs + B->prim_off[s1], *k2 = B->coefs + B->prim_off[s2],
                 *k3 = B->coefs + B->prim_off[s3], *k4 = B->coefs + B->prim_off[s4];
    const double *n1 = B->norm + B->norm_off[s1], *n2 = B->norm + B->norm_off[s2],
                 *n3 = B->norm + B->norm_off[s3], *n4 = B->norm + B->norm_off[s4];
    const int *a1 = B->cart + 3 * B->cart_off[s1], *a2 = B->cart + 3 * B->cart_off[s2],
              *a3 = B->cart + 3 * B->cart_off[s3], *a4 = B->cart + 3 * B->cart_off[s4];

    const int Ltot = lm[0] + lm[1] + lm[2] + lm[3];
    const int LT = Ltot + 1;
    double *rtab = work;
    double *R = rtab + (size_t)LT * LT * LT * (3 * Ltot + 2);
    double *Exb = R + (size_t)LT * LT * LT;
    const int eb_j = lm[1] + 1, eb_t = lm[0] + lm[1] + 1;
    const size_t eb_sz = (size_t)(lm[0] + 1) * eb_j * eb_t;
    double *Eyb = Exb + eb_sz, *Ezb = Eyb + eb_sz;
    double *preE = Ezb + eb_sz;
    const int ek_j = lm[3] + 1, ek_t = lm[2] + lm[3] + 1;
    const size_t ek_sz = (size_t)(lm[2] + 1) * ek_j * ek_t;
    double *Vp = preE + (size_t)np[2] * np[3] * ek_sz * 3;
    const size_t nV = (size_t)nb[0] * nb[1] * nb[2] * nb[3];
    const size_t nP = (size_t)np[0] * np[1] * np[2] * np[3];
    memset(Vp, 0, nV * nP * sizeof(double));
#define PREE(k, l, d) (preE + (((size_t)(k) * np[3] + (l)) * 3 + (d)) * ek_sz)
#define VP(bi, bj, bk, bl, i, j, k, l) \
    Vp[((((((((size_t)(bi) * nb[1] + (bj)) * nb[2] + (bk)) * nb[3] + (bl)) * np[0] + (i)) * np[1] + (j)) * np[2] + (k)) * np[3] + (l))]

    for (int k = 0; k < np[2]; k++)
        for (int l = 0; l < np[3]; l++)
            for (int d = 0; d < 3; d++)
                sqo_expansion_coefficients(c3[d], c4[d], e3[k], e4[l], lm[2], lm[3], PREE(k, l, d));

    for (int i = 0; i < np[0]; i++)
        for (int j = 0; j < np[1]; j++) {
            sqo_expansion_coefficients(c1[0], c2[0], e1[i], e2[j], lm[0], lm[1], Exb);
            sqo_expansion_coefficients(c1[1], c2[1], e1[i], e2[j], lm[0], lm[1], Eyb);
            sqo_expansion_coefficients(c1[2], c2[2], e1[i], e2[j], lm[0], lm[1], Ezb);
            const double p = e1[i] + e2[j];
            double P[3];
            for (int d = 0; d < 3; d++) P[d] = (e1[i] * c1[d] + e2[j] * c2[d]) / p;
            for (int k = 0; k < np[2]; k++)
                for (int l = 0; l < np[3]; l++) {
                    const double q = e3[k] + e4[l];
                    double Q[3], PQ[3];
                    for (int d = 0; d < 3; d++) {
                        Q[d] = (e3[k] * c3[d] + e4[l] * c4[d]) / q;
                        PQ[d] = P[d] - Q[d];
                    }
                    const double alpha = p * q / (p + q);
                    hermite_coulomb(Ltot, Ltot, Ltot, alpha, PQ, R, rtab, !faithful);
                    const double *Exk = PREE(k, l, 0), *Eyk = PREE(k, l, 1), *Ezk = PREE(k, l, 2);
#define RR(t, u, v) R[((t) * LT + (u)) * LT + (v)]
#define EB(E, x, y, t) E[((x) * eb_j + (y)) * eb_t + (t)]
#define EK(E, x, y, t) E[((x) * ek_j + (y)) * ek_t + (t)]
                    for (int bi = 0; bi < nb[0]; bi++) {
                        const int x1 = a1[3 * bi], y1 = a1[3 * bi + 1], z1 = a1[3 * bi + 2];
                        for (int bj = 0; bj < nb[1]; bj++) {
                            const int x2 = a2[3 * bj], y2 = a2[3 * bj + 1], z2 = a2[3 * bj + 2];
                            for (int bk = 0; bk < nb[2]; bk++) {
                                const int x3 = a3[3 * bk], y3 = a3[3 * bk + 1], z3 = a3[3 * bk + 2];
                                for (int bl = 0; bl < nb[3]; bl++) {
                                    const int x4 = a4[3 * bl], y4 = a4[3 * bl + 1], z4 = a4[3 * bl + 2];
                                    double acc = VP(bi, bj, bk, bl, i, j, k, l);
                                    for (int tau = 0; tau <= x3 + x4; tau++)
                                        for (int nu = 0; nu <= y3 + y4; nu++)
                                            for (int phi = 0; phi <= z3 + z4; phi++) {
                                                const double sgn = ((tau + nu + phi) & 1) ? -1.0 : 1.0;
                                                const double E_temp = sgn * EK(Exk, x3, x4, tau) *
                                                                      EK(Eyk, y3, y4, nu) * EK(Ezk, z3, z4, phi);
                                                for (int t = 0; t <= x1 + x2; t++)
                                                    for (int u = 0; u <= y1 + y2; u++)
                                                        for (int v = 0; v <= z1 + z2; v++)
                                                            acc += E_temp * EB(Exb, x1, x2, t) *
                                                                   EB(Eyb, y1, y2, u) * EB(Ezb, z1, z2, v) *
                                                                   RR(t + tau, u + nu, v + phi);
                                            }
                                    acc *= n1[bi * np[0] + i] * n2[bj * np[1] + j] * n3[bk * np[2] + k] *
                                           n4[bl * np[3] + l];
                                    VP(bi, bj, bk, bl, i, j, k, l) = acc;
                                }
                            }
                        }
                    }
                    const double pref = 2 * pow(pi, 5.0 / 2.0) / (p * q * pow(p + q, 0.5));
                    for (int bi = 0; bi < nb[0]; bi++)
                        for (int bj = 0; bj < nb[1]; bj++)
                            for (int bk = 0; bk < nb[2]; bk++)
                                for (int bl = 0; bl < nb[3]; bl++) VP(bi, bj, bk, bl, i, j, k, l) *= pref;
#undef RR
#undef EB
#undef EK
                }
        }
    for (int bi = 0; bi < nb[0]; bi++)
        for (int bj = 0; bj < nb[1]; bj++)
            for (int bk = 0; bk < nb[2]; bk++)
                for (int bl = 0; bl < nb[3]; bl++) {
                    double s = 0.0;
                    for (int i = 0; i < np[0]; i++)
                        for (int j = 0; j < np[1]; j++)
                            for (int k = 0; k < np[2]; k++)
                                for (int l = 0; l < np[3]; l++)
                                    s += k1[i] * k2[j] * k3[k] * k4[l] * VP(bi, bj, bk, bl, i, j, k, l);
                    out[((bi * nb[1] + bj) * nb[2] + bk) * nb[3] + bl] = s;
                }
#undef PREE
#undef VP
}

static void basis_limits(const sqo_basis *B, int *maxL, int *maxprim, int *maxcart) {
    *maxL = 0;
    *maxprim = 0;
    *maxcart = 0;
    for (int s = 0; s < B->nshell; s++) {
        int l = shell_lmax(B, s);
        if (l > *maxL) *maxL = l;
        if (B->nprim[s] > *maxprim) *maxprim = B->nprim[s];
        if (B->ncart[s] > *maxcart) *maxcart = B->ncart[s];
    }
}

/* One contracted shell-quartet block, [nbf1][nbf2][nbf3][nbf4]. */
int sqo_eri_block(const sqo_basis *B, int s1, int s2, int s3, int s4, double *out, int faithful) {
    int maxL, maxprim, maxcart;
    basis_limits(B, &maxL, &maxprim, &maxcart);
    double *work = (double *)malloc(eri_work_size(B) * sizeof(double));
    if (!work) return 1;
    eri_block(B, s1, s2, s3, s4, out, work, faithful);
    free(work);
    return 0;
}

/* electronrepulsion.py:300-339: cs[i,j] = sqrt(max over the (ij|ij) block). */
int sqo_schwarz(const sqo_basis *B, double *cs, int nthreads, int faithful) {
    int maxL, maxprim, maxcart;
    basis_limits(B, &maxL, &maxprim, &maxcart);
    const int n = B->nshell;
    const size_t wsz = eri_work_size(B);
    const size_t bsz = (size_t)maxcart * maxcart * maxcart * maxcart;
    int err = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel
    {
        double *work = (double *)malloc(wsz * sizeof(double));
        double *blk = (double *)malloc(bsz * sizeof(double));
        if (!work || !blk) {
#pragma omp atomic write
            err = 1;
        } else {
#pragma omp for schedule(dynamic, 1)
            for (int ij = 0; ij < n * n; ij++) {
                const int i = ij / n, j = ij % n;
                if (j < i) continue;
                eri_block(B, i, j, i, j, blk, work, faithful);
                const size_t m = (size_t)B->ncart[i] * B->ncart[j] * B->ncart[i] * B->ncart[j];
                double mx = blk[0];
                for (size_t x = 1; x < m; x++)
                    if (blk[x] > mx) mx = blk[x];
                cs[i * n + j] = cs[j * n + i] = pow(mx, 0.5);
            }
        }
        free(work);
        free(blk);
    }
    return err;
}

/*
 * electronrepulsion.py:11-104.  Dense V[nbf^4].  The reference visits i<=j,
 * k<=l and keeps "ij >= kl" with ij = i(i+1)/2 + j; that index is not a
 * bijection, so some quartets are visited twice (same values written).  Here
 * each visited quartet is one task of an OpenMP loop; the scatter writes the
 * eight index permutations exactly as the reference does.  cs may be NULL.
 */
int sqo_eri_dense(const sqo_basis *B, const double *cs, double thr, double *V, int nthreads, int faithful) {
    int maxL, maxprim, maxcart;
    basis_limits(B, &maxL, &maxprim, &maxcart);
    const int n = B->nshell;
    const size_t nbf = (size_t)B->nbf;
    const size_t wsz = eri_work_size(B);
    const size_t bsz = (size_t)maxcart * maxcart * maxcart * maxcart;
    memset(V, 0, nbf * nbf * nbf * nbf * sizeof(double));
    int err = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel
    {
        double *work = (double *)malloc(wsz * sizeof(double));
        double *blk = (double *)malloc(bsz * sizeof(double));
        if (!work || !blk) {
#pragma omp atomic write
            err = 1;
        } else {
#pragma omp for schedule(dynamic, 1) collapse(2)
            for (int i = 0; i < n; i++)
                for (int j = 0; j < n; j++) {
                    if (j < i) continue;
                    const long ij = (long)i * (i + 1) / 2 + j;
                    for (int k = 0; k < n; k++)
                        for (int l = k; l < n; l++) {
                            const long kl = (long)k * (k + 1) / 2 + l;
                            if (ij < kl) continue;
                            if (cs && cs[i * n + j] * cs[k * n + l] < thr) continue;
                            eri_block(B, i, j, k, l, blk, work, faithful);
                            const int nb1 = B->ncart[i], nb2 = B->ncart[j], nb3 = B->ncart[k], nb4 = B->ncart[l];
                            const size_t o1 = B->bf_off[i], o2 = B->bf_off[j], o3 = B->bf_off[k], o4 = B->bf_off[l];
                            for (int a = 0; a < nb1; a++)
                                for (int b = 0; b < nb2; b++)
                                    for (int c = 0; c < nb3; c++)
                                        for (int d = 0; d < nb4; d++) {
                                            const double v = blk[((a * nb2 + b) * nb3 + c) * nb4 + d];
                                            const size_t A = o1 + a, Bq = o2 + b, C = o3 + c, D = o4 + d;
#define W(p, q, r, s) V[(((p) * nbf + (q)) * nbf + (r)) * nbf + (s)] = v
                                            W(A, Bq, C, D);
                                            W(Bq, A, C, D);
                                            W(A, Bq, D, C);
                                            W(Bq, A, D, C);
                                            W(C, D, A, Bq);
                                            W(C, D, Bq, A);
                                            W(D, C, A, Bq);
                                            W(D, C, Bq, A);
#undef W
                                        }
                        }
                }
        }
        free(work);
        free(blk);
    }
    return err;
}

/*
 * Contracted blocks for an explicit list of shell quartets (4 ints each); the
 * blocks are packed back to back in out.  Used to time a bounded sample of a
 * large workload and to check single quartets.
 */
int sqo_eri_quartets(const sqo_basis *B, const int *quartets, long nq, double *out, const long *out_off,
                     int nthreads, int faithful) {
    int maxL, maxprim, maxcart;
    basis_limits(B, &maxL, &maxprim, &maxcart);
    const size_t wsz = eri_work_size(B);
    int err = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel
    {
        double *work = (double *)malloc(wsz * sizeof(double));
        if (!work) {
#pragma omp atomic write
            err = 1;
        } else {
#pragma omp for schedule(dynamic, 4)
            for (long q = 0; q < nq; q++)
                eri_block(B, quartets[4 * q], quartets[4 * q + 1], quartets[4 * q + 2], quartets[4 * q + 3],
                          out + out_off[q], work, faithful);
        }
        free(work);
    }
    return err;
}

/*
 * Integral-direct J and K: the two einsums of hartreefock_in_memory.py:55-56,
 *   J[p,q] = sum_rs V[p,q,r,s] D[s,r],   K[p,q] = sum_rs V[p,s,q,r] D[s,r],
 * over the tensor that electronrepulsion.py:11-104 would store, without
 * storing it.  The shell quartets are those of the driver (i <= j, k <= l,
 * pair (i,j) at or after pair (k,l), Schwarz skip cs[i,j] cs[k,l] < thr),
 * enumerated once each.  Every element of a block stands for the distinct
 * index tuples of its 8-fold orbit (the tuples the driver's scatter writes);
 * the element that is the lexicographically smallest member of its orbit
 * inside this block's index ranges adds the orbit's tuples to J and K, so
 * each tensor entry is summed exactly once, as in the einsum.  OpenMP threads
 * accumulate into private matrices that are added at the end.  cs may be NULL.
 */
static int in_block(const sqo_basis *B, const int *sh, const long *t) {
    for (int q = 0; q < 4; q++)
        if (t[q] < B->bf_off[sh[q]] || t[q] >= B->bf_off[sh[q]] + B->ncart[sh[q]]) return 0;
    return 1;
}

static int tuple_less(const long *a, const long *b) {
    for (int q = 0; q < 4; q++) {
        if (a[q] != b[q]) return a[q] < b[q];
    }
    return 0;
}

int sqo_jk_direct(const sqo_basis *B, const double *cs, double thr, const double *D, double *J, double *K,
                  int nthreads) {
    int maxL, maxprim, maxcart;
    basis_limits(B, &maxL, &maxprim, &maxcart);
    const int n = B->nshell;
    const long nbf = B->nbf;
    const size_t wsz = eri_work_size(B);
    const size_t bsz = (size_t)maxcart * maxcart * maxcart * maxcart;
    const long npair = (long)n * (n + 1) / 2;
    int *pi = (int *)malloc(npair * sizeof(int)), *pj = (int *)malloc(npair * sizeof(int));
    if (!pi || !pj) return 1;
    long np_ = 0;
    for (int i = 0; i < n; i++)
        for (int j = i; j < n; j++) {
            pi[np_] = i;
            pj[np_] = j;
            np_++;
        }
    memset(J, 0, nbf * nbf * sizeof(double));
    memset(K, 0, nbf * nbf * sizeof(double));
    int err = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel
    {
        double *work = (double *)malloc(wsz * sizeof(double));
        double *blk = (double *)malloc(bsz * sizeof(double));
        double *Jt = (double *)calloc(nbf * nbf, sizeof(double));
        double *Kt = (double *)calloc(nbf * nbf, sizeof(double));
        if (!work || !blk || !Jt || !Kt) {
#pragma omp atomic write
            err = 1;
        } else {
#pragma omp for schedule(dynamic, 1)
            for (long P = npair - 1; P >= 0; P--) {
                const int i = pi[P], j = pj[P];
                for (long Q = 0; Q <= P; Q++) {
                    const int k = pi[Q], l = pj[Q];
                    if (cs && cs[i * n + j] * cs[k * n + l] < thr) continue;
                    const int sh[4] = {i, j, k, l};
                    eri_block(B, i, j, k, l, blk, work, 0);
                    const int nb1 = B->ncart[i], nb2 = B->ncart[j], nb3 = B->ncart[k], nb4 = B->ncart[l];
                    for (int a = 0; a < nb1; a++)
                        for (int b = 0; b < nb2; b++)
                            for (int c = 0; c < nb3; c++)
                                for (int d = 0; d < nb4; d++) {
                                    const double v = blk[((a * nb2 + b) * nb3 + c) * nb4 + d];
                                    const long A = B->bf_off[i] + a, Bq = B->bf_off[j] + b, C = B->bf_off[k] + c,
                                               Dd = B->bf_off[l] + d;
                                    const long perm[8][4] = {{A, Bq, C, Dd}, {Bq, A, C, Dd}, {A, Bq, Dd, C},
                                                             {Bq, A, Dd, C}, {C, Dd, A, Bq}, {C, Dd, Bq, A},
                                                             {Dd, C, A, Bq}, {Dd, C, Bq, A}};
                                    int first = 1;
                                    for (int x = 1; x < 8 && first; x++)
                                        if (in_block(B, sh, perm[x]) && tuple_less(perm[x], perm[0])) first = 0;
                                    if (!first) continue;
                                    for (int x = 0; x < 8; x++) {
                                        int dup = 0;
                                        for (int y = 0; y < x && !dup; y++)
                                            dup = perm[y][0] == perm[x][0] && perm[y][1] == perm[x][1] &&
                                                  perm[y][2] == perm[x][2] && perm[y][3] == perm[x][3];
                                        if (dup) continue;
                                        const long w = perm[x][0], xx = perm[x][1], y = perm[x][2], z = perm[x][3];
                                        Jt[w * nbf + xx] += v * D[z * nbf + y];
                                        Kt[w * nbf + y] += v * D[xx * nbf + z];
                                    }
                                }
                }
            }
#pragma omp critical
            {
                for (long x = 0; x < nbf * nbf; x++) {
                    J[x] += Jt[x];
                    K[x] += Kt[x];
                }
            }
        }
        free(work);
        free(blk);
        free(Jt);
        free(Kt);
    }
    free(pi);
    free(pj);
    return err;
}

/* Overlap: multipole.py:48-135 with multipole_moment = (0,0,0): M^0_0 = sqrt(pi/p). */
int sqo_overlap(const sqo_basis *B, double *S) {
    const double pi = 3.141592653589793;
    const int n = B->nshell, nbf = B->nbf;
    double E[3][512];
    for (int s1 = 0; s1 < n; s1++)
        for (int s2 = 0; s2 <= s1; s2++) {
            const int l1 = shell_lmax(B, s1), l2 = shell_lmax(B, s2);
            const int np1 = B->nprim[s1], np2 = B->nprim[s2], nb1 = B->ncart[s1], nb2 = B->ncart[s2];
            const int ej = l2 + 1, et = l1 + l2 + 1;
            for (int a = 0; a < nb1; a++)
                for (int b = 0; b < nb2; b++) {
                    const int *A1 = B->cart + 3 * (B->cart_off[s1] + a), *A2 = B->cart + 3 * (B->cart_off[s2] + b);
                    double s = 0.0;
                    for (int i = 0; i < np1; i++)
                        for (int j = 0; j < np2; j++) {
                            const double e1 = B->exps[B->prim_off[s1] + i], e2 = B->exps[B->prim_off[s2] + j];
                            for (int d = 0; d < 3; d++)
                                sqo_expansion_coefficients(B->center[3 * s1 + d], B->center[3 * s2 + d], e1, e2, l1, l2,
                                                           E[d]);
                            const double p = e1 + e2, M = pow(pi / p, 0.5);
                            double prim = M * M * M;
                            for (int d = 0; d < 3; d++) prim *= E[d][(A1[d] * ej + A2[d]) * et + 0];
                            prim *= B->norm[B->norm_off[s1] + a * np1 + i] * B->norm[B->norm_off[s2] + b * np2 + j];
                            s += B->coefs[B->prim_off[s1] + i] * B->coefs[B->prim_off[s2] + j] * prim;
                        }
                    const int r = B->bf_off[s1] + a, c = B->bf_off[s2] + b;
                    S[r * nbf + c] = s;
                    S[c * nbf + r] = s;
                }
        }
    return 0;
}

/* kineticenergy.py:42-133 (E tables built with l+2 on both shells). */
int sqo_kinetic(const sqo_basis *B, double *T) {
    const double pi = 3.141592653589793;
    const int n = B->nshell, nbf = B->nbf;
    double E[3][512];
    for (int s1 = 0; s1 < n; s1++)
        for (int s2 = 0; s2 <= s1; s2++) {
            const int l1 = shell_lmax(B, s1) + 2, l2 = shell_lmax(B, s2) + 2;
            const int np1 = B->nprim[s1], np2 = B->nprim[s2], nb1 = B->ncart[s1], nb2 = B->ncart[s2];
            const int ej = l2 + 1, et = l1 + l2 + 1;
#define EE(d, x, y) E[d][((x) * ej + (y)) * et + 0]
            for (int a = 0; a < nb1; a++)
                for (int b = 0; b < nb2; b++) {
                    const int *A1 = B->cart + 3 * (B->cart_off[s1] + a), *A2 = B->cart + 3 * (B->cart_off[s2] + b);
                    double s = 0.0;
                    for (int i = 0; i < np1; i++)
                        for (int j = 0; j < np2; j++) {
                            const double e1 = B->exps[B->prim_off[s1] + i], e2 = B->exps[B->prim_off[s2] + j];
                            for (int d = 0; d < 3; d++)
                                sqo_expansion_coefficients(B->center[3 * s1 + d], B->center[3 * s2 + d], e1, e2, l1, l2,
                                                           E[d]);
                            double D2[3];
                            for (int d = 0; d < 3; d++) {
                                const int x1 = A1[d], x2 = A2[d];
                                D2[d] = 4 * e1 * e1 * EE(d, x1 + 2, x2) - 2 * e1 * (2 * x1 + 1) * EE(d, x1, x2) +
                                        (x1 >= 2 ? x1 * (x1 - 1) * EE(d, x1 - 2, x2) : 0.0);
                            }
                            double prim = D2[0] * EE(1, A1[1], A2[1]) * EE(2, A1[2], A2[2]) +
                                          EE(0, A1[0], A2[0]) * D2[1] * EE(2, A1[2], A2[2]) +
                                          EE(0, A1[0], A2[0]) * EE(1, A1[1], A2[1]) * D2[2];
                            prim *= B->norm[B->norm_off[s1] + a * np1 + i] * B->norm[B->norm_off[s2] + b * np2 + j];
                            const double p = e1 + e2;
                            prim *= -1.0 / 2.0 * pow(pi / p, 3.0 / 2.0);
                            s += B->coefs[B->prim_off[s1] + i] * B->coefs[B->prim_off[s2] + j] * prim;
                        }
                    const int r = B->bf_off[s1] + a, c = B->bf_off[s2] + b;
                    T[r * nbf + c] = s;
                    T[c * nbf + r] = s;
                }
#undef EE
        }
    return 0;
}

/* nuclearattraction.py:47-135. */
int sqo_nuclear(const sqo_basis *B, int natom, const double *atom_xyz, const double *charges, double *Vn) {
    const double pi = 3.141592653589793;
    const int n = B->nshell, nbf = B->nbf;
    /* sized for shells up to f (l = 3): L = 6 */
    double E[3][512];
    double R[7 * 7 * 7], scratch[7 * 7 * 7 * 20];
    for (int s1 = 0; s1 < n; s1++)
        for (int s2 = 0; s2 <= s1; s2++) {
            const int l1 = shell_lmax(B, s1), l2 = shell_lmax(B, s2), L = l1 + l2;
            const int np1 = B->nprim[s1], np2 = B->nprim[s2], nb1 = B->ncart[s1], nb2 = B->ncart[s2];
            const int ej = l2 + 1, et = l1 + l2 + 1, LT = L + 1;
            double blk[100];
            memset(blk, 0, sizeof(blk));
            for (int i = 0; i < np1; i++)
                for (int j = 0; j < np2; j++) {
                    const double e1 = B->exps[B->prim_off[s1] + i], e2 = B->exps[B->prim_off[s2] + j];
                    for (int d = 0; d < 3; d++)
                        sqo_expansion_coefficients(B->center[3 * s1 + d], B->center[3 * s2 + d], e1, e2, l1, l2, E[d]);
                    const double p = e1 + e2;
                    double P[3];
                    for (int d = 0; d < 3; d++) P[d] = (e1 * B->center[3 * s1 + d] + e2 * B->center[3 * s2 + d]) / p;
                    double prim[100];
                    memset(prim, 0, sizeof(prim));
                    for (int at = 0; at < natom; at++) {
                        double PC[3];
                        for (int d = 0; d < 3; d++) PC[d] = P[d] - atom_xyz[3 * at + d];
                        hermite_coulomb(L, L, L, p, PC, R, scratch, 1);
                        for (int a = 0; a < nb1; a++) {
                            const int *A1 = B->cart + 3 * (B->cart_off[s1] + a);
                            const double tmp = B->norm[B->norm_off[s1] + a * np1 + i] * charges[at];
                            for (int b = 0; b < nb2; b++) {
                                const int *A2 = B->cart + 3 * (B->cart_off[s2] + b);
                                double acc = 0.0;
                                for (int t = 0; t <= A1[0] + A2[0]; t++)
                                    for (int u = 0; u <= A1[1] + A2[1]; u++)
                                        for (int v = 0; v <= A1[2] + A2[2]; v++)
                                            acc += E[0][(A1[0] * ej + A2[0]) * et + t] * E[1][(A1[1] * ej + A2[1]) * et + u] *
                                                   E[2][(A1[2] * ej + A2[2]) * et + v] * R[(t * LT + u) * LT + v];
                                prim[a * nb2 + b] += tmp * B->norm[B->norm_off[s2] + b * np2 + j] * acc;
                            }
                        }
                    }
                    const double cc = B->coefs[B->prim_off[s1] + i] * B->coefs[B->prim_off[s2] + j];
                    for (int x = 0; x < nb1 * nb2; x++) blk[x] += cc * prim[x] * (-2 * pi / p);
                }
            for (int a = 0; a < nb1; a++)
                for (int b = 0; b < nb2; b++) {
                    const int r = B->bf_off[s1] + a, c = B->bf_off[s2] + b;
                    Vn[r * nbf + c] = blk[a * nb2 + b];
                    Vn[c * nbf + r] = blk[a * nb2 + b];
                }
        }
    return 0;
}

int sqo_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
