// eri_warp.cuh -- generic warp-cooperative McMurchie-Davidson kernel for the
// high angular-momentum quartet classes (L = la+lb+lc+ld >= 5).
//
// One warp owns one contracted shell quartet at a time.  Per primitive quartet:
//   * lanes 0..L evaluate F_m(T) in parallel (one Taylor expansion each),
//     scaled by pref (-2 alpha)^m;
//   * the Hermite Coulomb recurrences (integralfunctions.py:100-148) run level
//     by level, the entries of one level spread over the lanes, in a
//     warp-private shared-memory buffer;
//   * the ket transform W[h][cd] += sum (-1)^{tau+nu+phi} E^{cd}_{tau nu phi}
//     R[h + (tau,nu,phi)] is spread over lanes by output entry (cd-major).
// Dense-tensor and Schwarz launches evaluate each F_m with the reference's own
// piecewise formula (boys_reference), J/K launches with the tabulated one.
// After the ket primitive loop the bra transform (ab|cd) += sum_h E^{ab}_h W[h][cd]
// runs with lanes owning output entries, accumulated in registers.  The
// arithmetic is that of the per-thread kernel (eri.cuh); the class is a
// runtime parameter, so one compiled kernel serves every class.
#pragma once

#include "boys.cuh"
#include "eri.cuh"

namespace sq {

constexpr int kWarpHmax = nherm(2 * SQ_LMAX * 2);          // Hermite table for L <= 4*lmax
constexpr int kWarpWmax = nherm(2 * SQ_LMAX) * ncart(SQ_LMAX) * ncart(SQ_LMAX);  // W entries
constexpr int kWarpAccMax = (ncart(SQ_LMAX) * ncart(SQ_LMAX) * ncart(SQ_LMAX) * ncart(SQ_LMAX) + 31) / 32;
constexpr int kWarpsPerBlock = 4;

struct WarpClass {
    int la, lb, lc, ld;
};

template <typename R>
struct WarpSmem {
    R rbuf[2][kWarpHmax];
    R W[kWarpWmax];
    R Fs[16];
};

// J/K epilogue scratch (FP64), overlaid on a warp's shared memory after its
// primitive loops: the integral block, then the six density blocks, each at
// the class's own size.  A warp's slice is the larger of the two uses, rounded
// to 16 bytes; kWarpEpi is the (dd|dd) need, which also covers the f classes
// that run here ((fp|dd): 1302 doubles).
constexpr int kWarpBlk = ncart(SQ_LMAX) * ncart(SQ_LMAX);
constexpr int kWarpEpi = kWarpBlk * kWarpBlk + 6 * kWarpBlk;
__host__ __device__ constexpr int warp_epi_size(int la, int lb, int lc, int ld) {
    return ncart(la) * ncart(lb) * ncart(lc) * ncart(ld) + ncart(la) * ncart(lb) + ncart(lc) * ncart(ld) +
           ncart(la) * ncart(lc) + ncart(lb) * ncart(ld) + ncart(la) * ncart(ld) + ncart(lb) * ncart(lc);
}
template <typename R>
__host__ __device__ constexpr size_t warp_stride() {
    return ((sizeof(WarpSmem<R>) > kWarpEpi * sizeof(double) ? sizeof(WarpSmem<R>) : kWarpEpi * sizeof(double)) +
            15) / 16 * 16;
}

// KACC: accumulator registers per lane (outputs / 32, rounded up to a bucket),
// so that the smaller classes do not carry the (dd|dd) register footprint.
template <typename R, int BOYS, int MODE, int KACC = kWarpAccMax>
__global__ void __launch_bounds__(32 * kWarpsPerBlock) eri_warp_kernel(const EriArgs args, const WarpClass cls) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    WarpSmem<R> &sm = *reinterpret_cast<WarpSmem<R> *>(smem_raw + warp * warp_stride<R>());
    // per-block tables: (t,u,v) of each flat Hermite index; E offsets of component pairs
    __shared__ int s_tuv[kWarpHmax];
    __shared__ short s_hoff_b[ncart(SQ_LMAX) * ncart(SQ_LMAX)];
    __shared__ short s_hoff_k[ncart(SQ_LMAX) * ncart(SQ_LMAX)];
    __shared__ int s_pw_b[ncart(SQ_LMAX) * ncart(SQ_LMAX)];  // packed (ax+bx, ay+by, az+bz)
    __shared__ int s_pw_k[ncart(SQ_LMAX) * ncart(SQ_LMAX)];

    const int la = cls.la, lb = cls.lb, lc = cls.lc, ld = cls.ld;
    const int NA = ncart(la), NB = ncart(lb), NC = ncart(lc), ND = ncart(ld);
    const int NAB = NA * NB, NCD = NC * ND;
    const int LAB = la + lb, L = LAB + lc + ld;
    const int HAB = nherm(LAB), HL = nherm(L);
    const int EB = herm_offset_rt(la, lb, NA, 0), EK = herm_offset_rt(lc, ld, NC, 0);
    const int NW = HAB * NCD, NACC = NAB * NCD;

    for (int e = threadIdx.x; e < HL; e += blockDim.x) {
        // invert herm_index
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
    for (int x = threadIdx.x; x < NAB; x += blockDim.x) {
        const int a = x / NB, b = x % NB;
        s_hoff_b[x] = (short)herm_offset_rt(la, lb, a, b);
        int ax, ay, az, bx, by, bz;
        cart_powers(la, a, ax, ay, az);
        cart_powers(lb, b, bx, by, bz);
        s_pw_b[x] = (ax + bx) | ((ay + by) << 8) | ((az + bz) << 16);
    }
    for (int x = threadIdx.x; x < NCD; x += blockDim.x) {
        const int c = x / ND, d = x % ND;
        s_hoff_k[x] = (short)herm_offset_rt(lc, ld, c, d);
        int cx, cy, cz, dx, dy, dz;
        cart_powers(lc, c, cx, cy, cz);
        cart_powers(ld, d, dx, dy, dz);
        s_pw_k[x] = (cx + dx) | ((cy + dy) << 8) | ((cz + dz) << 16);
    }
    __syncthreads();

    const sq_pairs &pr = args.pairs;
    const R *prim = prim_ptr<R>(pr);
    const R *herm = herm_ptr<R>(pr);
    const long long nwarps = (long long)gridDim.x * kWarpsPerBlock;
    const int kacc = (NACC + 31) >> 5;

    for (long long qi = (long long)blockIdx.x * kWarpsPerBlock + warp; qi < args.nq; qi += nwarps) {
        const int2 pq = args.quartets[qi];
        const int P = args.use_slots ? gload(args.slots.pair + pq.x) : pq.x;
        const int Q = args.use_slots ? gload(args.slots.pair + pq.y) : pq.y;
        const int i0 = gload(pr.pp_off + P), i1 = gload(pr.pp_off + P + 1);
        const int k0 = gload(pr.pp_off + Q), k1 = gload(pr.pp_off + Q + 1);
        // a sub-slot (chunk k of S) covers primitives [k np / S, (k+1) np / S) of its pair
        int ib0 = i0, ib1 = i1, kb0 = k0, kb1 = k1;
        if (args.use_slots && args.slots.sub) {
            const int code = gload(args.slots.sub + pq.x);
            if (code) {
                const int S = code & 0xffff, kc = code >> 16, np = i1 - i0;
                ib0 = i0 + (kc * np) / S;
                ib1 = i0 + ((kc + 1) * np) / S;
            }
            const int codek = gload(args.slots.sub + pq.y);
            if (codek) {
                const int S = codek & 0xffff, kc = codek >> 16, np = k1 - k0;
                kb0 = k0 + (kc * np) / S;
                kb1 = k0 + ((kc + 1) * np) / S;
            }
        }
        const R *hb = herm + gload(pr.herm_off + P);
        const R *hk = herm + gload(pr.herm_off + Q);
        R acc[KACC];
#pragma unroll
        for (int k = 0; k < KACC; ++k) acc[k] = R(0);

        for (int i = ib0; i < ib1; ++i) {
            const R p = gload(prim + 8 * i + 0);
            const R Px = gload(prim + 8 * i + 1), Py = gload(prim + 8 * i + 2), Pz = gload(prim + 8 * i + 3);
            const R Ub = gload(prim + 8 * i + 4);
            for (int w = lane; w < NW; w += 32) sm.W[w] = R(0);
            for (int k = kb0; k < kb1; ++k) {
                const R q = gload(prim + 8 * k + 0);
                const R X = Px - gload(prim + 8 * k + 1);
                const R Y = Py - gload(prim + 8 * k + 2);
                const R Z = Pz - gload(prim + 8 * k + 3);
                const R Uk = gload(prim + 8 * k + 4);
                const R r = rsqrt_r(p + q);
                const R alpha = p * q * (r * r);
                const R T = alpha * (X * X + Y * Y + Z * Z);
                // lane m <= L: Fs[m] = pref (-2 alpha)^m F_m(T)
                if (lane <= L) {
                    R Fm;
                    const int m = lane;
                    if constexpr (BOYS == BOYS_REF) {
                        Fm = (R)boys_reference(m, (double)T);
                    } else if constexpr (std::is_same<R, double>::value || BOYS == BOYS_FP64) {
                        const double Td = (double)T;
                        double f;
                        if (Td < SQ_BOYS_TMAX) {
                            const int kk = __double2int_rn(Td * SQ_BOYS_STEP_INV);
                            const double dd = Td - kk * (1.0 / SQ_BOYS_STEP_INV);
                            const double *row = args.tab64 + kk * SQ_BOYS_NCOL + m;
                            f = __ldg(row + kBoysTaylor64 - 1);
#pragma unroll
                            for (int j = kBoysTaylor64 - 1; j >= 1; --j) f = fma(f, -dd * (1.0 / j), __ldg(row + j - 1));
                        } else {
                            const double rr = rsqrt(Td);
                            f = kSqrtPiHalf * rr;
                            const double h = 0.5 * rr * rr;
                            for (int j = 0; j < m; ++j) f *= (2 * j + 1) * h;
                        }
                        Fm = (R)f;
                    } else {
                        float f;
                        if (T < (float)SQ_BOYS_TMAX) {
                            const int kk = __float2int_rn(T * (float)SQ_BOYS_STEP_INV);
                            const float dd = T - kk * (1.0f / SQ_BOYS_STEP_INV);
                            const float *row = args.tab32 + kk * SQ_BOYS_NCOL + m;
                            f = __ldg(row + kBoysTaylor32 - 1);
#pragma unroll
                            for (int j = kBoysTaylor32 - 1; j >= 1; --j) f = fmaf(f, -dd * (1.0f / j), __ldg(row + j - 1));
                        } else {
                            const float rr = rsqrtf(T);
                            f = (float)kSqrtPiHalf * rr;
                            const float h = 0.5f * rr * rr;
                            for (int j = 0; j < m; ++j) f *= (2 * j + 1) * h;
                        }
                        Fm = f;
                    }
                    // pref (-2 alpha)^m
                    R fac = R(kTwoPi52) * Ub * Uk * r;
                    const R m2a = R(-2) * alpha;
                    for (int j = 0; j < m; ++j) fac *= m2a;
                    sm.Fs[m] = Fm * fac;
                }
                __syncwarp();
                // Hermite recurrences, level L (top) down to 0
                R *cur = sm.rbuf[0], *nxt = sm.rbuf[1];
                if (lane == 0) cur[0] = sm.Fs[L];
                __syncwarp();
                for (int n = L - 1; n >= 0; --n) {
                    const int cnt = nherm(L - n);
                    for (int e = lane; e < cnt; e += 32) {
                        R val;
                        if (e == 0) {
                            val = sm.Fs[n];
                        } else {
                            const int tuv = s_tuv[e];
                            const int t = tuv & 255, u = (tuv >> 8) & 255, v = tuv >> 16;
                            if (t > 0) {
                                val = X * cur[herm_index(t - 1, u, v)];
                                if (t > 1) val = fma(R(t - 1), cur[herm_index(t - 2, u, v)], val);
                            } else if (u > 0) {
                                val = Y * cur[herm_index(0, u - 1, v)];
                                if (u > 1) val = fma(R(u - 1), cur[herm_index(0, u - 2, v)], val);
                            } else {
                                val = Z * cur[herm_index(0, 0, v - 1)];
                                if (v > 1) val = fma(R(v - 1), cur[herm_index(0, 0, v - 2)], val);
                            }
                        }
                        nxt[e] = val;
                    }
                    __syncwarp();
                    R *tmp = cur;
                    cur = nxt;
                    nxt = tmp;
                }
                // ket transform
                const R *ek = hk + (long long)(k - k0) * EK;
                for (int w = lane; w < NW; w += 32) {
                    const int cd = w / HAB, h = w - cd * HAB;
                    const int tuv = s_tuv[h];
                    const int t = tuv & 255, u = (tuv >> 8) & 255, v = tuv >> 16;
                    const int pw = s_pw_k[cd];
                    const int cx = pw & 255, cy = (pw >> 8) & 255, cz = pw >> 16;
                    const R *e = ek + s_hoff_k[cd];
                    R s = R(0);
                    for (int tau = 0; tau <= cx; ++tau)
                        for (int nu = 0; nu <= cy; ++nu)
                            for (int phi = 0; phi <= cz; ++phi) {
                                R ev = gload(e + (tau * (cy + 1) + nu) * (cz + 1) + phi);
                                if ((tau + nu + phi) & 1) ev = -ev;
                                s = fma(ev, cur[herm_index(t + tau, u + nu, v + phi)], s);
                            }
                    sm.W[w] += s;
                }
                __syncwarp();
            }
            // bra transform: lanes own output entries x = lane + 32 kk, x = ab * NCD + cd
            const R *eb = hb + (long long)(i - i0) * EB;
#pragma unroll
            for (int kk = 0; kk < KACC; ++kk) {
                if (kk < kacc) {
                    const int x = lane + 32 * kk;
                    if (x < NACC) {
                        const int ab = x / NCD, cd = x - ab * NCD;
                        const int pw = s_pw_b[ab];
                        const int ax = pw & 255, ay = (pw >> 8) & 255, az = pw >> 16;
                        const R *e = eb + s_hoff_b[ab];
                        R s = R(0);
                        for (int t = 0; t <= ax; ++t)
                            for (int u = 0; u <= ay; ++u)
                                for (int v = 0; v <= az; ++v)
                                    s = fma(gload(e + (t * (ay + 1) + u) * (az + 1) + v), sm.W[herm_index(t, u, v) + HAB * cd], s);
                        acc[kk] += s;
                    }
                }
            }
            __syncwarp();
        }

        // epilogue
        const int sa = gload(pr.shells + 2 * P), sb = gload(pr.shells + 2 * P + 1);
        const int sc = gload(pr.shells + 2 * Q), sd = gload(pr.shells + 2 * Q + 1);
        const long long n = args.basis.nbf;
        const int oa = gload(args.basis.bf_off + sa), ob = gload(args.basis.bf_off + sb);
        const int oc = gload(args.basis.bf_off + sc), od = gload(args.basis.bf_off + sd);
        if constexpr (MODE == MODE_SCHWARZ) {
            double mx = -1e300;
#pragma unroll
            for (int kk = 0; kk < KACC; ++kk)
                if (kk < kacc && lane + 32 * kk < NACC) mx = fmax(mx, (double)acc[kk]);
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
            if (lane == 0) args.q[P] = sqrt(mx);
        } else if constexpr (MODE == MODE_JK) {
            // J/K digestion in two steps, like the per-thread kernel: the warp
            // stages the integral block and the six density blocks in shared
            // memory, contracts them to the J and K blocks, and issues one atomic
            // per J/K block element (NAB + NCD + 4 mixed blocks) instead of six
            // per integral.
            double m = 8.0;
            if (sa == sb) m *= 0.5;
            if (sc == sd) m *= 0.5;
            if (P == Q) m *= 0.5;
            const double wJ = 0.5 * m, wK = 0.25 * m;
            const sq_basis &bs = args.basis;
            // packed at the class's own sizes (warp_epi_size <= kWarpEpi, checked at launch)
            double *ep = reinterpret_cast<double *>(&sm);
            double *Vb = ep;                 // [NAB][NCD]
            double *Dab = ep + NACC;         // [NA][NB]
            double *Dcd = Dab + NAB;         // [NC][ND]
            double *Dac = Dcd + NCD;         // [NA][NC]
            double *Dbd = Dac + NA * NC;     // [NB][ND]
            double *Dad = Dbd + NB * ND;     // [NA][ND]
            double *Dbc = Dad + NA * ND;     // [NB][NC]
            __syncwarp();
#pragma unroll
            for (int kk = 0; kk < KACC; ++kk)
                if (kk < kacc && lane + 32 * kk < NACC) Vb[lane + 32 * kk] = (double)acc[kk];
            const int nd = args.nd > 1 ? args.nd : 1;
            const int nJ = NAB + NCD, nK = NA * NC + NB * ND + NA * ND + NB * NC;
            for (int di = 0; di < nd; ++di) {
                const double *D = args.D + di * args.dstride;
                double *J = args.Jacc + di * args.dstride, *K = args.Kacc + di * args.dstride;
                for (int x = lane; x < NAB; x += 32) Dab[x] = gload(D + mat_index(bs, sa, x / NB, sb, x % NB));
                for (int x = lane; x < NCD; x += 32) Dcd[x] = gload(D + mat_index(bs, sc, x / ND, sd, x % ND));
                for (int x = lane; x < NA * NC; x += 32) Dac[x] = gload(D + mat_index(bs, sa, x / NC, sc, x % NC));
                for (int x = lane; x < NB * ND; x += 32) Dbd[x] = gload(D + mat_index(bs, sb, x / ND, sd, x % ND));
                for (int x = lane; x < NA * ND; x += 32) Dad[x] = gload(D + mat_index(bs, sa, x / ND, sd, x % ND));
                for (int x = lane; x < NB * NC; x += 32) Dbc[x] = gload(D + mat_index(bs, sb, x / NC, sc, x % NC));
                __syncwarp();
                for (int o = lane; o < nJ + nK; o += 32) {
                    double sum = 0.0;
                    long long dst;
                    double *T;
                    double w;
                    if (o < NAB) {  // J_ab = sum_cd (ab|cd) D_cd
                        for (int cd = 0; cd < NCD; ++cd) sum = fma(Vb[o * NCD + cd], Dcd[cd], sum);
                        dst = mat_index(bs, sa, o / NB, sb, o % NB);
                        T = J;
                        w = wJ;
                    } else if (o < nJ) {  // J_cd = sum_ab (ab|cd) D_ab
                        const int cd = o - NAB;
                        for (int ab = 0; ab < NAB; ++ab) sum = fma(Vb[ab * NCD + cd], Dab[ab], sum);
                        dst = mat_index(bs, sc, cd / ND, sd, cd % ND);
                        T = J;
                        w = wJ;
                    } else {
                        int r = o - nJ;
                        T = K;
                        w = wK;
                        if (r < NA * NC) {  // K_ac = sum_bd (ab|cd) D_bd
                            const int a = r / NC, c = r % NC;
                            for (int b = 0; b < NB; ++b)
                                for (int d = 0; d < ND; ++d)
                                    sum = fma(Vb[(a * NB + b) * NCD + c * ND + d], Dbd[b * ND + d], sum);
                            dst = mat_index(bs, sa, a, sc, c);
                        } else if ((r -= NA * NC) < NB * ND) {  // K_bd = sum_ac (ab|cd) D_ac
                            const int b = r / ND, d = r % ND;
                            for (int a = 0; a < NA; ++a)
                                for (int c = 0; c < NC; ++c)
                                    sum = fma(Vb[(a * NB + b) * NCD + c * ND + d], Dac[a * NC + c], sum);
                            dst = mat_index(bs, sb, b, sd, d);
                        } else if ((r -= NB * ND) < NA * ND) {  // K_ad = sum_bc (ab|cd) D_bc
                            const int a = r / ND, d = r % ND;
                            for (int b = 0; b < NB; ++b)
                                for (int c = 0; c < NC; ++c)
                                    sum = fma(Vb[(a * NB + b) * NCD + c * ND + d], Dbc[b * NC + c], sum);
                            dst = mat_index(bs, sa, a, sd, d);
                        } else {  // K_bc = sum_ad (ab|cd) D_ad
                            r -= NA * ND;
                            const int b = r / NC, c = r % NC;
                            for (int a = 0; a < NA; ++a)
                                for (int d = 0; d < ND; ++d)
                                    sum = fma(Vb[(a * NB + b) * NCD + c * ND + d], Dad[a * ND + d], sum);
                            dst = mat_index(bs, sb, b, sc, c);
                        }
                    }
                    atomicAdd(T + dst, w * sum);
                }
                __syncwarp();  // the density blocks are reloaded for the next density / quartet
            }
        } else {
#pragma unroll
            for (int kk = 0; kk < KACC; ++kk) {
                if (kk < kacc) {
                    const int x = lane + 32 * kk;
                    if (x < NACC) {
                        const int ab = x / NCD, cd = x - ab * NCD;
                        const long long A = oa + ab / NB, B = ob + ab % NB, C = oc + cd / ND, Dd = od + cd % ND;
                        const double v = (double)acc[kk];
                        if constexpr (MODE == MODE_DENSE) {
                            double *V = args.V;
                            V[((A * n + B) * n + C) * n + Dd] = v;
                            V[((B * n + A) * n + C) * n + Dd] = v;
                            V[((A * n + B) * n + Dd) * n + C] = v;
                            V[((B * n + A) * n + Dd) * n + C] = v;
                            V[((C * n + Dd) * n + A) * n + B] = v;
                            V[((Dd * n + C) * n + A) * n + B] = v;
                            V[((C * n + Dd) * n + B) * n + A] = v;
                            V[((Dd * n + C) * n + B) * n + A] = v;
                        }
                    }
                }
            }
        }
    }
}

template <typename R>
constexpr size_t warp_smem_bytes() {
    return warp_stride<R>() * kWarpsPerBlock;
}

inline cudaError_t launch_eri_warp(const EriArgs &args, const WarpClass &cls, int mode, int precision,
                                   cudaStream_t stream) {
    if (args.nq <= 0) return cudaSuccess;
    // the class must fit the per-warp tables (Hermite entries, W, accumulators, epilogue)
    const int nab = ncart(cls.la) * ncart(cls.lb), ncd = ncart(cls.lc) * ncart(cls.ld);
    const int L = cls.la + cls.lb + cls.lc + cls.ld;
    if (nab > kWarpBlk || ncd > kWarpBlk || L > 4 * SQ_LMAX || nherm(cls.la + cls.lb) * ncd > kWarpWmax ||
        warp_epi_size(cls.la, cls.lb, cls.lc, cls.ld) > kWarpEpi)
        return cudaErrorInvalidValue;
    long long blocks = (args.nq + kWarpsPerBlock - 1) / kWarpsPerBlock;
    const long long cap = args.cfg_threads > 0 ? args.cfg_blocks : sm_count() * 64;
    if (blocks > cap) blocks = cap;
    const dim3 grid((unsigned)blocks), block(32 * kWarpsPerBlock);
#define SQ_WARP_LAUNCH(R, B, M, K)                                                                              \
    do {                                                                                                        \
        auto kern = eri_warp_kernel<R, B, M, K>;                                                                \
        const size_t sz = warp_smem_bytes<R>();                                                                 \
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sz);       \
        if (e != cudaSuccess) return e;                                                                         \
        kern<<<grid, block, sz, stream>>>(args, cls);                                                           \
    } while (0)
    // Dense tensors and Schwarz factors are drop-in outputs: reference-compatible Boys.
    const int kacc = (ncart(cls.la) * ncart(cls.lb) * ncart(cls.lc) * ncart(cls.ld) + 31) / 32;
    if (mode == MODE_DENSE)
        SQ_WARP_LAUNCH(double, BOYS_REF, MODE_DENSE, kWarpAccMax);
    else if (mode == MODE_SCHWARZ)
        SQ_WARP_LAUNCH(double, BOYS_REF, MODE_SCHWARZ, kWarpAccMax);
    else if (precision == SQ_FP64) {
        // the FP64 J/K launches carry the Fock build's large-bound high-L quartets
        if (kacc <= 2)
            SQ_WARP_LAUNCH(double, BOYS_FP64, MODE_JK, 2);
        else if (kacc <= 8)
            SQ_WARP_LAUNCH(double, BOYS_FP64, MODE_JK, 8);
        else if (kacc <= 16)
            SQ_WARP_LAUNCH(double, BOYS_FP64, MODE_JK, 16);
        else
            SQ_WARP_LAUNCH(double, BOYS_FP64, MODE_JK, kWarpAccMax);
    } else if (precision == SQ_FP32)
        SQ_WARP_LAUNCH(float, BOYS_FP64, MODE_JK, kWarpAccMax);
    else
        SQ_WARP_LAUNCH(float, BOYS_FP32, MODE_JK, kWarpAccMax);
#undef SQ_WARP_LAUNCH
    return cudaGetLastError();
}

}  // namespace sq
