// eri_block.cu -- block-cooperative McMurchie-Davidson kernel for the shell
// quartet classes with f shells (SQ_MAX_L = 3, L = la+lb+lc+ld up to 12).
//
// The classes with s, p and d shells only (0-20) keep their per-thread and
// per-warp kernels.  An f class has up to 10^4 integrals per contracted
// quartet ((ff|ff)), too many for registers, so here one CTA owns one
// contracted quartet at a time and keeps everything in shared memory:
//   * threads m <= L evaluate F_m(T) (tabulated high-order grid for J/K
//     launches, the reference's own piecewise formula for dense-tensor and
//     Schwarz launches), scaled by pref (-2 alpha)^m;
//   * the Hermite Coulomb recurrences (integralfunctions.py:100-148) run level
//     by level, the entries of one level spread over the CTA;
//   * ket transform W[cd][h] += sum (-1)^{tau+nu+phi} E^{cd}_{tau nu phi} R[h + (tau,nu,phi)]
//     per ket primitive pair, bra transform acc[ab][cd] += sum_h E^{ab}_h W[cd][h]
//     per bra primitive pair, threads owning output entries;
//   * the epilogue writes the dense tensor (8-fold scatter, electronrepulsion.py:80-104),
//     the Schwarz factor sqrt(max (ij|ij)) (electronrepulsion.py:300-339), or
//     contracts the block with the density in shared memory and issues one
//     atomic per J/K element, like the warp kernel.
// The arithmetic per primitive quartet is that of electron_repulsion_integral
// (electronrepulsion.py:107-297) with the R table limited to t+u+v <= L.
// FP32 J/K launches (SQ_FP32, SQ_FP32_BOYS32) run the integral arithmetic in
// FP32 and the Boys function in FP64 for these classes.
#include "boys.cuh"
#include "capi_internal.cuh"
#include "eri.cuh"

namespace sq {

constexpr int kBlkLmax = 4 * SQ_MAX_L;                       // 12
constexpr int kBlkHmax = nherm(kBlkLmax);                    // 455 Hermite entries
constexpr int kBlkPair = ncart(SQ_MAX_L) * ncart(SQ_MAX_L);  // 100 component pairs
constexpr int kBlkThreadsMax = 256;

struct BlockClass {
    int la, lb, lc, ld;
};

// Shared-memory layout of one class, byte offsets (each 16-byte aligned).
struct BlockLayout {
    int off_F, off_r0, off_r1, off_W, off_acc, off_epi, total;
};

__host__ __device__ constexpr int align16(int x) { return (x + 15) / 16 * 16; }

template <typename R>
__host__ __device__ inline BlockLayout block_layout(int la, int lb, int lc, int ld, int mode) {
    const int NA = ncart(la), NB = ncart(lb), NC = ncart(lc), ND = ncart(ld);
    const int HL = nherm(la + lb + lc + ld), HAB = nherm(la + lb);
    const int NW = HAB * NC * ND, NACC = NA * NB * NC * ND;
    BlockLayout b{};
    b.off_F = 0;
    b.off_r0 = align16(b.off_F + 16 * (int)sizeof(R));
    b.off_r1 = align16(b.off_r0 + HL * (int)sizeof(R));
    b.off_W = align16(b.off_r1 + HL * (int)sizeof(R));
    b.off_acc = align16(b.off_W + NW * (int)sizeof(R));
    b.off_epi = align16(b.off_acc + NACC * (int)sizeof(R));
    int epi = 0;
    if (mode == MODE_JK) {
        // FP64 copy of the block (FP32 launches) and the six density blocks
        epi = (sizeof(R) == sizeof(double) ? 0 : NACC) + NA * NB + NC * ND + NA * NC + NB * ND + NA * ND + NB * NC;
    }
    b.total = align16(b.off_epi + epi * (int)sizeof(double));
    return b;
}

template <typename R, int BOYS, int MODE>
__global__ void __launch_bounds__(kBlkThreadsMax) eri_block_kernel(const EriArgs args, const BlockClass cls) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_tuv[kBlkHmax];
    __shared__ int s_hoff_b[kBlkPair], s_hoff_k[kBlkPair];
    __shared__ int s_pw_b[kBlkPair], s_pw_k[kBlkPair];  // packed (ax+bx, ay+by, az+bz)
    __shared__ double s_red[kBlkThreadsMax / 32];

    const int tid = threadIdx.x, nt = blockDim.x;
    const int la = cls.la, lb = cls.lb, lc = cls.lc, ld = cls.ld;
    const int NA = ncart(la), NB = ncart(lb), NC = ncart(lc), ND = ncart(ld);
    const int NAB = NA * NB, NCD = NC * ND;
    const int LAB = la + lb, L = LAB + lc + ld;
    const int HAB = nherm(LAB), HL = nherm(L);
    const int EB = herm_offset_rt(la, lb, NA, 0), EK = herm_offset_rt(lc, ld, NC, 0);
    const int NW = HAB * NCD, NACC = NAB * NCD;
    const BlockLayout lay = block_layout<R>(la, lb, lc, ld, MODE);
    R *Fs = reinterpret_cast<R *>(smem_raw + lay.off_F);
    R *rb0 = reinterpret_cast<R *>(smem_raw + lay.off_r0);
    R *rb1 = reinterpret_cast<R *>(smem_raw + lay.off_r1);
    R *W = reinterpret_cast<R *>(smem_raw + lay.off_W);
    R *acc = reinterpret_cast<R *>(smem_raw + lay.off_acc);
    double *epi = reinterpret_cast<double *>(smem_raw + lay.off_epi);

    for (int e = tid; e < HL; e += nt) {
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
    for (int x = tid; x < NAB; x += nt) {
        const int a = x / NB, b = x % NB;
        s_hoff_b[x] = herm_offset_rt(la, lb, a, b);
        int ax, ay, az, bx, by, bz;
        cart_powers(la, a, ax, ay, az);
        cart_powers(lb, b, bx, by, bz);
        s_pw_b[x] = (ax + bx) | ((ay + by) << 8) | ((az + bz) << 16);
    }
    for (int x = tid; x < NCD; x += nt) {
        const int c = x / ND, d = x % ND;
        s_hoff_k[x] = herm_offset_rt(lc, ld, c, d);
        int cx, cy, cz, dx, dy, dz;
        cart_powers(lc, c, cx, cy, cz);
        cart_powers(ld, d, dx, dy, dz);
        s_pw_k[x] = (cx + dx) | ((cy + dy) << 8) | ((cz + dz) << 16);
    }
    __syncthreads();

    const sq_pairs &pr = args.pairs;
    const R *prim = prim_ptr<R>(pr);
    const R *herm = herm_ptr<R>(pr);

    for (long long qi = blockIdx.x; qi < args.nq; qi += gridDim.x) {
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
        for (int x = tid; x < NACC; x += nt) acc[x] = R(0);

        for (int i = ib0; i < ib1; ++i) {
            const R p = gload(prim + 8 * i + 0);
            const R Px = gload(prim + 8 * i + 1), Py = gload(prim + 8 * i + 2), Pz = gload(prim + 8 * i + 3);
            const R Ub = gload(prim + 8 * i + 4);
            // each thread zeroes and later accumulates the same W entries
            for (int w = tid; w < NW; w += nt) W[w] = R(0);
            for (int k = kb0; k < kb1; ++k) {
                const R q = gload(prim + 8 * k + 0);
                const R X = Px - gload(prim + 8 * k + 1);
                const R Y = Py - gload(prim + 8 * k + 2);
                const R Z = Pz - gload(prim + 8 * k + 3);
                const R Uk = gload(prim + 8 * k + 4);
                const R r = rsqrt_r(p + q);
                const R alpha = p * q * (r * r);
                const R T = alpha * (X * X + Y * Y + Z * Z);
                // thread m <= L: Fs[m] = pref (-2 alpha)^m F_m(T); thread L also
                // seeds the top level of the recurrence
                if (tid <= L) {
                    const int m = tid;
                    double f;
                    if constexpr (BOYS == BOYS_REF)
                        f = boys_reference(m, (double)T);
                    else
                        f = boys_hi(m, (double)T, args.tab64);
                    R fac = R(kTwoPi52) * Ub * Uk * r;
                    const R m2a = R(-2) * alpha;
                    for (int j = 0; j < m; ++j) fac *= m2a;
                    const R val = (R)f * fac;
                    Fs[m] = val;
                    if (m == L) rb0[0] = val;
                }
                __syncthreads();
                // Hermite recurrences, level L-1 down to 0
                R *cur = rb0, *nxt = rb1;
                for (int n = L - 1; n >= 0; --n) {
                    const int cnt = nherm(L - n);
                    for (int e = tid; e < cnt; e += nt) {
                        R val;
                        if (e == 0) {
                            val = Fs[n];
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
                    __syncthreads();
                    R *tmp = cur;
                    cur = nxt;
                    nxt = tmp;
                }
                // ket transform
                const R *ek = hk + (long long)(k - k0) * EK;
                for (int w = tid; w < NW; w += nt) {
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
                    W[w] += s;
                }
                // Fs, rb0 and the R table are rewritten by the next ket primitive
                __syncthreads();
            }
            // bra transform: threads own output entries x = ab * NCD + cd
            const R *eb = hb + (long long)(i - i0) * EB;
            for (int x = tid; x < NACC; x += nt) {
                const int ab = x / NCD, cd = x - ab * NCD;
                const int pw = s_pw_b[ab];
                const int ax = pw & 255, ay = (pw >> 8) & 255, az = pw >> 16;
                const R *e = eb + s_hoff_b[ab];
                R s = R(0);
                for (int t = 0; t <= ax; ++t)
                    for (int u = 0; u <= ay; ++u)
                        for (int v = 0; v <= az; ++v)
                            s = fma(gload(e + (t * (ay + 1) + u) * (az + 1) + v), W[herm_index(t, u, v) + HAB * cd], s);
                acc[x] += s;
            }
            // W is zeroed again for the next bra primitive
            __syncthreads();
        }

        // epilogue
        const int sa = gload(pr.shells + 2 * P), sb = gload(pr.shells + 2 * P + 1);
        const int sc = gload(pr.shells + 2 * Q), sd = gload(pr.shells + 2 * Q + 1);
        if constexpr (MODE == MODE_SCHWARZ) {
            double mx = -1e300;
            for (int x = tid; x < NACC; x += nt) mx = fmax(mx, (double)acc[x]);
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
            if ((tid & 31) == 0) s_red[tid >> 5] = mx;
            __syncthreads();
            if (tid == 0) {
                for (int w = 1; w < (nt >> 5); ++w) mx = fmax(mx, s_red[w]);
                args.q[P] = sqrt(mx);
            }
        } else if constexpr (MODE == MODE_JK) {
            double m = 8.0;
            if (sa == sb) m *= 0.5;
            if (sc == sd) m *= 0.5;
            if (P == Q) m *= 0.5;
            const double wJ = 0.5 * m, wK = 0.25 * m;
            const sq_basis &bs = args.basis;
            double *Vb;
            double *Dab;
            if constexpr (std::is_same<R, double>::value) {
                Vb = acc;
                Dab = epi;
            } else {
                Vb = epi;
                Dab = epi + NACC;
                for (int x = tid; x < NACC; x += nt) Vb[x] = (double)acc[x];
            }
            double *Dcd = Dab + NAB;        // [NC][ND]
            double *Dac = Dcd + NCD;        // [NA][NC]
            double *Dbd = Dac + NA * NC;    // [NB][ND]
            double *Dad = Dbd + NB * ND;    // [NA][ND]
            double *Dbc = Dad + NA * ND;    // [NB][NC]
            const int nd = args.nd > 1 ? args.nd : 1;
            const int nJ = NAB + NCD, nK = NA * NC + NB * ND + NA * ND + NB * NC;
            for (int di = 0; di < nd; ++di) {
                const double *D = args.D + di * args.dstride;
                double *J = args.Jacc + di * args.dstride, *K = args.Kacc + di * args.dstride;
                for (int x = tid; x < NAB; x += nt) Dab[x] = gload(D + mat_index(bs, sa, x / NB, sb, x % NB));
                for (int x = tid; x < NCD; x += nt) Dcd[x] = gload(D + mat_index(bs, sc, x / ND, sd, x % ND));
                for (int x = tid; x < NA * NC; x += nt) Dac[x] = gload(D + mat_index(bs, sa, x / NC, sc, x % NC));
                for (int x = tid; x < NB * ND; x += nt) Dbd[x] = gload(D + mat_index(bs, sb, x / ND, sd, x % ND));
                for (int x = tid; x < NA * ND; x += nt) Dad[x] = gload(D + mat_index(bs, sa, x / ND, sd, x % ND));
                for (int x = tid; x < NB * NC; x += nt) Dbc[x] = gload(D + mat_index(bs, sb, x / NC, sc, x % NC));
                __syncthreads();
                for (int o = tid; o < nJ + nK; o += nt) {
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
                __syncthreads();  // the density blocks are reloaded for the next density
            }
        } else {
            const long long n = args.basis.nbf;
            const int oa = gload(args.basis.bf_off + sa), ob = gload(args.basis.bf_off + sb);
            const int oc = gload(args.basis.bf_off + sc), od = gload(args.basis.bf_off + sd);
            double *V = args.V;
            for (int x = tid; x < NACC; x += nt) {
                const int ab = x / NCD, cd = x - ab * NCD;
                const long long A = oa + ab / NB, B = ob + ab % NB, C = oc + cd / ND, Dd = od + cd % ND;
                const double v = (double)acc[x];
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
        // acc and the epilogue scratch belong to the next quartet
        __syncthreads();
    }
}

// Threads per CTA from the larger of the two transform sizes.
static int block_threads(int la, int lb, int lc, int ld) {
    const int nw = nherm(la + lb) * ncart(lc) * ncart(ld);
    const int nacc = ncart(la) * ncart(lb) * ncart(lc) * ncart(ld);
    const int work = nw > nacc ? nw : nacc;
    if (work <= 64) return 32;
    if (work <= 256) return 64;
    if (work <= 1024) return 128;
    return kBlkThreadsMax;
}

template <typename R, int BOYS, int MODE>
static cudaError_t launch_block(const EriArgs &args, const BlockClass &cls, cudaStream_t stream) {
    const BlockLayout lay = block_layout<R>(cls.la, cls.lb, cls.lc, cls.ld, MODE);
    auto kern = eri_block_kernel<R, BOYS, MODE>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, lay.total);
    if (e != cudaSuccess) return e;
    const int threads = block_threads(cls.la, cls.lb, cls.lc, cls.ld);
    long long blocks = args.nq;
    if (blocks > sm_count() * 32) blocks = sm_count() * 32;
    kern<<<(unsigned)blocks, threads, lay.total, stream>>>(args, cls);
    return cudaGetLastError();
}

cudaError_t launch_eri_block(const EriArgs &args, int la, int lb, int lc, int ld, int mode, int precision,
                             cudaStream_t stream) {
    if (args.nq <= 0) return cudaSuccess;
    if (la > SQ_MAX_L || lb > SQ_MAX_L || lc > SQ_MAX_L || ld > SQ_MAX_L) return cudaErrorInvalidValue;
    const BlockClass cls{la, lb, lc, ld};
    // dense tensors and Schwarz factors are drop-in outputs: reference-compatible Boys
    if (mode == MODE_DENSE) return launch_block<double, BOYS_REF, MODE_DENSE>(args, cls, stream);
    if (mode == MODE_SCHWARZ) return launch_block<double, BOYS_REF, MODE_SCHWARZ>(args, cls, stream);
    if (precision == SQ_FP64) return launch_block<double, BOYS_FP64, MODE_JK>(args, cls, stream);
    return launch_block<float, BOYS_FP64, MODE_JK>(args, cls, stream);
}

}  // namespace sq
