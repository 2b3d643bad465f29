// sq_common.cuh -- shared definitions for the SlowQuant GB300 integral kernels.
//
// Cartesian component order, per shell of angular momentum l, follows the
// reference basis reader (slowquant/molecule/basis_reader.py:50-70):
// x-power from l down to 0, then y-power from l-x down to 0, z = l-x-y.
// d: xx xy xz yy yz zz;  f: xxx xxy xxz xyy xyz xzz yyy yyz yzz zzz.
#pragma once

#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/slowquant_gb300.h"

#define SQ_LMAX 2            // highest shell angular momentum of the per-thread, warp and gradient
                             // kernels; classes with f shells (up to SQ_MAX_L) run on eri_block.cu

namespace sq {

__host__ __device__ constexpr int ncart(int l) { return (l + 1) * (l + 2) / 2; }

// Cartesian powers of component c of a shell with angular momentum l.
__host__ __device__ constexpr int cart_x(int l, int c) {
    int idx = 0;
    for (int x = l; x >= 0; --x)
        for (int y = l - x; y >= 0; --y) {
            if (idx == c) return x;
            ++idx;
        }
    return -1;
}
__host__ __device__ constexpr int cart_y(int l, int c) {
    int idx = 0;
    for (int x = l; x >= 0; --x)
        for (int y = l - x; y >= 0; --y) {
            if (idx == c) return y;
            ++idx;
        }
    return -1;
}
__host__ __device__ constexpr int cart_z(int l, int c) { return l - cart_x(l, c) - cart_y(l, c); }

// Pair class index for la >= lb: (0,0)=0 (1,0)=1 (1,1)=2 (2,0)=3 (2,1)=4 (2,2)=5 (3,0)=6 ...
__host__ __device__ constexpr int pair_class(int la, int lb) { return la * (la + 1) / 2 + lb; }

// Number of Hermite terms of one Cartesian component pair: prod_d (a_d + b_d + 1).
__host__ __device__ constexpr int herm_terms(int la, int a, int lb, int b) {
    return (cart_x(la, a) + cart_x(lb, b) + 1) * (cart_y(la, a) + cart_y(lb, b) + 1) *
           (cart_z(la, a) + cart_z(lb, b) + 1);
}

// Offset of component pair (a, b) inside the Hermite-expanded E block of one
// primitive pair of class (la, lb); components ordered a-major.
__host__ __device__ constexpr int herm_offset(int la, int lb, int a, int b) {
    int off = 0;
    for (int aa = 0; aa < ncart(la); ++aa)
        for (int bb = 0; bb < ncart(lb); ++bb) {
            if (aa == a && bb == b) return off;
            off += herm_terms(la, aa, lb, bb);
        }
    return off;
}
// Size (values per primitive pair) of the Hermite-expanded E block of class (la, lb).
__host__ __device__ constexpr int herm_size(int la, int lb) { return herm_offset(la, lb, ncart(la), 0); }

// Number of Hermite functions with t+u+v <= L.
__host__ __device__ constexpr int nherm(int L) { return (L + 1) * (L + 2) * (L + 3) / 6; }

// Double factorial as used for the per-component normalisation:
// 1/sqrt((2x-1)!!(2y-1)!!(2z-1)!!) (moleculefunctions.py:29-47 factorised).
__host__ __device__ constexpr double dfact_odd(int n) {  // (2n-1)!!
    double r = 1.0;
    for (int k = 2 * n - 1; k > 0; k -= 2) r *= k;
    return r;
}

// Index of matrix element (bf_off[s]+a, bf_off[t]+b): the full nbf x nbf
// layout for one molecule, or the packed per-molecule block of a batch.
__device__ __forceinline__ long long mat_index(const sq_basis &bs, int s, int a, int t, int b) {
    const long long row = (long long)__ldg(bs.bf_off + s) + a, col = (long long)__ldg(bs.bf_off + t) + b;
    if (bs.mat_base == nullptr) return row * bs.nbf + col;
    return __ldg(bs.mat_base + s) + row * __ldg(bs.mat_ld + s) + col;
}

// Streaming multiprocessors of the current device, queried once per device;
// grid caps of the grid-stride kernels are expressed in waves of this.
inline long long sm_count() {
    static std::atomic<int> cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
    int n = cache[dev].load(std::memory_order_relaxed);
    if (n <= 0) {
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) return 1;
        cache[dev].store(n, std::memory_order_relaxed);
    }
    return n;
}

__host__ __device__ inline long long mat_total(const sq_basis &bs) {
    return bs.mat_base == nullptr ? (long long)bs.nbf * bs.nbf : bs.mat_total;
}

// f32 <-> f64 conversion with integer instructions.  On GB300 the hardware
// conversion runs at the FP64 rate (about 1/58 of FP32), so FP32 kernels that
// hand values to FP64 code convert on the integer pipe instead.  Valid for
// zero and normal numbers (float denormals flush to zero; no inf/NaN inputs).
__device__ __forceinline__ double f2d_bits(float x) {
    const unsigned u = __float_as_uint(x);
    const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
    const unsigned ex = (u >> 23) & 0xffu;
    const unsigned long long body = ((unsigned long long)(ex + 896u) << 52) | ((unsigned long long)(u & 0x7fffffu) << 29);
    return __longlong_as_double((long long)(ex == 0 ? sign : (sign | body)));
}

// Round-to-nearest-even f64 -> f32 (zero and the float normal range; smaller
// magnitudes flush to zero, larger ones and NaN become +-inf).
__device__ __forceinline__ float d2f_bits(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    const int ex = (int)((b >> 52) & 0x7ffu) - 896;
    unsigned long long mant = b & 0xfffffffffffffULL;
    mant += 0xfffffffULL + ((mant >> 29) & 1ULL);
    const unsigned e2 = (unsigned)(ex + (int)(mant >> 52));
    const unsigned m23 = (unsigned)((mant >> 29) & 0x7fffffu);
    if (ex <= 0) return __uint_as_float(sign);
    if (e2 >= 255u) return __uint_as_float(sign | 0x7f800000u);
    return __uint_as_float(sign | (e2 << 23) | m23);
}

// Index helpers of the runtime-class kernels (warp, block and gradient kernels).
//
// Flat Hermite index: degree n = t+u+v ascending, then t descending, then u descending.
__host__ __device__ __forceinline__ int herm_index(int t, int u, int v) {
    const int n = t + u + v;
    return n * (n + 1) * (n + 2) / 6 + (n - t) * (n - t + 1) / 2 + (n - t - u);
}

__device__ __forceinline__ void cart_powers(int l, int c, int &x, int &y, int &z) {
    int idx = 0;
    for (int xx = l; xx >= 0; --xx)
        for (int yy = l - xx; yy >= 0; --yy) {
            if (idx == c) {
                x = xx;
                y = yy;
                z = l - xx - yy;
                return;
            }
            ++idx;
        }
    x = y = z = 0;
}

__device__ __forceinline__ int herm_offset_rt(int la, int lb, int a, int b) {
    const int nb = ncart(lb);
    int off = 0;
    for (int aa = 0; aa < ncart(la); ++aa) {
        int ax, ay, az;
        cart_powers(la, aa, ax, ay, az);
        for (int bb = 0; bb < nb; ++bb) {
            if (aa == a && bb == b) return off;
            int bx, by, bz;
            cart_powers(lb, bb, bx, by, bz);
            off += (ax + bx + 1) * (ay + by + 1) * (az + bz + 1);
        }
    }
    return off;
}

}  // namespace sq
