// sq_common.cuh -- shared definitions for the SlowQuant GB300 integral kernels.
//
// Cartesian component order, per shell of angular momentum l, follows the
// reference basis reader (slowquant/molecule/basis_reader.py:50-70):
// x-power from l down to 0, then y-power from l-x down to 0, z = l-x-y.
// d: xx xy xz yy yz zz;  f: xxx xxy xxz xyy xyz xzz yyy yyz yzz zzz.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/slowquant_gb300.h"

#define SQ_LMAX 2            // highest shell angular momentum with compiled ERI kernels
#define SQ_NPAIRCLASS 6      // (SQ_LMAX+1)(SQ_LMAX+2)/2 pair classes (la >= lb)

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

}  // namespace sq
