// jk_dense.cu -- J and K from a stored ERI tensor, the two einsums of
// slowquant/hartreefock/hartreefock_in_memory.py:55-56:
//   J[p][q] = sum_rs V[p][q][r][s] D[s][r],   K[p][q] = sum_rs V[p][s][q][r] D[s][r].
// Both read the same n^3 block V[p] for a given p:
//   J[p][q] = sum_{r,s} V[p][q][r][s] D^T[r][s],  K[p][q] = sum_{s,r} V[p][s][q][r] D[s][r],
// so one block per (p, slice of the block) streams V[p] from HBM once and
// produces both rows.  Thread t of a block reads consecutive elements (the
// last index fastest), so the V stream is coalesced; D (n^2 doubles) is
// staged in shared memory when it fits in 96 KB (n <= 110), otherwise read
// through L1/L2.  The K pass re-reads the row just streamed from L2.
// HBM-bound: 8 n^4 bytes per build.
#include "capi_internal.cuh"
#include "sq_common.cuh"

namespace sq {

constexpr int kJkDenseThreads = 256;

// grid (n, nsplit): block (p, y) covers rows a = y, y + nsplit, ... of the
// n x n^2 matrix V[p][a][:] (a = q for J, a = s for K).
__global__ void __launch_bounds__(kJkDenseThreads) jk_dense_kernel(int n, const double *__restrict__ V,
                                                                   const double *__restrict__ D, double *__restrict__ J,
                                                                   double *__restrict__ K, int use_smem) {
    extern __shared__ double sD[];
    const long long nn = (long long)n * n;
    const int p = blockIdx.x;
    if (use_smem) {
        for (long long x = threadIdx.x; x < nn; x += blockDim.x) sD[x] = __ldg(D + x);
        __syncthreads();
    }
    const double *Dp = use_smem ? sD : D;
    const double *Vp = V + (long long)p * n * nn;
    // J[p][a] = sum_{r,s} V[p][a][r][s] D[s][r]:   row a, element (r, s) pairs with D[s][r]
    // K[p][q] += sum_{r} V[p][a][q][r] D[a][r]:    row a (= s), element (q, r) feeds K[p][q]
    for (int a = blockIdx.y; a < n; a += gridDim.y) {
        const double *row = Vp + (long long)a * nn;
        double jsum = 0.0;
        for (long long x = threadIdx.x; x < nn; x += blockDim.x) {
            const int r = (int)(x / n), s = (int)(x - (long long)r * n);
            const double v = __ldg(row + x);
            jsum = fma(v, Dp[(long long)s * n + r], jsum);
        }
        // block reduction of jsum
        for (int off = 16; off > 0; off >>= 1) jsum += __shfl_xor_sync(0xffffffffu, jsum, off);
        __shared__ double red[kJkDenseThreads / 32];
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = jsum;
        __syncthreads();
        if (threadIdx.x < 32) {
            double v = threadIdx.x < kJkDenseThreads / 32 ? red[threadIdx.x] : 0.0;
            for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
            if (threadIdx.x == 0) J[(long long)p * n + a] = v;
        }
        __syncthreads();
        // K: element (q, r) of row a contributes V[p][a][q][r] D[a][r] to K[p][q]; a thread
        // owns q values and sums over r (the row is read again, now from L2 / L1)
        for (int q = threadIdx.x; q < n; q += blockDim.x) {
            const double *vr = row + (long long)q * n;
            const double *da = Dp + (long long)a * n;
            double ks = 0.0;
            for (int r = 0; r < n; ++r) ks = fma(__ldg(vr + r), da[r], ks);
            atomicAdd(K + (long long)p * n + q, ks);
        }
    }
}

}  // namespace sq

using namespace sq;

extern "C" int sq_jk_dense(int nbf, const double *V, const double *D, double *J, double *K, void *stream) {
    if (nbf < 0) return set_error(SQ_ERR_ARG, "sq_jk_dense: negative nbf");
    if (nbf == 0) return SQ_OK;
    if (!V || !D || !J || !K) return set_error(SQ_ERR_ARG, "sq_jk_dense: NULL pointer");
    const long long nn = (long long)nbf * nbf;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(K, 0, nn * sizeof(double), s);
    if (e != cudaSuccess) return set_error(SQ_ERR_CUDA, "sq_jk_dense: %s", cudaGetErrorString(e));
    const size_t smem = nn * sizeof(double);
    const int use_smem = smem <= 96 * 1024;
    if (use_smem) {
        e = cudaFuncSetAttribute(jk_dense_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return set_error(SQ_ERR_CUDA, "sq_jk_dense: %s", cudaGetErrorString(e));
    }
    // enough blocks to fill the GPU: n rows of p times a split of the a-rows
    int split = (int)((4LL * sm_count() + nbf - 1) / nbf);
    if (split > nbf) split = nbf;
    if (split < 1) split = 1;
    jk_dense_kernel<<<dim3((unsigned)nbf, (unsigned)split), kJkDenseThreads, use_smem ? smem : 0, s>>>(nbf, V, D, J, K,
                                                                                                  use_smem);
    return check_launch("sq_jk_dense");
}
