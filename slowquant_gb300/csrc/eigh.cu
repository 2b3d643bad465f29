// eigh.cu -- batched symmetric eigensolver for the SCF of many small molecules.
//
// The SCF step diagonalises S^{-1/2}T F S^{-1/2} (hartreefock_in_memory.py:63-66,
// numpy eigh in the reference).  A batch of molecules needs hundreds of small
// FP64 diagonalisations per iteration; one CTA per matrix runs the cyclic
// Jacobi method (Golub & Van Loan, "Matrix Computations", sec. 8.5) with the
// round-robin ordering, so each step applies n/2 disjoint rotations in
// parallel: the matrix lives in shared memory (n <= 128), and so do the
// eigenvectors when both fit (n <= 118; else they are rotated in the output
// buffer).  Sweeps stop when the off-diagonal Frobenius norm is below tol *
// the matrix norm (or after max_sweeps).  Eigenvalues are returned in
// ascending order with their vectors as columns, like numpy/torch eigh.
#include <cstdint>

#include "capi_internal.cuh"

namespace sq {

constexpr int kEighMaxN = 128;
constexpr int kEighThreads = 256;
// dynamic shared memory allowed for A and V (static arrays below take ~6 KB of the 227 KB)
constexpr size_t kEighSmemBudget = 220 * 1024;

// Round-robin tournament: position k of step s holds player rr(s, k).
__device__ __forceinline__ int rr_player(int s, int k, int m) {
    // m even players; player m-1 stays fixed, the others rotate
    if (k == m - 1) return m - 1;
    return (k + s) % (m - 1);
}

__device__ __forceinline__ double block_sum(double v, double *s_red) {
    const int tid = threadIdx.x;
    s_red[tid] = v;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if (tid < st) s_red[tid] += s_red[tid + st];
        __syncthreads();
    }
    const double r = s_red[0];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kEighThreads) jacobi_eigh_kernel(const long long *off, const int *dim,
                                                                   const double *A_in, double *W, double *V,
                                                                   const long long *woff, double tol, int max_sweeps,
                                                                   int *sweeps_out, int max_n, int v_in_smem) {
    // shared: A (n x ld, ld = n | 1 so column walks do not hit one bank), then V
    // (same shape) when it fits; otherwise V is updated in the output buffer
    extern __shared__ __align__(16) double smem[];
    __shared__ double s_c[kEighMaxN / 2], s_s[kEighMaxN / 2];
    __shared__ int s_p[kEighMaxN / 2], s_q[kEighMaxN / 2];
    __shared__ double s_red[kEighThreads];
    __shared__ int s_rank[kEighMaxN];
    const int mi = blockIdx.x;
    const int n = dim[mi];
    if (n < 1 || n > max_n) {  // inconsistent description: leave this matrix untouched
        if (threadIdx.x == 0 && sweeps_out) sweeps_out[mi] = -1;
        return;
    }
    const int ld = n | 1;
    const int ldmax = max_n | 1;
    double *sA = smem;
    const long long base = off[mi];
    const double *A = A_in + base;
    double *Vout = V + base;
    double *sV = v_in_smem ? smem + (long long)max_n * ldmax : nullptr;
    double *Vm = v_in_smem ? sV : Vout;  // working eigenvector storage
    const int ldv = v_in_smem ? ld : n;
    const int tid = threadIdx.x;
    for (int x = tid; x < n * n; x += blockDim.x) {
        const int r = x / n, c = x % n;
        sA[r * ld + c] = A[x];
        Vm[r * ldv + c] = (r == c) ? 1.0 : 0.0;
    }
    __syncthreads();
    const int m = (n % 2 == 0) ? n : n + 1;  // players (one dummy if n is odd)
    const int npairs = m / 2;
    int sweep = 0;
    for (; sweep < max_sweeps; ++sweep) {
        // convergence test: off-diagonal vs total Frobenius norm
        double off2 = 0.0, tot2 = 0.0;
        for (int x = tid; x < n * n; x += blockDim.x) {
            const int r = x / n, c = x % n;
            const double v = sA[r * ld + c] * sA[r * ld + c];
            tot2 += v;
            if (r != c) off2 += v;
        }
        off2 = block_sum(off2, s_red);
        tot2 = block_sum(tot2, s_red);
        if (off2 <= tol * tol * tot2 || n < 2) break;
        for (int step = 0; step < m - 1; ++step) {
            // rotation angle of each pair (symmetric Schur 2x2)
            for (int k = tid; k < npairs; k += blockDim.x) {
                int p = rr_player(step, k, m), q = rr_player(step, m - 1 - k, m);
                if (p > q) {
                    const int t = p;
                    p = q;
                    q = t;
                }
                double c = 1.0, s = 0.0;
                if (q < n) {
                    const double apq = sA[p * ld + q];
                    if (apq != 0.0) {
                        const double theta = (sA[q * ld + q] - sA[p * ld + p]) / (2.0 * apq);
                        const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                        c = 1.0 / sqrt(t * t + 1.0);
                        s = t * c;
                    }
                }
                s_p[k] = p;
                s_q[k] = q;
                s_c[k] = c;
                s_s[k] = s;
            }
            __syncthreads();
            // rows: A <- J^T A  (rows p, q of every pair)
            for (int x = tid; x < npairs * n; x += blockDim.x) {
                const int k = x / n, j = x % n;
                const int p = s_p[k], q = s_q[k];
                if (q >= n) continue;
                const double c = s_c[k], s = s_s[k];
                const double ap = sA[p * ld + j], aq = sA[q * ld + j];
                sA[p * ld + j] = c * ap - s * aq;
                sA[q * ld + j] = s * ap + c * aq;
            }
            __syncthreads();
            // columns: A <- A J, V <- V J
            for (int x = tid; x < npairs * n; x += blockDim.x) {
                const int k = x / n, i = x % n;
                const int p = s_p[k], q = s_q[k];
                if (q >= n) continue;
                const double c = s_c[k], s = s_s[k];
                const double ap = sA[i * ld + p], aq = sA[i * ld + q];
                sA[i * ld + p] = c * ap - s * aq;
                sA[i * ld + q] = s * ap + c * aq;
                const double vp = Vm[i * ldv + p], vq = Vm[i * ldv + q];
                Vm[i * ldv + p] = c * vp - s * vq;
                Vm[i * ldv + q] = s * vp + c * vq;
            }
            __syncthreads();
        }
    }
    // ascending order: rank of each eigenvalue (ties by index), then write the
    // eigenvector columns into place
    double *w = W + woff[mi];
    for (int i = tid; i < n; i += blockDim.x) {
        const double di = sA[i * ld + i];
        int rank = 0;
        for (int j = 0; j < n; ++j) {
            const double dj = sA[j * ld + j];
            rank += (dj < di) || (dj == di && j < i);
        }
        w[rank] = di;
        s_rank[i] = rank;
    }
    __syncthreads();
    // stage V in the (now free) A storage, then scatter the permuted columns
    for (int x = tid; x < n * n; x += blockDim.x) {
        const int r = x / n, c = x % n;
        sA[r * ld + c] = Vm[r * ldv + c];
    }
    __syncthreads();
    for (int x = tid; x < n * n; x += blockDim.x) {
        const int r = x / n, c = x % n;
        Vout[r * n + s_rank[c]] = sA[r * ld + c];
    }
    if (tid == 0 && sweeps_out) sweeps_out[mi] = sweep;
}

}  // namespace sq

extern "C" int sq_batched_eigh(int nmat, const long long *offsets, const int *dims, int max_dim, const double *A,
                               double *W, double *V, const long long *w_offsets, double tol, int max_sweeps,
                               int *sweeps, void *stream) {
    if (nmat < 0 || !offsets || !dims || !A || !W || !V || !w_offsets)
        return sq::set_error(SQ_ERR_ARG, "sq_batched_eigh: bad argument");
    if (max_dim > sq::kEighMaxN || max_dim < 1)
        return sq::set_error(SQ_ERR_ARG, "sq_batched_eigh: matrix dimension %d outside 1..%d", max_dim, sq::kEighMaxN);
    if (max_sweeps < 0) return sq::set_error(SQ_ERR_ARG, "sq_batched_eigh: max_sweeps < 0");
    if (nmat == 0) return SQ_OK;
    // A in shared memory; V too when both fit (n up to 118), else V works in place in the output
    const size_t one = (size_t)max_dim * (max_dim | 1) * sizeof(double);
    const int v_in_smem = 2 * one <= sq::kEighSmemBudget ? 1 : 0;
    const size_t smem = v_in_smem ? 2 * one : one;
    cudaError_t e = cudaFuncSetAttribute(sq::jacobi_eigh_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return sq::set_error(SQ_ERR_CUDA, "sq_batched_eigh: %s", cudaGetErrorString(e));
    sq::jacobi_eigh_kernel<<<nmat, sq::kEighThreads, smem, (cudaStream_t)stream>>>(
        offsets, dims, A, W, V, w_offsets, tol, max_sweeps, sweeps, max_dim, v_in_smem);
    return sq::check_launch("sq_batched_eigh");
}
