// ao2mo.cu -- AO -> MO integral transformation (slowquant/molecularintegrals/
// integralfunctions.py:186-211) as repeated "transform the last index and
// move it to the front" passes:
//   out[l][r] = sum_{d < n} G[r][d] C[d][l],   r < rows, l < m,
// with G a rows x n row-major array and C the n x m MO coefficients.  Four
// passes turn g[a][b][c][d] into g[i][j][k][l], two turn h[a][b] into h[i][j];
// writing the transformed index first makes the permutation free.
//
// FP64 register-tiled GEMM: a block computes a 64-row x 64-column tile with
// 256 threads, 4 x 4 outputs each; the K dimension (n) is staged 16 at a time
// through shared memory.  Rows are the fastest thread index so that the
// transposed stores of a warp cover 16 consecutive rows of two output columns
// (two 128-byte segments).  The kernel is FP64-pipe bound (2 n FLOPs per
// output against 8 bytes).
#include "capi_internal.cuh"
#include "sq_common.cuh"

namespace sq {

constexpr int kTileR = 64, kTileL = 64, kTileK = 16;

__global__ void __launch_bounds__(256) ao2mo_rotate_kernel(long long rows, int n, int m, const double *__restrict__ G,
                                                         const double *__restrict__ C, double *__restrict__ out) {
    __shared__ double sG[kTileK][kTileR + 1];  // [k][row]: rows contiguous for the compute reads
    __shared__ double sC[kTileK][kTileL];
    const int tid = threadIdx.x;
    const int tr = tid & 15, tl = tid >> 4;  // 16 x 16 threads
    const long long r0 = (long long)blockIdx.x * kTileR;
    const int l0 = blockIdx.y * kTileL;
    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;

    for (int k0 = 0; k0 < n; k0 += kTileK) {
        // G tile: 64 rows x 16 k, read along k (contiguous in G): thread t loads
        // row t / 4, k-quarter t % 4 (4 consecutive doubles)
        {
            const int row = tid >> 2, kq = (tid & 3) * 4;
            const long long r = r0 + row;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int k = k0 + kq + q;
                sG[kq + q][row] = (r < rows && k < n) ? __ldg(G + r * n + k) : 0.0;
            }
        }
        // C tile: 16 k x 64 l, read along l
        {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int e = tid + 256 * q;
                const int k = e >> 6, l = e & 63;
                sC[k][l] = (k0 + k < n && l0 + l < m) ? __ldg(C + (long long)(k0 + k) * m + l0 + l) : 0.0;
            }
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kTileK; ++kk) {
            double a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = sG[kk][tr + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = sC[kk][tl + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int l = l0 + tl + 16 * j;
        if (l >= m) continue;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const long long r = r0 + tr + 16 * i;
            if (r < rows) out[(long long)l * rows + r] = acc[i][j];
        }
    }
}

}  // namespace sq

using namespace sq;

extern "C" int sq_ao2mo_rotate(long long rows, int n, int m, const double *G, const double *C, double *out,
                               void *stream) {
    if (rows < 0 || n < 0 || m < 0) return set_error(SQ_ERR_ARG, "sq_ao2mo_rotate: negative size");
    if (rows == 0 || m == 0) return SQ_OK;
    if (!G || !C || !out) return set_error(SQ_ERR_ARG, "sq_ao2mo_rotate: NULL pointer");
    if (G == out) return set_error(SQ_ERR_ARG, "sq_ao2mo_rotate: out must not alias G");
    const long long gx = (rows + kTileR - 1) / kTileR;
    const int gy = (m + kTileL - 1) / kTileL;
    if (gx > 0x7fffffffLL || gy > 65535) return set_error(SQ_ERR_ARG, "sq_ao2mo_rotate: problem too large");
    ao2mo_rotate_kernel<<<dim3((unsigned)gx, (unsigned)gy), 256, 0, (cudaStream_t)stream>>>(rows, n, m, G, C, out);
    return check_launch("sq_ao2mo_rotate");
}
