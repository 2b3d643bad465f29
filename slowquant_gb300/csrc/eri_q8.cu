// eri_q8.cu -- per-thread J/K kernels of quartet class (ds|pp).
// The dispatch table in capi.cu calls this launcher.
#include "eri.cuh"

namespace sq {

cudaError_t launch_qc_8(const EriArgs &a, int mode, int prec, cudaStream_t s) {
    return launch_eri_class<2, 0, 1, 1>(a, mode, prec, s);
}

}  // namespace sq
