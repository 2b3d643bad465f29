// eri_q0.cu -- per-thread J/K kernels of quartet class (ss|ss).
// The dispatch table in capi.cu calls this launcher.
#include "eri.cuh"

namespace sq {

cudaError_t launch_qc_0(const EriArgs &a, int mode, int prec, cudaStream_t s) {
    return launch_eri_class<0, 0, 0, 0>(a, mode, prec, s);
}

}  // namespace sq
