// eri_q7.cu -- per-thread J/K kernels of quartet class (ds|ps).
// The dispatch table in capi.cu calls this launcher.
#include "eri.cuh"

namespace sq {

cudaError_t launch_qc_7(const EriArgs &a, int mode, int prec, cudaStream_t s) {
    return launch_eri_class<2, 0, 1, 0>(a, mode, prec, s);
}

}  // namespace sq
