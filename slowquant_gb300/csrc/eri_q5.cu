// eri_q5.cu -- per-thread J/K kernels of quartet class (pp|pp).
// The dispatch table in capi.cu calls this launcher.
#include "eri.cuh"

namespace sq {

cudaError_t launch_qc_5(const EriArgs &a, int mode, int prec, cudaStream_t s) {
    return launch_eri_class<1, 1, 1, 1>(a, mode, prec, s);
}

}  // namespace sq
