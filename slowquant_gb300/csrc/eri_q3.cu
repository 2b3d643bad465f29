// eri_q3.cu -- per-thread J/K kernels of quartet class (pp|ss).
// The dispatch table in capi.cu calls this launcher.
#include "eri.cuh"

namespace sq {

cudaError_t launch_qc_3(const EriArgs &a, int mode, int prec, cudaStream_t s) {
    return launch_eri_class<1, 1, 0, 0>(a, mode, prec, s);
}

}  // namespace sq
