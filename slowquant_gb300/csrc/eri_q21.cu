// eri_q21.cu -- per-thread J/K kernels of quartet class (fs|ss), an f-shell class
// light enough (L <= 4) for the register-blocked kernel.
// The dispatch table in capi.cu calls this launcher.
#include "eri.cuh"

namespace sq {

cudaError_t launch_qc_21(const EriArgs &a, int mode, int prec, cudaStream_t s) {
    return launch_eri_class<3, 0, 0, 0>(a, mode, prec, s);
}

}  // namespace sq
