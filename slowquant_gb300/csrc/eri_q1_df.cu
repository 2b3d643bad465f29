// eri_q1_df.cu -- double-float per-thread J/K kernel of quartet class (ps|ss)
// (about 46-bit arithmetic on the FP32 pipe, csrc/df64.cuh).  The dispatch
// table in capi.cu calls this launcher.
#include "eri.cuh"

namespace sq {

cudaError_t launch_qc_1_df(const EriArgs &a, int mode, int prec, cudaStream_t s) {
    return launch_eri_class_df<1, 0, 0, 0>(a, mode, prec, s);
}

}  // namespace sq
