// eri_q10_df.cu -- double-float per-thread J/K kernel of quartet class (dp|ss)
// (about 46-bit arithmetic on the FP32 pipe, csrc/df64.cuh).  The dispatch
// table in capi.cu calls this launcher.
#include "eri.cuh"

namespace sq {

cudaError_t launch_qc_10_df(const EriArgs &a, int mode, int prec, cudaStream_t s) {
    return launch_eri_class_df<2, 1, 0, 0>(a, mode, prec, s);
}

}  // namespace sq
