// eri_q13.cu -- per-thread J/K kernel of quartet class (dp|ds), FP32 integral
// arithmetic with the FP64 Boys recursion only (its FP64 and all-FP32-Boys launches
// run on the generic warp kernel).  The dispatch table in capi.cu calls this launcher.
#include "eri.cuh"

namespace sq {

cudaError_t launch_qc_13_f32(const EriArgs &a, int mode, int prec, cudaStream_t s) {
    return launch_eri_class_f32<2, 1, 2, 0>(a, mode, prec, s);
}

// FP64 per-thread variant: its register block spills to local memory, which
// still beats the generic warp kernel's lane utilisation for this class.
cudaError_t launch_qc_13_f64(const EriArgs &a, int mode, int prec, cudaStream_t s) {
    return launch_eri_class_f64<2, 1, 2, 0>(a, mode, prec, s);
}

}  // namespace sq
