// eri_q15.cu -- per-thread J/K kernel of quartet class (dd|ss), FP32 integral
// arithmetic with the FP64 Boys recursion only (its all-FP32-Boys launches run on
// the generic warp kernel; FP64 is in eri_q15_f64.cu).  The dispatch table in
// capi.cu calls this launcher.
#include "eri.cuh"

namespace sq {

cudaError_t launch_qc_15_f32(const EriArgs &a, int mode, int prec, cudaStream_t s) {
    return launch_eri_class_f32<2, 2, 0, 0>(a, mode, prec, s);
}

}  // namespace sq
