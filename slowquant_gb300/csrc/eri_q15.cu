// eri_q15.cu -- per-thread J/K kernels of quartet class (dd|ss): FP32 integral
// arithmetic with the FP64 Boys recursion, and FP64 (its all-FP32-Boys launches
// run on the generic warp kernel).  The dispatch tables in capi.cu call these launchers.
#include "eri.cuh"

namespace sq {

cudaError_t launch_qc_15_f32(const EriArgs &a, int mode, int prec, cudaStream_t s) {
    return launch_eri_class_f32<2, 2, 0, 0>(a, mode, prec, s);
}

cudaError_t launch_qc_15_f64(const EriArgs &a, int mode, int prec, cudaStream_t s) {
    return launch_eri_class_f64<2, 2, 0, 0>(a, mode, prec, s);
}

}  // namespace sq
