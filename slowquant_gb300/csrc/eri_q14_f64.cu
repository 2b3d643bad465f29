// eri_q14_f64.cu -- per-thread FP64 J/K kernel of quartet class (dp|dp).  Its
// register block spills partly to local memory; it still outruns the generic
// warp kernel (whose FP64 lanes are about half idle) and shares SMs with the
// other classes' launches.  The dispatch table in capi.cu calls this launcher.
#include "eri.cuh"

namespace sq {

cudaError_t launch_qc_14_f64(const EriArgs &a, int mode, int prec, cudaStream_t s) {
    return launch_eri_class_f64<2, 1, 2, 1>(a, mode, prec, s);
}

}  // namespace sq
