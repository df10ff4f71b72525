// Explicit instantiation of the variable-order / multi-case launchers in single precision (the
// mixed form; compiled with fast FP32 division and square root like the uniform FP32 unit).
#include "dg_var.cuh"

namespace dg {

VStageFn<float> vstage_fn_fp32() { return vrun_stage<float>; }
VTimesFn<float> vtimes_fn_fp32() { return vkernel_times<float>; }
VTuneFn<float> vtune_fn_fp32() { return vtime_items<float>; }

}  // namespace dg
