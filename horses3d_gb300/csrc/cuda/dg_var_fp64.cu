// Explicit instantiation of the variable-order / multi-case launchers in double precision.
#include "dg_var.cuh"

namespace dg {

VStageFn<double> vstage_fn_fp64() { return vrun_stage<double>; }
VTimesFn<double> vtimes_fn_fp64() { return vkernel_times<double>; }
VTuneFn<double> vtune_fn_fp64() { return vtime_items<double>; }

}  // namespace dg
