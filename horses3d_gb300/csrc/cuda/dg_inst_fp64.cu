// Explicit instantiations of the double stage launchers for P = 2..8 and both node families.
#include "dg_launch.cuh"

namespace dg {

MonitorFns<double> monitor_fns_fp64(int P, bool gl) {
    MonitorFns<double> f{nullptr};
    if (P == 6) {
        f.dt = gl ? monitor_dt<6, true, double> : monitor_dt<6, false, double>;
    }
    return f;
}

StageFn<double> stage_fn_fp64(int P, bool gl) {
    switch (P) {
        case 2: return gl ? run_stage<2, true, double> : run_stage<2, false, double>;
        case 3: return gl ? run_stage<3, true, double> : run_stage<3, false, double>;
        case 4: return gl ? run_stage<4, true, double> : run_stage<4, false, double>;
        case 5: return gl ? run_stage<5, true, double> : run_stage<5, false, double>;
        case 6: return gl ? run_stage<6, true, double> : run_stage<6, false, double>;
        case 7: return gl ? run_stage<7, true, double> : run_stage<7, false, double>;
        case 8: return gl ? run_stage<8, true, double> : run_stage<8, false, double>;
        default: return nullptr;
    }
}

KernelTimesFn<double> times_fn_fp64(int P, bool gl) {
    switch (P) {
        case 2: return gl ? kernel_times<2, true, double> : kernel_times<2, false, double>;
        case 3: return gl ? kernel_times<3, true, double> : kernel_times<3, false, double>;
        case 4: return gl ? kernel_times<4, true, double> : kernel_times<4, false, double>;
        case 5: return gl ? kernel_times<5, true, double> : kernel_times<5, false, double>;
        case 6: return gl ? kernel_times<6, true, double> : kernel_times<6, false, double>;
        case 7: return gl ? kernel_times<7, true, double> : kernel_times<7, false, double>;
        case 8: return gl ? kernel_times<8, true, double> : kernel_times<8, false, double>;
        default: return nullptr;
    }
}

}  // namespace dg
