// Explicit instantiations of the float stage launchers for P = 2..8 and both node families.
#include "dg_launch.cuh"

namespace dg {

MonitorFns<float> monitor_fns_fp32(int P, bool gl) {
    MonitorFns<float> f{nullptr};
    if (P == 6) {
        f.dt = gl ? monitor_dt<6, true, float> : monitor_dt<6, false, float>;
    }
    return f;
}

StageFn<float> stage_fn_fp32(int P, bool gl) {
    switch (P) {
        case 2: return gl ? run_stage<2, true, float> : run_stage<2, false, float>;
        case 3: return gl ? run_stage<3, true, float> : run_stage<3, false, float>;
        case 4: return gl ? run_stage<4, true, float> : run_stage<4, false, float>;
        case 5: return gl ? run_stage<5, true, float> : run_stage<5, false, float>;
        case 6: return gl ? run_stage<6, true, float> : run_stage<6, false, float>;
        case 7: return gl ? run_stage<7, true, float> : run_stage<7, false, float>;
        case 8: return gl ? run_stage<8, true, float> : run_stage<8, false, float>;
        default: return nullptr;
    }
}

KernelTimesFn<float> times_fn_fp32(int P, bool gl) {
    switch (P) {
        case 2: return gl ? kernel_times<2, true, float> : kernel_times<2, false, float>;
        case 3: return gl ? kernel_times<3, true, float> : kernel_times<3, false, float>;
        case 4: return gl ? kernel_times<4, true, float> : kernel_times<4, false, float>;
        case 5: return gl ? kernel_times<5, true, float> : kernel_times<5, false, float>;
        case 6: return gl ? kernel_times<6, true, float> : kernel_times<6, false, float>;
        case 7: return gl ? kernel_times<7, true, float> : kernel_times<7, false, float>;
        case 8: return gl ? kernel_times<8, true, float> : kernel_times<8, false, float>;
        default: return nullptr;
    }
}

}  // namespace dg
