#include "status.hpp"

#include "horses3d_gb300.h"

namespace h3d {

namespace {
thread_local std::string g_last_error;
}

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

const char* last_error() { return g_last_error.c_str(); }

}  // namespace h3d

extern "C" {

const char* dg_last_error(void) { return h3d::last_error(); }

const char* dg_strerror(int code) {
    switch (code) {
        case DG_OK: return "ok";
        case DG_ERR_INVALID: return "invalid argument";
        case DG_ERR_UNSUPPORTED: return "option not supported by the GPU path";
        case DG_ERR_CUDA: return "CUDA runtime error";
        case DG_ERR_NAN: return "NaN or Inf in the solution";
        case DG_ERR_TIMEOUT: return "bounded device wait timed out";
        case DG_ERR_NOMEM: return "out of memory";
        case DG_ERR_NODEVICE: return "no CUDA device";
        case DG_ERR_IO: return "I/O error";
        default: return "unknown status";
    }
}

const char* dg_version(void) { return "horses3d_gb300 0.1.0 (sm_103a)"; }

}  // extern "C"
