// status.cpp - thread-local last-error message and status names.
#include "status.h"

#include <cstring>

namespace {
thread_local char g_last_error[512] = "";
}

namespace ct {

ct_status fail(ct_status s, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_last_error, sizeof g_last_error, fmt, ap);
    va_end(ap);
    return s;
}

void clear_error() { g_last_error[0] = '\0'; }

}  // namespace ct

extern "C" {

const char* ct_version(void) { return "cthermal 0.1 (sm_103a)"; }

const char* ct_last_error(void) { return g_last_error; }

const char* ct_status_string(ct_status s) {
    switch (s) {
        case CT_OK: return "ok";
        case CT_NOT_CONVERGED: return "not converged";
        case CT_BREAKDOWN: return "breakdown";
        case CT_CUDA_ERROR: return "CUDA error";
        case CT_TIMEOUT: return "timeout";
        case CT_BAD_ARG: return "bad argument";
        case CT_NOT_FINALIZED: return "model not finalized";
        case CT_NO_DEVICE: return "no CUDA device";
        case CT_OUT_OF_MEMORY: return "out of device memory";
        case CT_IO_ERROR: return "I/O error";
    }
    return "unknown status";
}

}  // extern "C"
