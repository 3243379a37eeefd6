// Status strings and the per-thread last-error message of the C ABI.
#include <cstdio>
#include <cstring>

#include "fvgb.h"
#include "fvgb_host_common.h"

namespace {
thread_local char g_last_error[512] = {0};
}

extern "C" fvgb_status fvgb_fail(fvgb_status st, const char* msg) {
    std::snprintf(g_last_error, sizeof g_last_error, "%s", msg ? msg : "");
    return st;
}

extern "C" void fvgb_clear_error(void) { g_last_error[0] = 0; }

extern "C" const char* fvgb_last_error(void) { return g_last_error; }

extern "C" int32_t fvgb_abi_version(void) { return (1 << 16) | 0; }

extern "C" const char* fvgb_status_string(int status) {
    switch (status) {
        case FVGB_OK: return "FVGB_OK";
        case FVGB_ERR_INVALID_ARG: return "FVGB_ERR_INVALID_ARG";
        case FVGB_ERR_OOM: return "FVGB_ERR_OOM";
        case FVGB_ERR_NOT_CONVERGED: return "FVGB_ERR_NOT_CONVERGED";
        case FVGB_ERR_BREAKDOWN: return "FVGB_ERR_BREAKDOWN";
        case FVGB_ERR_CUDA: return "FVGB_ERR_CUDA";
        case FVGB_ERR_UNSUPPORTED: return "FVGB_ERR_UNSUPPORTED";
        case FVGB_ERR_BUDGET: return "FVGB_ERR_BUDGET";
        case FVGB_ERR_CANCELLED: return "FVGB_ERR_CANCELLED";
        default: return "FVGB_ERR_UNKNOWN";
    }
}
