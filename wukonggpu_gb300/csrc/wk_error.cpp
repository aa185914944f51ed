// Status strings and the per-thread last-error message of the C ABI.
//
// Kept apart from the CUDA runtime code so that the host-only generator
// library (libwkgen.so: wk_gen.cpp + this file) reports errors the same way
// as libwkgpu.so without linking CUDA.
#include <cstdarg>
#include <cstdio>

#include "wk_internal.h"

namespace wk {

static thread_local char g_err[512] = "";

int set_error(int status, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return status;
}

}  // namespace wk

extern "C" const char *wk_last_error(void) { return wk::g_err; }

extern "C" const char *wk_status_str(int s) {
    switch (s) {
        case WK_OK: return "ok";
        case WK_EINVAL: return "invalid argument";
        case WK_ENOMEM: return "out of memory";
        case WK_ETIMEDOUT: return "timed out";
        case WK_EDEVICE: return "device error";
        case WK_ENOSTORE: return "no store";
        case WK_EOVERFLOW: return "overflow";
        case WK_ECANCELED: return "cancelled";
        case WK_EREJECTED: return "rejected at admission";
        default: return "unknown status";
    }
}
