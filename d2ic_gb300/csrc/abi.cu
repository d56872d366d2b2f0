// Library-wide pieces of the C ABI: version and error reporting.
#include <stdarg.h>
#include <string.h>

#include "common.cuh"

namespace d2ic {

static thread_local char g_err[1024] = "";

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int cuda_status(cudaError_t e, const char *what) {
    set_error("%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
    if (e == cudaErrorMemoryAllocation) return D2IC_OOM;
    return D2IC_CUDA_ERROR;
}

}  // namespace d2ic

extern "C" const char *d2ic_last_error_string(void) { return d2ic::g_err; }

extern "C" int d2ic_version(void) { return 101; }

extern "C" size_t d2ic_frame_descriptor_bytes(void) { return sizeof(d2ic_frame_t); }
