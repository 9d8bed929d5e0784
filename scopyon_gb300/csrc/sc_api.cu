// Library-level entry points: version and error reporting.
#include <stdarg.h>
#include <stdio.h>

#include "sc_common.cuh"

namespace sc {

static thread_local char g_last_error[512] = "";

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
}

int cuda_status(cudaError_t err, const char *what) {
    if (err == cudaSuccess) return SC_OK;
    set_error("%s: %s", what, cudaGetErrorString(err));
    return SC_ERR_CUDA;
}

int launch_status(const char *what) { return cuda_status(cudaGetLastError(), what); }

}  // namespace sc

extern "C" int sc_get_version(void) { return 1; }

extern "C" const char *sc_last_error(void) { return sc::g_last_error; }
