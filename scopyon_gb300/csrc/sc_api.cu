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

namespace {
__global__ void counter_add_kernel(int64_t *c, int64_t delta) { *c += delta; }
}  // namespace

extern "C" int sc_counter_add(int64_t *d_counter, int64_t delta, void *stream) {
    SC_REQUIRE(d_counter != nullptr, "sc_counter_add: counter is NULL");
    counter_add_kernel<<<1, 1, 0, sc::as_stream(stream)>>>(d_counter, delta);
    return sc::launch_status("sc_counter_add");
}
