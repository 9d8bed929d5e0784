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

extern "C" int sc_box_block_floats(int nq) { return SC_BOX_BLOCK_FLOATS(nq); }

extern "C" int sc_set_l2_fetch_granularity(int bytes) {
    SC_REQUIRE(bytes == 0 || bytes == 32 || bytes == 64 || bytes == 128,
               "sc_set_l2_fetch_granularity: %d bytes (0, 32, 64 or 128)", bytes);
    return sc::cuda_status(cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, (size_t)bytes),
                           "sc_set_l2_fetch_granularity");
}

extern "C" int sc_copy_async(void *dst, const void *src, size_t bytes, void *stream) {
    if (bytes == 0) return SC_OK;
    SC_REQUIRE(dst != nullptr && src != nullptr, "sc_copy_async: NULL pointer");
    return sc::cuda_status(
        cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, sc::as_stream(stream)),
        "sc_copy_async");
}

extern "C" int sc_struct_sizes(size_t *out, int n) {
    SC_REQUIRE(out != nullptr && n >= 6, "sc_struct_sizes: need room for 6 sizes");
    out[0] = sizeof(ScStepRec);
    out[1] = sizeof(ScStepParams);
    out[2] = sizeof(ScSplatParams);
    out[3] = sizeof(ScCameraParams);
    out[4] = sizeof(ScDiffuseParams);
    out[5] = sizeof(ScGaussParams);
    return SC_OK;
}

extern "C" const char *sc_last_error(void) { return sc::g_last_error; }

namespace {
__global__ void counter_add_kernel(int64_t *c, int64_t delta) { *c += delta; }
}  // namespace

extern "C" int sc_counter_add(int64_t *d_counter, int64_t delta, void *stream) {
    SC_REQUIRE(d_counter != nullptr, "sc_counter_add: counter is NULL");
    counter_add_kernel<<<1, 1, 0, sc::as_stream(stream)>>>(d_counter, delta);
    return sc::launch_status("sc_counter_add");
}

// Host side of the frame upload: one pass over a sub-step's (n x 5) rows
// [depth, x, y, id, state] that checks the ids against the known slot order,
// copies the rows into the (pinned) staging buffer and takes the depth range.
// Returns 1 at the first id that differs (dst then partly written), else 0.
extern "C" int sc_stage_rows(const double *src, int64_t n, const double *ids, double *dst,
                             double *depth_range) {
    if (n < 0 || (n > 0 && (!src || !ids || !dst)) || !depth_range) {
        sc::set_error("sc_stage_rows: bad arguments");
        return SC_ERR_ARG;
    }
    double lo = 0.0, hi = 0.0;
    bool nan_seen = false;
    for (int64_t i = 0; i < n; ++i) {
        const double *r = src + 5 * i;
        if (!(r[3] == ids[i])) return 1;  // a NaN id differs too
        double *d = dst + 5 * i;
        d[0] = r[0];
        d[1] = r[1];
        d[2] = r[2];
        d[3] = r[3];
        d[4] = r[4];
        const double z = r[0];
        if (z != z) nan_seen = true;
        if (i == 0) {
            lo = hi = z;
        } else {
            lo = z < lo ? z : lo;
            hi = z > hi ? z : hi;
        }
    }
    const double nan = __builtin_nan("");
    depth_range[0] = nan_seen ? nan : lo;
    depth_range[1] = nan_seen ? nan : hi;
    return 0;
}

namespace sc {

int resident_grid(const void *fn, int block, size_t smem, int64_t want) {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        sms < 1)
        sms = 152;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, block, smem) != cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    const int64_t wave = (int64_t)sms * per_sm;
    if (want < 1) want = 1;
    return (int)(want < wave ? want : wave);
}

}  // namespace sc
