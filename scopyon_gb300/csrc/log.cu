// Laplacian-of-Gaussian scale space and its local maxima: the blob search of
// spot_detection (src/scopyon/analysis/spot_detection.py:14-46, which calls
// scikit-image's blob_log), written from the published method.
//
// For each scale sigma_s the scale-normalised LoG is
//   cube[i][j][s] = -sigma_s^2 * (d2 (x) phi + phi (x) d2)(image)[i][j],
// with phi the normalised Gaussian kernel and d2 its second derivative, both
// of radius int(4 sigma + 0.5), and scipy.ndimage's 'reflect' edges
// (d c b a | a b c d | d c b a, repeated).  Two separable FP64 passes: along
// axis 0 (both kernels), then along axis 1 (the other kernel of each pair).
// A blob is a cell above the threshold that is the maximum of its 3 x 3 x 3
// neighbourhood (cells past the cube's edges ignored).
#include "sc_common.cuh"

namespace {

// 'reflect' index of k on an axis of n samples.
__device__ __forceinline__ int reflect(int k, int n) {
    const int m = 2 * n;
    int q = k % m;
    if (q < 0) q += m;
    return q < n ? q : m - 1 - q;
}

// Pass 1: a[s][i][j] = sum_t d2_s[t] img[i + t - R][j], b[s][i][j] the same
// with phi_s (correlation along axis 0; the kernels are symmetric).
__global__ void log_axis0_kernel(const double *__restrict__ img, int nw, int nh,
                                 const double *__restrict__ phi, const double *__restrict__ d2,
                                 const int32_t *__restrict__ off, const int32_t *__restrict__ rad,
                                 int n_scales, double *__restrict__ a, double *__restrict__ b) {
    const int64_t cells = (int64_t)nw * nh;
    const int64_t total = cells * n_scales;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total;
         g += (int64_t)gridDim.x * blockDim.x) {
        const int s = (int)(g / cells);
        const int64_t c = g - (int64_t)s * cells;
        const int i = (int)(c / nh), j = (int)(c - (int64_t)i * nh);
        const int R = rad[s], o = off[s];
        double sa = 0.0, sb = 0.0;
        for (int t = -R; t <= R; ++t) {
            const double v = img[(int64_t)reflect(i + t, nw) * nh + j];
            sa = fma(d2[o + t + R], v, sa);
            sb = fma(phi[o + t + R], v, sb);
        }
        a[g] = sa;
        b[g] = sb;
    }
}

// Pass 2: cube[i][j][s] = -sigma_s^2 (sum_t phi_s[t] a[s][i][j + t - R] +
// sum_t d2_s[t] b[s][i][j + t - R]).
__global__ void log_axis1_kernel(const double *__restrict__ a, const double *__restrict__ b,
                                 int nw, int nh, const double *__restrict__ phi,
                                 const double *__restrict__ d2, const int32_t *__restrict__ off,
                                 const int32_t *__restrict__ rad,
                                 const double *__restrict__ sigma, int n_scales,
                                 double *__restrict__ cube) {
    const int64_t cells = (int64_t)nw * nh;
    const int64_t total = cells * n_scales;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total;
         g += (int64_t)gridDim.x * blockDim.x) {
        const int s = (int)(g / cells);
        const int64_t c = g - (int64_t)s * cells;
        const int i = (int)(c / nh), j = (int)(c - (int64_t)i * nh);
        const int R = rad[s], o = off[s];
        const double *ra = a + (int64_t)s * cells + (int64_t)i * nh;
        const double *rb = b + (int64_t)s * cells + (int64_t)i * nh;
        double sa = 0.0, sb = 0.0;
        for (int t = -R; t <= R; ++t) {
            const int q = reflect(j + t, nh);
            sa = fma(phi[o + t + R], ra[q], sa);
            sb = fma(d2[o + t + R], rb[q], sb);
        }
        cube[c * n_scales + s] = -(sa + sb) * (sigma[s] * sigma[s]);
    }
}

// Cells above the threshold that equal the maximum of their 3 x 3 x 3
// neighbourhood, appended as (i, j, s) triples in no particular order.
__global__ void log_peaks_kernel(const double *__restrict__ cube, int nw, int nh, int n_scales,
                                 double threshold, int32_t *count, int32_t *peaks, int capacity) {
    const int64_t total = (int64_t)nw * nh * n_scales;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total;
         g += (int64_t)gridDim.x * blockDim.x) {
        const double v = cube[g];
        if (!(v > threshold)) continue;
        const int s = (int)(g % n_scales);
        const int64_t c = g / n_scales;
        const int i = (int)(c / nh), j = (int)(c - (int64_t)i * nh);
        bool top = true;
        for (int di = -1; di <= 1 && top; ++di) {
            const int ii = i + di;
            if (ii < 0 || ii >= nw) continue;
            for (int dj = -1; dj <= 1 && top; ++dj) {
                const int jj = j + dj;
                if (jj < 0 || jj >= nh) continue;
                const double *row = cube + ((int64_t)ii * nh + jj) * n_scales;
                for (int ds = -1; ds <= 1; ++ds) {
                    const int ss = s + ds;
                    if (ss < 0 || ss >= n_scales) continue;
                    if (row[ss] > v) {
                        top = false;
                        break;
                    }
                }
            }
        }
        if (!top) continue;
        const int k = atomicAdd(count, 1);
        if (k < capacity) {
            peaks[3 * k] = i;
            peaks[3 * k + 1] = j;
            peaks[3 * k + 2] = s;
        }
    }
}

int grid_for(int64_t total) {
    int64_t g = (total + 255) / 256;
    return (int)(g < 152 * 16 ? (g > 0 ? g : 1) : 152 * 16);
}

}  // namespace

extern "C" int sc_log_cube(const double *d_img, int nw, int nh, const double *d_phi,
                           const double *d_d2, const int32_t *d_tap_off, const int32_t *d_radius,
                           const double *d_sigma, int n_scales, double *d_work, size_t work_bytes,
                           double *d_cube, void *stream) {
    SC_REQUIRE(nw > 0 && nh > 0 && n_scales > 0, "sc_log_cube: %d x %d x %d", nw, nh, n_scales);
    SC_REQUIRE(d_img && d_phi && d_d2 && d_tap_off && d_radius && d_sigma && d_cube,
               "sc_log_cube: NULL pointer");
    const int64_t total = (int64_t)nw * nh * n_scales;
    SC_REQUIRE_CAP(d_work && work_bytes >= (size_t)total * 2 * sizeof(double),
                   "sc_log_cube: work %zu < %zu bytes", work_bytes,
                   (size_t)total * 2 * sizeof(double));
    cudaStream_t st = sc::as_stream(stream);
    double *a = d_work, *b = d_work + total;
    log_axis0_kernel<<<grid_for(total), 256, 0, st>>>(d_img, nw, nh, d_phi, d_d2, d_tap_off,
                                                      d_radius, n_scales, a, b);
    log_axis1_kernel<<<grid_for(total), 256, 0, st>>>(a, b, nw, nh, d_phi, d_d2, d_tap_off,
                                                      d_radius, d_sigma, n_scales, d_cube);
    return sc::launch_status("sc_log_cube");
}

extern "C" int sc_log_peaks(const double *d_cube, int nw, int nh, int n_scales, double threshold,
                            int32_t *d_count, int32_t *d_peaks, int capacity, void *stream) {
    SC_REQUIRE(nw > 0 && nh > 0 && n_scales > 0, "sc_log_peaks: %d x %d x %d", nw, nh, n_scales);
    SC_REQUIRE(d_cube && d_count && d_peaks && capacity > 0, "sc_log_peaks: NULL pointer");
    cudaStream_t st = sc::as_stream(stream);
    int rc = sc::cuda_status(cudaMemsetAsync(d_count, 0, sizeof(int32_t), st), "sc_log_peaks");
    if (rc) return rc;
    const int64_t total = (int64_t)nw * nh * n_scales;
    log_peaks_kernel<<<grid_for(total), 256, 0, st>>>(d_cube, nw, nh, n_scales, threshold,
                                                      d_count, d_peaks, capacity);
    return sc::launch_status("sc_log_peaks");
}
