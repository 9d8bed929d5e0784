// Camera models and analog-to-digital conversion, one pass over the frame.
//
// Reference: _EPIFMSimulator.__detector_output and
// __get_analog_to_digital_converter_counts (src/scopyon/_epifm.py:1430-1484),
// with the detector classes EMCCD / CCD / CMOS (:329-433):
//   photons += background_mean when the background switch is on (:1437-1438;
//   the caller passes background = 0 otherwise), then expected = QE * photons
//   (:1441), so expected = QE * (photons + background)
//   EMCCD: signal ~ compound Poisson-Gamma (EM gain), noise ~ N(0, readout)
//   CCD:   signal ~ Poisson(expected), noise ~ N(0, readout)
//   CMOS:  signal ~ Poisson(expected), noise ~ tabulated distribution (additive)
//   sCMOS (this engine only): noise ~ N(0, sigma_ij) with a per-pixel sigma map
//   ADC = clip(min(signal + noise, fullwell) / gain + offset, 0, 2^bit - 1)
//   (rounding the ADC count to an integer is an option of this engine only;
//   the reference's ADC count is an unrounded float, and parity runs keep
//   the option off)
// Draws come either from Philox4x32-10 (native, one counter stream per pixel)
// or from caller arrays recorded from the reference (injected), in which case
// the ADC arithmetic is the reference's FP64 sequence.
#include "sc_common.cuh"

namespace {

struct CamConsts {
    int n, camera, exact, rounding, table_n;
    double qe, background, readout, emgain, fullwell, adc_max, offset0, gain0;
    float qe_f, background_f, readout_f, emgain_f, fullwell_f, adc_max_f, offset0_f, inv_gain0_f;
    uint64_t seed, counter;
    const int64_t *frame;
    const double *photons64;  // exact mode: FP64 photons in place of the FP32 ones
    double *expect64;         // exact mode: FP64 expectation out
};

// Poisson variate.  Small means: sequential inversion.  Large means: the
// transformed rejection method PTRS (W. Hormann, "The transformed rejection
// method for generating Poisson random variables", Insurance: Mathematics and
// Economics 12 (1993) 39-45), with log(k!) from Stirling's series.  Divisions
// and the logarithms of the acceptance test use the approximate intrinsics
// (relative error ~1e-7): they move the accepted distribution by far less
// than any test of a frame's counts can see, and a pixel's draw costs about
// half the instructions of the IEEE forms.
__device__ float poisson(sc::rng_stream &rs, float lam, int32_t *status) {
    if (!(lam > 0.f)) return 0.f;
    if (lam < 12.f) {
        const float u = rs.uniform();
        float p = expf(-lam), s = p;
        int k = 0;
        while (u > s && k < 200) {
            ++k;
            p *= __fdividef(lam, (float)k);
            s += p;
        }
        return (float)k;
    }
    const float slam = sqrtf(lam), inv_lam = __fdividef(1.f, lam);
    const float b = 0.931f + 2.53f * slam;
    const float a = -0.059f + 0.02483f * b;
    const float invalpha = 1.1239f + __fdividef(1.1328f, b - 3.4f);
    const float vr = 0.9277f - __fdividef(3.6224f, b - 2.f);
    for (int it = 0; it < 64; ++it) {
        const float U = rs.uniform() - 0.5f;
        const float V = rs.uniform();
        const float us = 0.5f - fabsf(U);
        const float k = floorf((__fdividef(2.f * a, us) + b) * U + lam + 0.43f);
        if (us >= 0.07f && V <= vr) return k;
        if (k < 0.f || (us < 0.013f && V > us)) continue;
        // -lam + k log(lam) - log(k!) via Stirling, written relative to k - lam
        const float kk = fmaxf(k, 1.f);
        const float ikk = __fdividef(1.f, kk);
        const float d = (k - lam) * inv_lam;
        const float lfact_rel = (k - lam) - k * log1pf(d) - 0.5f * __logf(6.2831853f * kk) -
                                ikk * (1.f / 12.f) + ikk * ikk * ikk * (1.f / 360.f);
        const float rhs = k == 0.f ? -lam : lfact_rel;
        // log(V / alpha / (a / us^2 + b)) <= rhs
        if (__logf(__fdividef(V * invalpha, __fdividef(a, us * us) + b)) <= rhs) return k;
    }
    sc::flag_status(status, 3, 0, 0, 0);
    return rintf(lam);
}

// Gamma(shape, 1) for shape >= 1: G. Marsaglia and W. W. Tsang, "A simple
// method for generating gamma variables", ACM TOMS 26 (2000) 363-372.
__device__ float gamma_ge1(sc::rng_stream &rs, float shape, int32_t *status) {
    const float d = shape - 1.f / 3.f;
    const float c = rsqrtf(9.f * d);
    for (int it = 0; it < 64; ++it) {
        const float x = rs.normal();
        const float t = c * x;
        if (t <= -1.f) continue;
        const float u = rs.uniform();
        const float vm1 = t * (3.f + t * (3.f + t));  // (1 + t)^3 - 1
        const float x2 = x * x;
        if (u < 1.f - 0.0331f * x2 * x2) return d * (1.f + vm1);
        if (logf(u) < 0.5f * x2 + d * (3.f * log1pf(t) - vm1)) return d * (1.f + vm1);
    }
    sc::flag_status(status, 3, 1, 0, 0);
    return shape;
}

__device__ __forceinline__ int table_index(const double *cdf, int n, double u) {
    // searchsorted(cdf, u, side='right')
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (cdf[mid] <= u) lo = mid + 1;
        else hi = mid;
    }
    return lo < n ? lo : n - 1;
}

// One pixel's native draws (Philox stream keyed by the seed and the pixel, at
// the frame's counter; FP32 throughout, GB300's FP64 rate being ~1/64 of
// FP32) and its ADC count.
__device__ __forceinline__ void native_pixel(const CamConsts &c, int p, float ef, uint64_t counter,
                                             const float *__restrict__ offset_f,
                                             const float *__restrict__ inv_gain_f,
                                             const float *__restrict__ sigma,
                                             const double *__restrict__ table_value,
                                             const double *__restrict__ table_cdf,
                                             double *__restrict__ adc64, float *__restrict__ adc32,
                                             int32_t *status) {
    sc::rng_stream rs(c.seed, (uint32_t)p, (uint32_t)counter, (uint32_t)(counter >> 32));
    float signal, noise;
    switch (c.camera) {
        case SC_CAM_EMCCD: {
            const float n_in = poisson(rs, ef, status);
            signal = n_in > 0.f ? rintf(c.emgain_f * gamma_ge1(rs, n_in, status)) : 0.f;
            noise = c.readout_f > 0.f ? c.readout_f * rs.normal() : 0.f;
            break;
        }
        case SC_CAM_CCD:
            signal = poisson(rs, ef, status);
            noise = c.readout_f > 0.f ? c.readout_f * rs.normal() : 0.f;
            break;
        case SC_CAM_CMOS_TABLE:
            noise = (float)table_value[table_index(table_cdf, c.table_n, rs.uniform_d())];
            signal = poisson(rs, ef, status);
            break;
        default:  // SC_CAM_SCMOS
            signal = poisson(rs, ef, status);
            noise = (sigma ? sigma[p] : c.readout_f) * rs.normal();
            break;
    }
    float v = fminf(signal + noise, c.fullwell_f);
    v = v * (inv_gain_f ? inv_gain_f[p] : c.inv_gain0_f) + (offset_f ? offset_f[p] : c.offset0_f);
    v = fminf(fmaxf(v, 0.f), c.adc_max_f);
    if (c.rounding) v = rintf(v);
    if (adc32) adc32[p] = v;
    if (adc64) adc64[p] = sc::f2d_exact(v);
}

// Injected draws: the reference's FP64 arithmetic on the caller's draws.
__global__ void camera_exact_kernel(CamConsts c, const float *__restrict__ photons,
                                    const double *__restrict__ offset, const double *__restrict__ gain,
                                    const double *__restrict__ table_value,
                                    const double *__restrict__ table_cdf,
                                    const double *__restrict__ inj_noise,
                                    const double *__restrict__ inj_signal,
                                    const double *__restrict__ inj_uniform,
                                    float *__restrict__ expect, double *__restrict__ adc64,
                                    float *__restrict__ adc32) {
    const int stride = gridDim.x * blockDim.x;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < c.n; p += stride) {
        // E = QE (photons + background) with the reference's FP64 rounding
        const double ph = (c.photons64 ? c.photons64[p] : (double)photons[p]) + c.background;
        const double e = __dmul_rn(c.qe, ph);
        if (expect) expect[p] = (float)e;
        if (c.expect64) c.expect64[p] = e;
        double noise, signal;
        if (c.camera == SC_CAM_CMOS_TABLE && inj_uniform)
            noise = table_value[table_index(table_cdf, c.table_n, inj_uniform[p])];
        else
            noise = inj_noise ? inj_noise[p] : 0.0;
        signal = inj_signal ? inj_signal[p] : 0.0;
        double v = signal + noise;
        if (v > c.fullwell) v = c.fullwell;
        v /= gain ? gain[p] : c.gain0;
        v += offset ? offset[p] : c.offset0;
        if (v > c.adc_max) v = c.adc_max;
        if (v < 0) v = 0;
        if (c.rounding) v = rint(v);
        if (adc64) adc64[p] = v;
        if (adc32) adc32[p] = (float)v;
    }
}

// Native draws, a pixel per thread (frames of a few hundred thousand pixels,
// which need every resident warp).
__global__ void camera_pixel_kernel(CamConsts c, const float *__restrict__ photons,
                                    const float *__restrict__ offset_f,
                                    const float *__restrict__ inv_gain_f,
                                    const float *__restrict__ sigma,
                                    const double *__restrict__ table_value,
                                    const double *__restrict__ table_cdf,
                                    float *__restrict__ expect, double *__restrict__ adc64,
                                    float *__restrict__ adc32, int32_t *status) {
    const int stride = gridDim.x * blockDim.x;
    const uint64_t counter = c.counter + (c.frame ? (uint64_t)*c.frame : 0);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < c.n; p += stride) {
        const float ef = c.qe_f * (photons[p] + c.background_f);
        if (expect) expect[p] = ef;
        native_pixel(c, p, ef, counter, offset_f, inv_gain_f, sigma, table_value, table_cdf,
                     adc64, adc32, status);
    }
}

constexpr int kCamThreads = 256;
constexpr int kCamMaxPer = 8;  // pixels per lane per chunk, at most

// Native draws.  Each warp takes chunks of 32 * per pixels: it writes their
// expectations, sorts the pixels by the Poisson method they need (inversion
// below lambda = 12 and empty pixels to the front of a shared list, PTRS to
// the back) with ballots, then draws them 32 at a time, one list after the
// other.  A pixel's draws are those of its own Philox stream whichever lane
// takes it, so the counts do not depend on the grouping; the grouping keeps
// a warp from running both methods' loops for one set of 32 pixels (6% off
// an 8192^2 frame).  Frames too small to fill the GPU twice over take
// camera_pixel_kernel instead.
__global__ void __launch_bounds__(kCamThreads)
camera_native_kernel(CamConsts c, int per, const float *__restrict__ photons,
                     const float *__restrict__ offset_f, const float *__restrict__ inv_gain_f,
                     const float *__restrict__ sigma, const double *__restrict__ table_value,
                     const double *__restrict__ table_cdf, float *__restrict__ expect,
                     double *__restrict__ adc64, float *__restrict__ adc32, int32_t *status) {
    constexpr int kWarps = kCamThreads / 32, kList = 32 * kCamMaxPer;
    __shared__ int s_pix[kWarps][kList];
    __shared__ float s_ef[kWarps][kList];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t counter = c.counter + (c.frame ? (uint64_t)*c.frame : 0);
    const int chunk = 32 * per;
    const int64_t warps = (int64_t)gridDim.x * kWarps;
    int *pix = s_pix[warp];
    float *efs = s_ef[warp];
    const unsigned below = (1u << lane) - 1u;
    for (int64_t base = ((int64_t)blockIdx.x * kWarps + warp) * chunk; base < c.n;
         base += warps * chunk) {
        int n_front = 0, n_back = 0;
        for (int j = 0; j < per; ++j) {
            const int64_t p = base + j * 32 + lane;
            const bool valid = p < c.n;
            float ef = 0.f;
            if (valid) {
                ef = c.qe_f * (photons[p] + c.background_f);
                if (expect) expect[p] = ef;
            }
            const bool ptrs = valid && ef >= 12.f;  // poisson()'s own threshold
            const bool front = valid && !ptrs;
            const unsigned mf = __ballot_sync(~0u, front), mp = __ballot_sync(~0u, ptrs);
            if (front) {
                const int k = n_front + __popc(mf & below);
                pix[k] = (int)p;
                efs[k] = ef;
            }
            if (ptrs) {
                const int k = kList - 1 - (n_back + __popc(mp & below));
                pix[k] = (int)p;
                efs[k] = ef;
            }
            n_front += __popc(mf);
            n_back += __popc(mp);
        }
        __syncwarp();
        for (int k = lane; k < n_front; k += 32)
            native_pixel(c, pix[k], efs[k], counter, offset_f, inv_gain_f, sigma, table_value,
                         table_cdf, adc64, adc32, status);
        for (int k = lane; k < n_back; k += 32)
            native_pixel(c, pix[kList - 1 - k], efs[kList - 1 - k], counter, offset_f, inv_gain_f,
                         sigma, table_value, table_cdf, adc64, adc32, status);
        __syncwarp();
    }
}

// ---------------------------------------------------------------- exact EMCCD
// i1e(y) = I1(y) exp(-y).  CUDA's cyl_bessel_i1 is finite below ~710; above
// 600 the asymptotic expansion (Abramowitz & Stegun 9.7.1, nu = 1) is used.
__device__ double i1e_d(double y) {
    if (y < 600.0) return cyl_bessel_i1(y) * exp(-y);
    const double mu = 4.0;
    double term = 1.0, sum = 1.0;
    for (int k = 1; k <= 10; ++k) {
        const double odd = (double)(2 * k - 1);
        term *= -(mu - odd * odd) / ((double)k * 8.0 * y);
        sum += term;
    }
    return sum / sqrt(2.0 * M_PI * y);
}

// One warp per pixel: support [s_min, s_max), weights p(S) with the exponent
// shifted by E (the continuous maximum, so nothing overflows), total, then
// the first S whose cumulative weight exceeds u * total.
__global__ void emccd_exact_kernel(const double *photons, double qe, double background,
                                   const double *uniform, int n, double g, double *signal,
                                   int32_t *status) {
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; p < n; p += warps) {
        const double e = __dmul_rn(qe, photons[p] + background);
        if (!(e > 0.0)) {
            if (lane == 0) signal[p] = 0.0;
            continue;
        }
        const double sig = sqrt(e) * 5 + 10;
        const double smin_d = fmax(0.0, g * trunc(e - sig));
        const double smax_d = g * trunc(e + sig);
        const int64_t s_min = (int64_t)smin_d, count = (int64_t)smax_d - s_min;
        if (count <= 0) {
            if (lane == 0) {
                signal[p] = 0.0;
                sc::flag_status(status, 2, p, 0, 0);
            }
            continue;
        }
        const double a = 1.0 / g;
        auto weight = [&](int64_t idx) -> double {
            const double S = (double)(s_min + idx);
            if (S <= 0.0) return 1.0 / (2 * a * e) * exp(-e);
            const double X = a * S;
            const double Y = 2 * sqrt(e * X);
            return 1.0 / Y * exp(-X + Y - e) * i1e_d(Y);
        };
        double total = 0.0;
        for (int64_t base = 0; base < count; base += 32) {
            const int64_t idx = base + lane;
            double w = idx < count ? weight(idx) : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
            total += w;
        }
        const double target = uniform[p] * total;
        double run = 0.0;
        int64_t found = count - 1;
        for (int64_t base = 0; base < count; base += 32) {
            const int64_t idx = base + lane;
            double w = idx < count ? weight(idx) : 0.0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const double nb = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += nb;
            }
            const unsigned hit = __ballot_sync(0xffffffffu, idx < count && run + w > target);
            if (hit) {
                found = base + (__ffs(hit) - 1);
                break;
            }
            run += __shfl_sync(0xffffffffu, w, 31);
        }
        if (lane == 0) signal[p] = (double)(s_min + found);
    }
}

}  // namespace

extern "C" int sc_camera(const ScCameraParams *p, const float *d_photons, const double *d_offset,
                         const double *d_gain, const float *d_offset_f, const float *d_inv_gain_f,
                         const float *d_sigma, const double *d_table_value,
                         const double *d_table_cdf, const double *d_inj_noise,
                         const double *d_inj_signal, const double *d_inj_uniform, float *d_expect,
                         double *d_adc64, float *d_adc32, int32_t *d_status, void *stream) {
    SC_REQUIRE(p != nullptr, "sc_camera: params are NULL");
    SC_REQUIRE(p->nw > 0 && p->nh > 0, "sc_camera: image %dx%d", p->nw, p->nh);
    SC_REQUIRE(p->camera >= SC_CAM_EMCCD && p->camera <= SC_CAM_SCMOS, "sc_camera: camera %d",
               p->camera);
    SC_REQUIRE(p->bit > 0 && p->bit <= 32, "sc_camera: bit=%d", p->bit);
    SC_REQUIRE((d_photons != nullptr || (p->exact && p->d_photons64 != nullptr)) &&
                   (d_adc64 || d_adc32),
               "sc_camera: NULL input/output");
    SC_REQUIRE(p->exact || (p->d_photons64 == nullptr && p->d_expect64 == nullptr),
               "sc_camera: FP64 photons and expectation are exact-mode buffers");
    if (p->camera == SC_CAM_CMOS_TABLE)
        SC_REQUIRE(p->table_n > 0 && d_table_value && d_table_cdf,
                   "sc_camera: CMOS table mode needs the noise table");
    if (p->exact) {
        SC_REQUIRE(d_inj_signal != nullptr, "sc_camera: exact mode needs injected signal");
        SC_REQUIRE(p->camera == SC_CAM_CMOS_TABLE ? (d_inj_uniform || d_inj_noise) : true,
                   "sc_camera: CMOS exact mode needs injected uniforms or noise");
    }
    CamConsts c;
    c.n = p->nw * p->nh;
    c.camera = p->camera;
    c.exact = p->exact;
    c.rounding = p->rounding;
    c.table_n = p->table_n;
    c.qe = p->qe;
    c.background = p->background;
    c.readout = p->readout_noise;
    c.emgain = p->emgain;
    c.fullwell = p->fullwell;
    c.adc_max = (double)((1ull << p->bit) - 1);
    c.offset0 = p->offset0;
    c.gain0 = p->gain0;
    c.qe_f = (float)p->qe;
    c.background_f = (float)p->background;
    c.readout_f = (float)p->readout_noise;
    c.emgain_f = (float)p->emgain;
    c.fullwell_f = (float)p->fullwell;
    c.adc_max_f = (float)c.adc_max;
    c.offset0_f = (float)p->offset0;
    c.inv_gain0_f = (float)(1.0 / p->gain0);
    c.seed = p->seed;
    c.counter = p->counter;
    c.frame = p->d_frame;
    c.photons64 = p->d_photons64;
    c.expect64 = p->d_expect64;
    cudaStream_t st = sc::as_stream(stream);
    if (p->exact) {
        const int block = 256;
        int grid = (c.n + block - 1) / block;
        if (grid > 152 * 16) grid = 152 * 16;
        camera_exact_kernel<<<grid, block, 0, st>>>(c, d_photons, d_offset, d_gain, d_table_value,
                                                    d_table_cdf, d_inj_noise, d_inj_signal,
                                                    d_inj_uniform, d_expect, d_adc64, d_adc32);
    } else {
        // chunks of 32 * per pixels per warp, 8 per lane once the frame fills
        // the GPU's resident threads (152 SMs x 2048) 8 times; below twice, a
        // pixel per thread
        int per = (int)((int64_t)c.n / (152 * 2048));
        if (per < 2) {
            const int block = 256;
            int grid = (c.n + block - 1) / block;
            if (grid > 152 * 16) grid = 152 * 16;
            camera_pixel_kernel<<<grid, block, 0, st>>>(c, d_photons, d_offset_f, d_inv_gain_f,
                                                        d_sigma, d_table_value, d_table_cdf,
                                                        d_expect, d_adc64, d_adc32, d_status);
            return sc::launch_status("sc_camera");
        }
        per = per > kCamMaxPer ? kCamMaxPer : per;
        // at most one wave of resident blocks: the chunks are strided over the
        // grid, so a second wave would start late and finish late
        static int resident = 0;
        if (resident == 0) {
            int b = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, camera_native_kernel,
                                                              kCamThreads, 0) != cudaSuccess ||
                b < 1)
                b = 1;
            resident = b;
        }
        const int64_t chunks = ((int64_t)c.n + 32 * per - 1) / (32 * per);
        const int64_t blocks = (chunks + kCamThreads / 32 - 1) / (kCamThreads / 32);
        const int64_t wave = (int64_t)152 * resident;
        const int grid = (int)(blocks < wave ? blocks : wave);
        camera_native_kernel<<<grid, kCamThreads, 0, st>>>(
            c, per, d_photons, d_offset_f, d_inv_gain_f, d_sigma, d_table_value, d_table_cdf,
            d_expect, d_adc64, d_adc32, d_status);
    }
    return sc::launch_status("sc_camera");
}

extern "C" int sc_emccd_exact(const double *d_photons, double qe, double background,
                              const double *d_uniform, int n_pixels, double emgain,
                              double *d_signal, int32_t *d_status, void *stream) {
    SC_REQUIRE(n_pixels >= 0, "sc_emccd_exact: n_pixels=%d", n_pixels);
    SC_REQUIRE(emgain >= 1 && emgain == floor(emgain),
               "sc_emccd_exact: emgain must be a positive integer (got %g)", emgain);
    if (n_pixels == 0) return SC_OK;
    SC_REQUIRE(d_photons && d_uniform && d_signal, "sc_emccd_exact: NULL pointer");
    const int block = 256;
    int grid = (n_pixels * 32 + block - 1) / block;
    if (grid > 152 * 8) grid = 152 * 8;
    emccd_exact_kernel<<<grid, block, 0, sc::as_stream(stream)>>>(d_photons, qe, background,
                                                                  d_uniform, n_pixels, emgain,
                                                                  d_signal, d_status);
    return sc::launch_status("sc_emccd_exact");
}
