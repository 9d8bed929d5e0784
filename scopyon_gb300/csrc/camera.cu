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
// Draws come either from Philox4x32-10 (native, one counter block per pixel pair)
// or from caller arrays recorded from the reference (injected), in which case
// the ADC arithmetic is the reference's FP64 sequence.
#include "sc_common.cuh"
#include "camera.cuh"

namespace {

using namespace sc::cam;

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

int64_t pois_entries() {
    int64_t n = 0;
    for (int j = 0; j < kPoisJ; ++j) n += pois_support(j);
    return n;
}

// One thread per j: the span, then the CDF summed in FP64 from
// p_k = exp(k log j - j - log k!), as 32-bit fixed point.
__global__ void pois_cdf_kernel(void *base) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= kPoisJ) return;
    char *b = static_cast<char *>(base);
    int2 *span = reinterpret_cast<int2 *>(b);
    uint32_t *cdf = reinterpret_cast<uint32_t *>(b + kPoisCdfAt);
    int o = 0;
    for (int i = 0; i < j; ++i) o += pois_support(i);
    const int K = pois_support(j);
    span[j] = make_int2(o, K - 1);
    const double lj = j > 0 ? log((double)j) : 0.0;
    double F = 0.0;
    for (int k = 0; k < K; ++k) {
        const double pk = j == 0 ? (k == 0 ? 1.0 : 0.0)
                                 : exp((double)k * lj - (double)j - lgamma((double)k + 1.0));
        F += pk;
        cdf[o + k] = k == K - 1 ? 0u : (uint32_t)fmin(rint(F * 4294967296.0), 4294967295.0);
    }
}

// One thread per (j, g): the first k below K_j - 1 whose upper edge lies
// above g 2^24, else K_j - 1.
__global__ void pois_guide_kernel(void *base) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= kPoisJ * kPoisG) return;
    const int j = idx / kPoisG, g = idx % kPoisG;
    char *b = static_cast<char *>(base);
    const int2 sp = reinterpret_cast<const int2 *>(b)[j];
    uint16_t *guide = reinterpret_cast<uint16_t *>(b + kPoisGuideAt);
    const uint32_t *cdf = reinterpret_cast<const uint32_t *>(b + kPoisCdfAt) + sp.x;
    const uint32_t target = (uint32_t)g << 24;
    int k = 0;
    while (k < sp.y && cdf[k] <= target) ++k;
    guide[idx] = (uint16_t)k;
}

// The per-pixel inputs of pixel pair q (photons, read-noise sigma, 1/gain,
// offset): float2 loads when VEC, else two scalar loads (the last pair of an
// odd frame repeats its one pixel).
struct PairIn {
    float2 ph, sg, g, o;
};

template <int CAM, bool VEC>
__device__ __forceinline__ PairIn load_pair(const CamConsts &c, int q,
                                            const float *__restrict__ photons,
                                            const float *__restrict__ offset_f,
                                            const float *__restrict__ inv_gain_f,
                                            const float *__restrict__ sigma) {
    // streamed once: loaded evict-first, so that the Poisson tables keep L1
    const bool scmos = CAM == SC_CAM_SCMOS && sigma;
    PairIn in;
    if (VEC) {
        in.ph = __ldcs(reinterpret_cast<const float2 *>(photons) + q);
        in.sg = scmos ? __ldcs(reinterpret_cast<const float2 *>(sigma) + q)
                      : make_float2(c.readout_f, c.readout_f);
        in.g = inv_gain_f ? __ldcs(reinterpret_cast<const float2 *>(inv_gain_f) + q)
                          : make_float2(c.inv_gain0_f, c.inv_gain0_f);
        in.o = offset_f ? __ldcs(reinterpret_cast<const float2 *>(offset_f) + q)
                        : make_float2(c.offset0_f, c.offset0_f);
    } else {
        const int p = 2 * q, p1 = min(p + 1, c.n - 1);
        in.ph = make_float2(__ldcs(photons + p), __ldcs(photons + p1));
        in.sg = scmos ? make_float2(__ldcs(sigma + p), __ldcs(sigma + p1))
                      : make_float2(c.readout_f, c.readout_f);
        in.g = inv_gain_f ? make_float2(__ldcs(inv_gain_f + p), __ldcs(inv_gain_f + p1))
                          : make_float2(c.inv_gain0_f, c.inv_gain0_f);
        in.o = offset_f ? make_float2(__ldcs(offset_f + p), __ldcs(offset_f + p1))
                        : make_float2(c.offset0_f, c.offset0_f);
    }
    return in;
}

// Native draws, a pixel pair per thread (pixels 2q and 2q + 1, one Philox
// block between them; see pair_draws).  VEC: the per-pixel inputs and the
// FP32 outputs are 8-byte aligned and the frame has an even pixel count, so
// a pair's values move as float2.  Each thread loads its next pair's inputs
// before it draws the current pair, so that a load's DRAM latency overlaps
// a pair's arithmetic.  No lane loops on a rejection in the common case, so
// a warp's lanes stay together.
#ifndef SC_CAM_MIN_BLOCKS
#define SC_CAM_MIN_BLOCKS 1
#endif
template <int CAM, bool VEC>
__global__ void __launch_bounds__(256, SC_CAM_MIN_BLOCKS)
camera_native_kernel(CamConsts c, const void *__restrict__ ptab, const float *__restrict__ photons,
                     const float *__restrict__ offset_f, const float *__restrict__ inv_gain_f,
                     const float *__restrict__ sigma, const double *__restrict__ table_value,
                     const double *__restrict__ table_cdf, float *__restrict__ expect,
                     double *__restrict__ adc64, float *__restrict__ adc32, int32_t *status) {
    const PoisTab t = pois_tab(ptab);
    const uint64_t counter = c.counter + (c.frame ? (uint64_t)*c.frame : 0);
    const uint32_t c0 = (uint32_t)counter, c1 = (uint32_t)(counter >> 32);
    const int n_pairs = (c.n + 1) >> 1;
    const int stride = gridDim.x * blockDim.x;
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n_pairs) return;
    PairIn in = load_pair<CAM, VEC>(c, q, photons, offset_f, inv_gain_f, sigma);
    for (; q < n_pairs; q += stride) {
        const int qn = q + stride;
        PairIn next = in;
        if (qn < n_pairs) next = load_pair<CAM, VEC>(c, qn, photons, offset_f, inv_gain_f, sigma);
        const PairDraws d = pair_draws<CAM>(c, q, c0, c1);
        const int p = 2 * q;
        const float e0 = c.qe_f * (in.ph.x + c.background_f);
        const float e1 = c.qe_f * (in.ph.y + c.background_f);
        const float v0 = pixel_adc<CAM>(c, t, p, e0, in.sg.x, in.g.x, in.o.x, d, 0, c0, c1,
                                        table_value, table_cdf, status);
        const bool two = VEC || p + 1 < c.n;
        const float v1 = two ? pixel_adc<CAM>(c, t, p + 1, e1, in.sg.y, in.g.y, in.o.y, d, 1, c0,
                                              c1, table_value, table_cdf, status)
                             : 0.f;
        if (VEC) {
            if (expect) __stcs(reinterpret_cast<float2 *>(expect) + q, make_float2(e0, e1));
            if (adc32) __stcs(reinterpret_cast<float2 *>(adc32) + q, make_float2(v0, v1));
        } else {
            if (expect) expect[p] = e0;
            if (adc32) adc32[p] = v0;
            if (two) {
                if (expect) expect[p + 1] = e1;
                if (adc32) adc32[p + 1] = v1;
            }
        }
        if (adc64) {
            adc64[p] = sc::f2d_exact(v0);
            if (two) adc64[p + 1] = sc::f2d_exact(v1);
        }
        in = next;
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

namespace sc {
namespace cam {

int cam_consts(const ScCameraParams *p, CamConsts &c) {
    SC_REQUIRE(p != nullptr, "camera params are NULL");
    SC_REQUIRE(p->bit > 0 && p->bit <= 32, "camera: bit=%d", p->bit);
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
    return SC_OK;
}

}  // namespace cam
}  // namespace sc

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
    if (!p->exact)
        SC_REQUIRE(p->d_poisson_table != nullptr,
                   "sc_camera: native draws need the Poisson tables (sc_poisson_table)");
    if (p->exact) {
        SC_REQUIRE(d_inj_signal != nullptr, "sc_camera: exact mode needs injected signal");
        SC_REQUIRE(p->camera == SC_CAM_CMOS_TABLE ? (d_inj_uniform || d_inj_noise) : true,
                   "sc_camera: CMOS exact mode needs injected uniforms or noise");
    }
    CamConsts c;
    int rc = sc::cam::cam_consts(p, c);
    if (rc) return rc;
    cudaStream_t st = sc::as_stream(stream);
    if (p->exact) {
        const int block = 256;
        int grid = (c.n + block - 1) / block;
        if (grid > 152 * 16) grid = 152 * 16;
        camera_exact_kernel<<<grid, block, 0, st>>>(c, d_photons, d_offset, d_gain, d_table_value,
                                                    d_table_cdf, d_inj_noise, d_inj_signal,
                                                    d_inj_uniform, d_expect, d_adc64, d_adc32);
    } else {
        const int block = 256;
        const int64_t want = (((int64_t)c.n + 1) / 2 + block - 1) / block;
        auto al8 = [](const void *ptr) { return ((uintptr_t)ptr & 7) == 0; };
        const bool vec = (c.n & 1) == 0 && al8(d_photons) && al8(d_offset_f) &&
                         al8(d_inv_gain_f) && al8(d_sigma) && al8(d_expect) && al8(d_adc32);
        switch (c.camera * 2 + (vec ? 1 : 0)) {
#define SC_CAM_LAUNCH(K, V)                                                                       \
    case K * 2 + V:                                                                             \
        camera_native_kernel<K, V><<<sc::resident_grid((const void *)camera_native_kernel<K, V>, \
                                                       block, 0, want),                         \
                                      block, 0, st>>>(                                          \
            c, p->d_poisson_table, d_photons, d_offset_f, d_inv_gain_f, d_sigma, d_table_value,   \
            d_table_cdf, d_expect, d_adc64, d_adc32, d_status);                                   \
        break;
            SC_CAM_LAUNCH(SC_CAM_EMCCD, 0)
            SC_CAM_LAUNCH(SC_CAM_EMCCD, 1)
            SC_CAM_LAUNCH(SC_CAM_CCD, 0)
            SC_CAM_LAUNCH(SC_CAM_CCD, 1)
            SC_CAM_LAUNCH(SC_CAM_CMOS_TABLE, 0)
            SC_CAM_LAUNCH(SC_CAM_CMOS_TABLE, 1)
            SC_CAM_LAUNCH(SC_CAM_SCMOS, 0)
            SC_CAM_LAUNCH(SC_CAM_SCMOS, 1)
#undef SC_CAM_LAUNCH
        }
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

extern "C" size_t sc_poisson_table_bytes(void) {
    return kPoisCdfAt + sizeof(uint32_t) * (size_t)pois_entries();
}

extern "C" int sc_poisson_table(void *d_table, size_t bytes, void *stream) {
    SC_REQUIRE(d_table != nullptr, "sc_poisson_table: NULL buffer");
    SC_REQUIRE_CAP(bytes >= sc_poisson_table_bytes(), "sc_poisson_table: buffer %zu < %zu bytes",
                   bytes, sc_poisson_table_bytes());
    SC_REQUIRE(((uintptr_t)d_table & 15) == 0, "sc_poisson_table: buffer not 16-byte aligned");
    cudaStream_t st = sc::as_stream(stream);
    pois_cdf_kernel<<<1, kPoisJ, 0, st>>>(d_table);
    pois_guide_kernel<<<(kPoisJ * kPoisG + 255) / 256, 256, 0, st>>>(d_table);
    return sc::launch_status("sc_poisson_table");
}
