// Camera draws of one pixel, shared by the camera kernels (camera.cu) and the
// persistent batched-frame kernel (splat.cu).  See camera.cu for the models
// and their reference lines (src/scopyon/_epifm.py:329-433, :1430-1484).
#pragma once

#include "sc_common.cuh"

namespace sc {
namespace cam {

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
__device__ inline float poisson(sc::rng_stream &rs, float lam, int32_t *status) {
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
__device__ inline float gamma_ge1(sc::rng_stream &rs, float shape, int32_t *status) {
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

// ------------------------------------------------ Poisson inverse-CDF tables
// Poisson(j) for j = 0 .. kPoisJ - 1 over k = 0 .. K_j - 1 as 32-bit fixed
// point: C_j[k] = F_j(k) 2^32, rounded from the FP64 sum (the last entry,
// whose upper edge is 2^32, is stored as 0 and never compared), and per j
// kPoisG starting points for the search (the first k with C_j[k] above
// g 2^24).  Layout of the caller's buffer: int2 {first entry, K_j - 1}
// [kPoisJ], uint16 guide [kPoisJ][kPoisG], uint32 CDF [sum K_j].
constexpr int kPoisJ = 256, kPoisG = 256;
constexpr size_t kPoisGuideAt = sizeof(int2) * kPoisJ;
constexpr size_t kPoisCdfAt = kPoisGuideAt + sizeof(uint16_t) * kPoisJ * kPoisG;

// Support of the Poisson(j) table: j + 10 sqrt(j) + 12 values (the mass past
// it, below 1e-20, is far below one step of 2^-32).
__host__ __device__ __forceinline__ int pois_support(int j) {
    return j + (int)ceil(10.0 * sqrt((double)j)) + 12;
}

struct PoisTab {
    const int2 *span;
    const uint16_t *guide;
    const uint32_t *cdf;
};

__device__ __forceinline__ PoisTab pois_tab(const void *base) {
    const char *b = static_cast<const char *>(base);
    return PoisTab{reinterpret_cast<const int2 *>(b),
                   reinterpret_cast<const uint16_t *>(b + kPoisGuideAt),
                   reinterpret_cast<const uint32_t *>(b + kPoisCdfAt)};
}

// Poisson(lam) from one 32-bit uniform word u, with no rejection.  A sum of
// independent Poisson variates is Poisson with the summed mean, so the draw
// is K + M with K ~ Poisson(j), j = floor(lam), and M ~ Poisson(lam - j):
//   K: inversion of the fixed-point CDF, C_j[K - 1] <= u < C_j[K];
//   M: sequential inversion at v = (u - C_j[K - 1] + 1/2) / (C_j[K] -
//      C_j[K - 1]), which, given K, is uniform on (0, 1) and independent of
//      K, to within one step of the bin's width (a bin of probability p holds
//      p 2^32 values of u).
// Means of kPoisJ and more take PTRS on the pixel's fallback stream.
// The caller takes means of kPoisJ and more (and NaN) elsewhere.
__device__ __forceinline__ float poisson_u32(const PoisTab &t, float lam, uint32_t u) {
    if (!(lam > 0.f)) return 0.f;
    const int j = (int)lam;
    const float r = lam - (float)j;
    int k = 0;
    float v;
    if (j > 0) {
        const int2 sp = __ldg(t.span + j);
        const uint32_t *cdf = t.cdf + sp.x;
        k = __ldg(t.guide + j * kPoisG + (u >> 24));
        uint32_t lo = k > 0 ? __ldg(cdf + k - 1) : 0u;
        uint32_t hi = __ldg(cdf + k);
        while (k < sp.y && u >= hi) {
            lo = hi;
            hi = __ldg(cdf + ++k);
        }
        // the bin's width (mod 2^32: the last bin's upper edge 2^32 is stored as 0)
        const uint32_t w = hi - lo;
        v = fminf(__fdividef((float)(u - lo) + 0.5f, (float)w), 0.99999994f);
    } else {
        v = sc::u01f(u);
    }
    // Poisson(r), r in [0, 1): the first four cumulative sums without a
    // branch (v lies past the fourth with probability below 2%), then the
    // sequential search (P(M >= 16) < 1e-13)
    float p = __expf(-r), s = p;
    int m = v > s;
    p *= r;
    s += p;
    m += v > s;
    p *= 0.5f * r;
    s += p;
    m += v > s;
    p *= (1.f / 3.f) * r;
    s += p;
    if (v > s) {
        m = 4;
        p *= 0.25f * r;
        s += p;
        while (v > s && m < 16) {
            ++m;
            p *= __fdividef(r, (float)m);
            s += p;
        }
    }
    return (float)(k + m);
}

// Two independent standard normals from two 32-bit words (Box-Muller: the
// cosine and the sine branch).  The radius is x rsqrt(x) (relative error a
// few 1e-7, far below what any test of the draws resolves), with x kept
// above 0: u01f rounds its largest values to 1, and x rsqrt(x) of 0 is 0 * inf.
__device__ __forceinline__ void bm_pair(uint32_t a, uint32_t b, float &n0, float &n1) {
    const float x = fmaxf(-2.0f * __logf(sc::u01f(a)), 1e-30f);
    const float r = x * rsqrtf(x);
    float sn, cs;
    sc::sincos_2pi(sc::u01f(b), &sn, &cs);
    n0 = r * cs;
    n1 = r * sn;
}

// Uniform in (0, 1) from one 32-bit word, double precision.
__device__ __forceinline__ double u01d32(uint32_t x) {
    return ((double)x + 0.5) * (1.0 / 4294967296.0);
}

// EMCCD output electrons with the reference's law (EMCCD.probability_
// distribution, _epifm.py:365-400): S = 0 with the weight of no
// photo-electron, S >= 1 with weight proportional to the Poisson-gamma density
// at S, on the support [g floor(E - sigma), g floor(E + sigma)), sigma =
// 5 sqrt(E) + 10.  Drawn as n ~ Poisson(E), S = rint(g Gamma(n)) for n > 0,
// and drawn again when S leaves the support or rounds to 0 with n > 0 (the
// law has no density mass below S = 1/2 beside the atom at 0).
__device__ inline float emccd_native(const PoisTab &t, float e, float g, uint32_t u,
                                     sc::rng_stream &rs, int32_t *status) {
    if (!(e > 0.f)) return 0.f;
    const float sig = sqrtf(e) * 5.f + 10.f;
    const float s_min = fmaxf(0.f, g * truncf(e - sig)), s_max = g * truncf(e + sig);
    for (int it = 0; it < 32; ++it) {
        const uint32_t w = it == 0 ? u : rs.next();
        const float n = e < (float)kPoisJ ? poisson_u32(t, e, w) : poisson(rs, e, status);
        const float s = n > 0.f ? rintf(g * gamma_ge1(rs, n, status)) : 0.f;
        if (n > 0.f && s < 1.f) continue;
        if (s >= s_min && s < s_max) return s;
    }
    sc::flag_status(status, 3, 2, 0, 0);
    return rintf(g * e);
}

// Native draws.  Pixels 2q and 2q + 1 share one Philox4x32-10 block (key:
// the seed; counter: (q, frame counter, 0)): word x is pixel 2q's Poisson
// word and y pixel 2q + 1's; z and w give the pair's read noise, the cosine
// branch of Box-Muller to pixel 2q and the sine branch to 2q + 1 (the CMOS
// table's noise: word z, resp. w, as one uniform).  Pixel p's rare fallbacks
// (PTRS above kPoisJ, the EMCCD gain and its redraws) use its own stream,
// counter (p, frame counter, 1, 2, ...).  So a pixel's counts depend on its
// index and the frame only, never on the launch shape.
struct PairDraws {
    uint32_t pois[2], word[2];
    float normal[2];
};

template <int CAM>
__device__ __forceinline__ PairDraws pair_draws(const CamConsts &c, int q, uint32_t c0,
                                                uint32_t c1) {
    const sc::u4 r = sc::philox4x32_10(sc::u4{(uint32_t)q, c0, c1, 0u}, (uint32_t)c.seed,
                                       (uint32_t)(c.seed >> 32));
    PairDraws d;
    d.pois[0] = r.x;
    d.pois[1] = r.y;
    d.word[0] = r.z;
    d.word[1] = r.w;
    d.normal[0] = d.normal[1] = 0.f;
    if (CAM != SC_CAM_CMOS_TABLE) bm_pair(r.z, r.w, d.normal[0], d.normal[1]);
    return d;
}

// Poisson(lam) for means of kPoisJ and more (PTRS) on pixel p's fallback
// stream.
__device__ __forceinline__ float poisson_far(uint64_t seed, int p, uint32_t c0, uint32_t c1,
                                          float lam, int32_t *status) {
    sc::rng_stream rs(seed, (uint32_t)p, c0, c1);
    rs.ctr.w = 1;
    return poisson(rs, lam, status);
}

// The ADC count of pixel p in native mode: expectation ef, read-noise sigma
// sg, 1/gain g and offset o, with the pixel's half h of its pair's draws.
template <int CAM>
__device__ __forceinline__ float pixel_adc(const CamConsts &c, const PoisTab &t, int p, float ef,
                                           float sg, float g, float o, const PairDraws &d, int h,
                                           uint32_t c0, uint32_t c1,
                                           const double *__restrict__ table_value,
                                           const double *__restrict__ table_cdf,
                                           int32_t *status) {
    float signal, noise;
    if (CAM == SC_CAM_EMCCD) {
        sc::rng_stream rs(c.seed, (uint32_t)p, c0, c1);
        rs.ctr.w = 1;
        signal = emccd_native(t, ef, c.emgain_f, d.pois[h], rs, status);
        noise = c.readout_f > 0.f ? c.readout_f * d.normal[h] : 0.f;
    } else {
        signal = ef < (float)kPoisJ ? poisson_u32(t, ef, d.pois[h])
                                    : poisson_far(c.seed, p, c0, c1, ef, status);
        noise = CAM == SC_CAM_CMOS_TABLE
                    ? (float)table_value[table_index(table_cdf, c.table_n, u01d32(d.word[h]))]
                    : sg * d.normal[h];
    }
    float v = fminf(signal + noise, c.fullwell_f);
    v = fmaf(v, g, o);
    v = fminf(fmaxf(v, 0.f), c.adc_max_f);
    if (c.rounding) v = rintf(v);
    return v;
}

// The ADC count of one pixel p alone (its pair's block drawn for it).
template <int CAM>
__device__ __forceinline__ float native_adc(const CamConsts &c, const PoisTab &t, int p, float ef,
                                            float sg, float g, float o, uint64_t counter,
                                            const double *__restrict__ table_value,
                                            const double *__restrict__ table_cdf,
                                            int32_t *status) {
    const uint32_t c0 = (uint32_t)counter, c1 = (uint32_t)(counter >> 32);
    const PairDraws d = pair_draws<CAM>(c, p >> 1, c0, c1);
    return pixel_adc<CAM>(c, t, p, ef, sg, g, o, d, p & 1, c0, c1, table_value, table_cdf,
                          status);
}

// CamConsts of a parameter block (host).
int cam_consts(const ScCameraParams *p, CamConsts &c);

}  // namespace cam
}  // namespace sc
