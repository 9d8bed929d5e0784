// PSF tables: radial profiles per depth key (FP64) and the quadrant
// summed-area tables the splat reads (double-float pairs).
//
// Radial profile, reference src/scopyon/_epifm.py:181-213 (Born-Wolf) and
// :133-134 (Gaussian).  Cartesian grid, reference :99-126: the (2n-1)^2 grid
// P[a][b] = interp(radial, psf)(min(sqrt(((a-c) res)^2 + ((b-c) res)^2), rmax))
// with c = n-1.  P is mirror-symmetric about c along each axis, so only the
// quadrant Q[p][q] = P[c+p][c+q] is tabulated, as its exclusive prefix sum
// G[u][v] = sum_{p<u, q<v} Q[p][q]; any footprint rectangle of P is a signed
// sum of G entries (see splat.cu).
#include "sc_common.cuh"
#include "fold.cuh"

namespace {

constexpr int kBornWolfTerms = 100;

__global__ void radial_born_wolf_kernel(double wavelength, double na, const double *depths,
                                        int n_r, double res, double *out) {
    __shared__ double ph_re[kBornWolfTerms], ph_im[kBornWolfTerms], rho_s[kBornWolfTerms];
    const int key = blockIdx.y;
    const double z = depths[key];
    const double k = 2.0 * M_PI / wavelength;
    const double alpha = k * na;
    const double half = na / 2;
    const double gamma = k * (half * half);
    const double drho = 1.0 / kBornWolfTerms;
    for (int t = threadIdx.x; t < kBornWolfTerms; t += blockDim.x) {
        const double rho = (double)(t + 1) * drho;
        // phase exp(-2 i z gamma rho^2), evaluated in the reference's product order
        const double theta = (((-2.0 * z) * gamma) * rho) * rho;
        double s, c;
        sincos(theta, &s, &c);
        ph_re[t] = (c * rho) * drho;
        ph_im[t] = (s * rho) * drho;
        rho_s[t] = rho;
    }
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_r) return;
    const double r = (double)i * res;
    const double ra = r * alpha;
    double sre = 0.0, sim = 0.0;
    for (int t = 0; t < kBornWolfTerms; ++t) {
        const double j = j0(ra * rho_s[t]);
        sre += ph_re[t] * j;
        sim += ph_im[t] * j;
    }
    const double mag = hypot(sre, sim);
    out[(size_t)key * n_r + i] = (mag * mag) * (alpha * alpha / M_PI);
}

__global__ void radial_gaussian_kernel(double sigma, int n_keys, int n_r, double res,
                                       double *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_r) return;
    const double r = (double)i * res;
    const double q = r / sigma;
    const double v = exp(-0.5 * (q * q)) / (2 * M_PI * sigma * sigma);
    for (int key = blockIdx.y; key < n_keys; key += gridDim.y) out[(size_t)key * n_r + i] = v;
}

// Block-wide inclusive scan of one double per thread (blockDim.x == 1024).
__device__ double block_inclusive_scan(double v, double *warp_tot) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        double n = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += n;
    }
    if (lane == 31) warp_tot[warp] = v;
    __syncthreads();
    if (warp == 0) {
        double t = warp_tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            double n = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += n;
        }
        warp_tot[lane] = t;
    }
    __syncthreads();
    if (warp > 0) v += warp_tot[warp - 1];
    __syncthreads();
    return v;
}

constexpr int kSatThreads = 1024;
constexpr int kSatMaxCols = 4;  // columns per thread: n_r <= 4096

// One CTA per depth key.  Row by row over p, each thread keeps running column
// sums of its columns; a block scan across columns turns them into G[p+1][.].
__global__ void __launch_bounds__(kSatThreads)
quadrant_sat_kernel(const double *radial, int n_r, double res, float *sat, int pitch) {
    extern __shared__ double y_s[];  // n_r radial values
    __shared__ double warp_tot[32];
    const int key = blockIdx.x;
    const double *y = radial + (size_t)key * n_r;
    for (int i = threadIdx.x; i < n_r; i += blockDim.x) y_s[i] = y[i];
    __syncthreads();
    float2 *g = reinterpret_cast<float2 *>(sat) + (size_t)key * (n_r + 1) * pitch;
    const int cols = (n_r + kSatThreads - 1) / kSatThreads;
    const int q0 = threadIdx.x * cols;
    const double rmax = (double)(n_r - 1) * res;
    double colsum[kSatMaxCols];
#pragma unroll
    for (int c = 0; c < kSatMaxCols; ++c) colsum[c] = 0.0;
    // row u = 0 is all zeros, as is column v = 0
    for (int v = threadIdx.x; v <= n_r; v += blockDim.x) g[v] = make_float2(0.f, 0.f);
    for (int p = 0; p < n_r; ++p) {
        const double dp = (double)p * res;
        double local = 0.0;
        double pref[kSatMaxCols];
#pragma unroll
        for (int c = 0; c < kSatMaxCols; ++c) {
            const int q = q0 + c;
            double val = 0.0;
            if (c < cols && q < n_r) {
                const double dq = (double)q * res;
                double rr = sqrt(dq * dq + dp * dp);
                if (rr > rmax) rr = rmax;
                // searchsorted(left) on r_i = i * res, then clip to [1, n_r - 1]
                int hi = (int)ceil(rr / res);
                if (hi > n_r) hi = n_r;
                while (hi > 0 && (double)(hi - 1) * res >= rr) --hi;
                while (hi < n_r && (double)hi * res < rr) ++hi;
                if (hi < 1) hi = 1;
                if (hi > n_r - 1) hi = n_r - 1;
                const int lo = hi - 1;
                const double x_lo = (double)lo * res, x_hi = (double)hi * res;
                val = ((rr - x_lo) / (x_hi - x_lo)) * y_s[hi] + ((x_hi - rr) / (x_hi - x_lo)) * y_s[lo];
                colsum[c] += val;
                local += colsum[c];
            }
            pref[c] = local;
        }
        const double incl = block_inclusive_scan(local, warp_tot);
        const double excl = incl - local;
        float2 *row = g + (size_t)(p + 1) * pitch;
        if (threadIdx.x == 0) row[0] = make_float2(0.f, 0.f);
#pragma unroll
        for (int c = 0; c < kSatMaxCols; ++c) {
            const int q = q0 + c;
            if (c < cols && q < n_r) {
                const double G = excl + pref[c];
                const float h = (float)G;
                row[q + 1] = make_float2(h, (float)(G - (double)h));
            }
        }
    }
}

// Box table: entry (key, r_x, r_y, q_x, q_y) is the grid sum over rows
// [m_x, m_x + P) and columns [m_y, m_y + P) clipped to [0, 2n-1), where
// m = q * P + r - P.  Each sum is a signed combination of quadrant-table
// entries, accumulated in FP64 and rounded once to FP32.
__global__ void box_table_kernel(const float2 *__restrict__ sat, int n_r, int pitch, int P,
                                 int nq, float *__restrict__ box) {
    const int key = blockIdx.y;
    const int n_signal = 2 * n_r - 1;
    const float2 *G = sat + (size_t)key * (n_r + 1) * pitch;
    const int nb = SC_BOX_BLOCK_FLOATS(nq);
    const int per_key = P * P * nb;  // < 2^31 for any grid the API accepts
    float *out = box + (size_t)key * per_key;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < per_key; e += gridDim.x * blockDim.x) {
        const int inner = e % nb, phase = e / nb;
        if (inner >= nq * nq) {  // block padding
            out[e] = 0.f;
            continue;
        }
        const int qy = inner % nq, qx = inner / nq;
        const int ry = phase % P;
        const int rx = phase / P;
        int a0 = qx * P + rx - P, b0 = qy * P + ry - P;
        int a1 = min(a0 + P, n_signal), b1 = min(b0 + P, n_signal);
        a0 = max(a0, 0);
        b0 = max(b0, 0);
        double v = 0.0;
        if (a1 > a0 && b1 > b0) {
            int uu[3], vv[3];
            float us[3], vs[3];
            const int nu = sc::fold(a0, a1, n_r, uu, us);
            const int nv = sc::fold(b0, b1, n_r, vv, vs);
            for (int iu = 0; iu < nu; ++iu) {
                const float2 *row = G + (size_t)uu[iu] * pitch;
                for (int iv = 0; iv < nv; ++iv) {
                    const float2 g = row[vv[iv]];
                    v += (double)(us[iu] * vs[iv]) * ((double)g.x + (double)g.y);
                }
            }
        }
        out[e] = (float)v;
    }
}

}  // namespace

extern "C" int sc_psf_radial(int kind, double wavelength, double na, double sigma,
                             const double *d_depths, int n_keys, int n_r, double res,
                             double *d_radial, void *stream) {
    SC_REQUIRE(n_keys > 0 && n_keys <= 65535, "sc_psf_radial: n_keys=%d out of range", n_keys);
    SC_REQUIRE(n_r >= 2 && n_r <= 4096, "sc_psf_radial: n_r=%d out of range [2, 4096]", n_r);
    SC_REQUIRE(res > 0, "sc_psf_radial: res must be positive");
    SC_REQUIRE(d_radial != nullptr, "sc_psf_radial: output is NULL");
    dim3 block(256), grid((n_r + 255) / 256, n_keys);
    if (kind == SC_PSF_BORN_WOLF) {
        SC_REQUIRE(wavelength > 0 && na > 0, "sc_psf_radial: wavelength and NA must be positive");
        SC_REQUIRE(d_depths != nullptr, "sc_psf_radial: depths are NULL");
        radial_born_wolf_kernel<<<grid, block, 0, sc::as_stream(stream)>>>(
            wavelength, na, d_depths, n_r, res, d_radial);
    } else if (kind == SC_PSF_GAUSSIAN) {
        SC_REQUIRE(sigma > 0, "sc_psf_radial: Gaussian radial_width must be positive");
        grid.y = n_keys < 1024 ? n_keys : 1024;
        radial_gaussian_kernel<<<grid, block, 0, sc::as_stream(stream)>>>(sigma, n_keys, n_r, res,
                                                                         d_radial);
    } else {
        sc::set_error("sc_psf_radial: unknown PSF kind %d", kind);
        return SC_ERR_ARG;
    }
    return sc::launch_status("sc_psf_radial");
}

extern "C" int sc_psf_quadrant_sat(const double *d_radial, int n_keys, int n_r, double res,
                                   float *d_sat, int sat_pitch, void *stream) {
    SC_REQUIRE(n_keys > 0, "sc_psf_quadrant_sat: n_keys=%d", n_keys);
    SC_REQUIRE(n_r >= 2 && n_r <= kSatThreads * kSatMaxCols,
               "sc_psf_quadrant_sat: n_r=%d out of range", n_r);
    SC_REQUIRE(sat_pitch >= n_r + 1, "sc_psf_quadrant_sat: pitch %d < n_r + 1", sat_pitch);
    SC_REQUIRE(d_radial && d_sat, "sc_psf_quadrant_sat: NULL pointer");
    size_t smem = (size_t)n_r * sizeof(double);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(quadrant_sat_kernel,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return sc::cuda_status(e, "sc_psf_quadrant_sat: smem attribute");
    }
    quadrant_sat_kernel<<<n_keys, kSatThreads, smem, sc::as_stream(stream)>>>(d_radial, n_r, res,
                                                                            d_sat, sat_pitch);
    return sc::launch_status("sc_psf_quadrant_sat");
}

extern "C" int sc_psf_box_table(const float *d_sat, int n_keys, int n_r, int sat_pitch, int box_p,
                                float *d_box, void *stream) {
    SC_REQUIRE(n_keys > 0 && n_keys <= 65535, "sc_psf_box_table: n_keys=%d", n_keys);
    SC_REQUIRE(n_r >= 2 && sat_pitch >= n_r + 1, "sc_psf_box_table: n_r=%d pitch=%d", n_r,
               sat_pitch);
    SC_REQUIRE(box_p >= 1 && box_p <= 4096, "sc_psf_box_table: P=%d out of range", box_p);
    SC_REQUIRE(d_sat && d_box, "sc_psf_box_table: NULL pointer");
    const int n_signal = 2 * n_r - 1;
    const int nq = (n_signal + box_p - 1) / box_p + 1;
    dim3 grid(256, n_keys);
    box_table_kernel<<<grid, 256, 0, sc::as_stream(stream)>>>(
        reinterpret_cast<const float2 *>(d_sat), n_r, sat_pitch, box_p, nq, d_box);
    return sc::launch_status("sc_psf_box_table");
}
