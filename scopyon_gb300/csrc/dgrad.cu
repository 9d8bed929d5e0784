// Gradient through diffusion: Brownian sub-step positions regenerated from
// Philox counters, a Gaussian-approximated likelihood of the summed frame,
// and the reparameterised derivative with respect to the diffusion
// coefficient D.
//
// An emitter starting at p0 moves as p_t = p0 + s Z_t, s = sqrt(2 D dt),
// Z_t = n_0 + ... + n_{t-1} (the reference's move_points,
// src/scopyon/sampling.py:88-119, in 2-D); its photons I are spread evenly
// over the T sub-steps of the exposure (the unit_time weights of
// _epifm.py:1183-1199).  Since dp_t / dD = Z_t s / (2 D) = (p_t - p0) / (2 D),
//   dL/dD = sum_{e,t} (dL/dp_t) . (p_t - p0) / (2 D).
// The positions are regenerated from the same counters in the backward pass,
// so no trajectory is kept between the passes.
#include "sc_common.cuh"

namespace {

// Standard normals (x, y) of emitter e at sub-step t: FP32 Box-Muller on
// Philox4x32-10 words, counter (e, t, 0, 0xd1ff05e0).
__device__ __forceinline__ float2 step_normals(uint64_t seed, int e, int t) {
    const sc::u4 r = sc::philox4x32_10({(uint32_t)e, (uint32_t)t, 0u, 0xd1ff05e0u},
                                       (uint32_t)seed, (uint32_t)(seed >> 32));
    const float u1 = sc::u01f(r.x), u2 = sc::u01f(r.y);
    const float rad = sqrtf(-2.f * __logf(u1));
    float sn, cs;
    sc::sincos_2pi(u2, &sn, &cs);
    return make_float2(rad * cs, rad * sn);
}

// out[t][e] = (x_t, y_t, z, I / T) for t < T: one thread per emitter walks
// its chain.  normals (optional, [T][N][2]) replace the Philox draws.
__global__ void diffusion_positions_kernel(const float4 *__restrict__ emit, int n, int T,
                                           const float *__restrict__ D, float dt, uint64_t seed,
                                           const float *__restrict__ normals,
                                           float4 *__restrict__ out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const float4 p0 = emit[e];
    const float s = sqrtf(2.f * *D * dt);
    const float w = p0.w / (float)T;
    float zx = 0.f, zy = 0.f;  // Z_t
    for (int t = 0; t < T; ++t) {
        out[(size_t)t * n + e] = make_float4(fmaf(s, zx, p0.x), fmaf(s, zy, p0.y), p0.z, w);
        float2 nv;
        if (normals) {
            const float *q = normals + ((size_t)t * n + e) * 2;
            nv = make_float2(q[0], q[1]);
        } else {
            nv = step_normals(seed, e, t);
        }
        zx += nv.x;
        zy += nv.y;
    }
}

constexpr int kThreads = 256;
constexpr int kChunk = 1024;
constexpr int kMaxParts = 1216;  // 8 CTAs on each of 152 SMs

__device__ __forceinline__ double block_sum(double acc, double *part) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < kThreads / 32; ++w) t += part[w];
    return t;
}

int parts_of(int64_t n) {
    int64_t p = (n + kChunk - 1) / kChunk;
    return (int)(p < 1 ? 1 : (p > kMaxParts ? kMaxParts : p));
}

// Gaussian approximation of the camera likelihood per pixel, variance
// v = mu + r2 (shot noise plus the readout variance r2, per pixel or scalar):
//   L = sum (k - mu)^2 / (2 v) + log(v) / 2,
//   dL/dmu = -(k - mu) / v - (k - mu)^2 / (2 v^2) + 1 / (2 v).
__global__ void __launch_bounds__(kThreads)
gauss_nll_kernel(const float *__restrict__ mu, const float *__restrict__ k, int64_t n,
                 const float *__restrict__ r2_map, float r2, float *grad, double *partial) {
    __shared__ double part[kThreads / 32];
    const int parts = gridDim.x;
    double acc = 0.0;
    for (int64_t c0 = (int64_t)blockIdx.x * kChunk; c0 < n; c0 += (int64_t)parts * kChunk) {
        const int64_t c1 = c0 + kChunk < n ? c0 + kChunk : n;
        for (int64_t q = c0 + threadIdx.x; q < c1; q += kThreads) {
            const float m = mu[q], r = k[q] - m;
            const float v = m + (r2_map ? r2_map[q] : r2);
            const float iv = 1.f / v, hr = 0.5f * r * r * iv;
            // each pixel's term in FP32 (within a few ulp), summed in FP64
            acc += sc::f2d_exact(hr) + 0.5 * sc::f2d_exact(logf(v));
            if (grad) grad[q] = -r * iv - hr * iv + 0.5f * iv;
        }
    }
    const double t = block_sum(acc, part);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

// sum over (t, e) of gx (x_t - x0) + gy (y_t - y0), in FP64, per part.
__global__ void __launch_bounds__(kThreads)
dD_partial_kernel(const float4 *__restrict__ pos, const float4 *__restrict__ emit, int n,
                  int64_t total, const float4 *__restrict__ grad, double *partial) {
    __shared__ double part[kThreads / 32];
    const int parts = gridDim.x;
    double acc = 0.0;
    for (int64_t c0 = (int64_t)blockIdx.x * kChunk; c0 < total; c0 += (int64_t)parts * kChunk) {
        const int64_t c1 = c0 + kChunk < total ? c0 + kChunk : total;
        int e = (int)((c0 + threadIdx.x) % n);  // emitter of value q (q = t n + e)
        for (int64_t q = c0 + threadIdx.x; q < c1; q += kThreads) {
            const float4 p = pos[q], g = grad[q], p0 = emit[e];
            acc += sc::f2d_exact(g.x) * sc::f2d_exact(p.x - p0.x) +
                   sc::f2d_exact(g.y) * sc::f2d_exact(p.y - p0.y);
            e += kThreads;
            while (e >= n) e -= n;
        }
    }
    const double t = block_sum(acc, part);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

// out = scale * sum of partial[0 .. parts) (scale: 1, or 1 / (2 D)), one
// warp: lane l sums partials l, l + 32, ... in order, then a butterfly.
__global__ void finish_kernel(const double *partial, int parts, const float *D, double *out) {
    const int lane = threadIdx.x;
    double t = 0.0;
    for (int k = lane; k < parts; k += 32) t += partial[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) out[0] = D ? t / (2.0 * (double)*D) : t;
}

}  // namespace

extern "C" size_t sc_dgrad_scratch_bytes(int64_t n_values) {
    return (size_t)parts_of(n_values) * sizeof(double);
}

extern "C" int sc_diffusion_positions(const float *d_emit, int n, int T, const float *d_D, double dt,
                                      uint64_t seed, const float *d_normals, float *d_out,
                                      void *stream) {
    SC_REQUIRE(n >= 0 && T >= 1, "sc_diffusion_positions: n=%d T=%d", n, T);
    SC_REQUIRE((int64_t)n * T < (1ll << 31), "sc_diffusion_positions: too many positions");
    SC_REQUIRE(dt > 0, "sc_diffusion_positions: dt must be positive");
    if (n == 0) return SC_OK;
    SC_REQUIRE(d_emit && d_D && d_out, "sc_diffusion_positions: NULL pointer");
    diffusion_positions_kernel<<<(n + 127) / 128, 128, 0, sc::as_stream(stream)>>>(
        reinterpret_cast<const float4 *>(d_emit), n, T, d_D, (float)dt, seed, d_normals,
        reinterpret_cast<float4 *>(d_out));
    return sc::launch_status("sc_diffusion_positions");
}

extern "C" int sc_gauss_nll(const float *d_mu, const float *d_counts, int64_t n,
                            const float *d_var_map, double var, void *d_scratch,
                            size_t scratch_bytes, double *d_loss, float *d_grad_mu, void *stream) {
    SC_REQUIRE(n > 0, "sc_gauss_nll: n=%lld", (long long)n);
    SC_REQUIRE(d_mu && d_counts && d_loss, "sc_gauss_nll: NULL pointer");
    const int parts = parts_of(n);
    SC_REQUIRE_CAP(d_scratch && scratch_bytes >= (size_t)parts * sizeof(double),
               "sc_gauss_nll: scratch %zu < %zu bytes", scratch_bytes, (size_t)parts * sizeof(double));
    cudaStream_t s = sc::as_stream(stream);
    double *partial = static_cast<double *>(d_scratch);
    gauss_nll_kernel<<<parts, kThreads, 0, s>>>(d_mu, d_counts, n, d_var_map, (float)var,
                                                 d_grad_mu, partial);
    finish_kernel<<<1, 32, 0, s>>>(partial, parts, nullptr, d_loss);
    return sc::launch_status("sc_gauss_nll");
}

extern "C" int sc_diffusion_dD(const float *d_pos, const float *d_emit, int n, int T,
                               const float *d_grad_pos, const float *d_D, void *d_scratch,
                               size_t scratch_bytes, double *d_dD, void *stream) {
    SC_REQUIRE(n > 0 && T >= 1, "sc_diffusion_dD: n=%d T=%d", n, T);
    SC_REQUIRE(d_pos && d_emit && d_grad_pos && d_D && d_dD, "sc_diffusion_dD: NULL pointer");
    const int64_t total = (int64_t)n * T;
    const int parts = parts_of(total);
    SC_REQUIRE_CAP(d_scratch && scratch_bytes >= (size_t)parts * sizeof(double),
               "sc_diffusion_dD: scratch %zu < %zu bytes", scratch_bytes,
               (size_t)parts * sizeof(double));
    cudaStream_t s = sc::as_stream(stream);
    double *partial = static_cast<double *>(d_scratch);
    dD_partial_kernel<<<parts, kThreads, 0, s>>>(
        reinterpret_cast<const float4 *>(d_pos), reinterpret_cast<const float4 *>(d_emit), n, total,
        reinterpret_cast<const float4 *>(d_grad_pos), partial);
    finish_kernel<<<1, 32, 0, s>>>(partial, parts, d_D, d_dD);
    return sc::launch_status("sc_diffusion_dD");
}
