// Differentiable Born-Wolf expected image: forward and hand-written adjoint.
//
// The reference sums a 1-nm Born-Wolf grid over each pixel with bounds
// rounded up to the grid (overlay_signal_, src/scopyon/_epifm.py:224-282) and
// picks the grid of the 1-nm depth key below |depth| (:76-88), so its image
// is piecewise constant in x, y and z.  This model makes it continuous:
//   * along x and y each grid value fills one 1-nm cell, and a pixel takes
//     the exact integral of that piecewise-constant function over its
//     extent: the bilinear interpolation of the grid's 2-D prefix sum S at
//     the pixel's corners, alpha = (edge - x0) / res + 1 (x0 the position of
//     grid row 0, clamped to the grid);
//   * along z the two depth keys around |z - z_focal| / res are blended
//     linearly (the last key beyond the cutoff, as the reference's key -1);
//   * with the TIRF excitation A(z) = exp(-|z - z_focal| / d) (:1281-1289):
//   mu[f][i][j] = bg[f] + sum_e I_e A(z_e) cnorm B_e(i, j),
//   cnorm = psf_normalization * res^2 (photons of an in-focus emitter).
// The prefix sums come from the engine's quadrant tables (double-float
// entries, folded as fold.cuh does) and are evaluated in FP64, since a pixel
// is a difference of four large prefix values.  A warp takes one emitter:
// its lanes fill the corner values for both depth keys in shared memory
// (value and, for the adjoint, the two partial derivatives of the bilinear
// prefix), then sweep the footprint's pixels.  The forward adds FP64 atomics
// into a frame buffer; the adjoint reduces each emitter's gradient over its
// pixels in a fixed order (deterministic).
#include "sc_common.cuh"
#include "fold.cuh"

namespace {

constexpr int kBwWin = 16;      // corners per axis, at most (15 pixels)
constexpr int kBwFwdWarps = 4;  // warps per block, forward
constexpr int kBwBwdWarps = 2;  // warps per block, adjoint

struct BWConsts {
    int nw, nh, n_frames, n_emit, n_r, n_signal, pitch, key_hi;
    int64_t table_stride;
    double px, res, inv_pen, z_focal, cnorm, half_w, half_h, half_sig;
    const float2 *sat;
    const int32_t *key_slot;
};

// Full-grid 2-D prefix S(a, b) = sum_{p < a, q < b} P[p][q], a, b in
// [0, n_signal], from the quadrant table G (FP64 sum of the hi + lo terms).
__device__ __forceinline__ double prefix2(const float2 *__restrict__ G, const BWConsts &c, int a,
                                          int b) {
    if (a <= 0 || b <= 0) return 0.0;
    int uu[3], vv[3];
    float us[3], vs[3];
    const int nu = sc::fold(0, a, c.n_r, uu, us), nv = sc::fold(0, b, c.n_r, vv, vs);
    double s = 0.0;
    for (int iu = 0; iu < nu; ++iu) {
        const float2 *row = G + (int64_t)uu[iu] * c.pitch;
        for (int iv = 0; iv < nv; ++iv) {
            const float2 g = __ldg(row + vv[iv]);
            s += (double)(us[iu] * vs[iv]) * ((double)g.x + (double)g.y);
        }
    }
    return s;
}

// Corner coordinate in lattice units, clamped to [0, n_signal]: the lattice
// cell a and the fraction f; `free` is false where the clamp holds (no
// derivative).
__device__ __forceinline__ void corner(double alpha, int n_signal, int &a, double &f, bool &free) {
    free = alpha > 0.0 && alpha < (double)n_signal;
    const double al = fmin(fmax(alpha, 0.0), (double)n_signal);
    a = min((int)floor(al), n_signal - 1);
    f = al - (double)a;
}

struct Emitter {
    int i_lo, j_lo, nx, ny;    // first pixel and pixel counts of the footprint
    double x0, y0;             // positions of grid row / column 0 on the pixel axes
    int slot0, slot1;          // tables of the two depth keys
    double t, dt;              // blend weight of key 1, dt / d|z - z_focal|
    double A, dA, sgn;         // excitation, dA / d|z - z_focal|, sign(z - z_focal)
    float I;
    bool ok;
};

__device__ __forceinline__ Emitter emitter_geometry(const BWConsts &c, float4 e, int32_t *status,
                                                    int f, int n) {
    Emitter m;
    const double x = (double)e.x, y = (double)e.y, dz = (double)e.z - c.z_focal;
    m.I = e.w;
    m.sgn = (dz > 0.0) - (dz < 0.0);
    const double zr = fabs(dz);
    m.A = c.inv_pen > 0.0 ? exp(-zr * c.inv_pen) : 1.0;
    m.dA = -c.inv_pen * m.A;
    const double zq = zr / c.res;
    int k;
    if (zq >= (double)c.key_hi) {
        k = c.key_hi - 1;
        m.t = 1.0;
        m.dt = 0.0;
    } else {
        k = (int)floor(zq);
        m.t = zq - (double)k;
        m.dt = 1.0 / c.res;
    }
    m.slot0 = c.key_slot[k];
    m.slot1 = c.key_slot[k + 1];
    m.ok = m.slot0 >= 0 && m.slot1 >= 0 && isfinite(x) && isfinite(y) && isfinite(dz);
    if (!m.ok) {
        if ((threadIdx.x & 31) == 0) sc::flag_status(status, 1, f, n, k);
        return m;
    }
    m.x0 = (c.half_w + x) - c.half_sig;
    m.y0 = (c.half_h + y) - c.half_sig;
    // the grid covers [x0 - res, x0 - res + n_signal res) on the pixel axis
    const double span = c.res * (double)c.n_signal;
    const int i_lo = max(0, (int)floor((m.x0 - c.res) / c.px));
    const int i_hi = min(c.nw - 1, (int)floor((m.x0 - c.res + span) / c.px));
    const int j_lo = max(0, (int)floor((m.y0 - c.res) / c.px));
    const int j_hi = min(c.nh - 1, (int)floor((m.y0 - c.res + span) / c.px));
    m.i_lo = i_lo;
    m.j_lo = j_lo;
    m.nx = min(max(i_hi - i_lo + 1, 0), kBwWin - 1);
    m.ny = min(max(j_hi - j_lo + 1, 0), kBwWin - 1);
    if (i_hi - i_lo + 1 > kBwWin - 1 || j_hi - j_lo + 1 > kBwWin - 1) {
        if ((threadIdx.x & 31) == 0) sc::flag_status(status, 2, f, n, i_hi - i_lo + 1);
        m.ok = false;
    }
    return m;
}

// Corner values of one depth key's table for the emitter's footprint: F (the
// bilinear prefix) and, with derivatives, Fa = dF/dalpha and Fb = dF/dbeta,
// at the (nx + 1) x (ny + 1) pixel corners, into shared memory.
template <bool DERIV>
__device__ __forceinline__ void fill_corners(const BWConsts &c, const Emitter &m, int slot,
                                             double *F, double *Fa, double *Fb, int lane) {
    const float2 *G = c.sat + (int64_t)slot * c.table_stride;
    const int ncx = m.nx + 1, ncy = m.ny + 1;
    for (int q = lane; q < ncx * ncy; q += 32) {
        const int ci = q / ncy, cj = q - (q / ncy) * ncy;
        const double alpha = ((double)(m.i_lo + ci) * c.px - m.x0) / c.res + 1.0;
        const double beta = ((double)(m.j_lo + cj) * c.px - m.y0) / c.res + 1.0;
        int a, b;
        double fa, fb;
        bool free_a, free_b;
        corner(alpha, c.n_signal, a, fa, free_a);
        corner(beta, c.n_signal, b, fb, free_b);
        const double s00 = prefix2(G, c, a, b), s10 = prefix2(G, c, a + 1, b);
        const double s01 = prefix2(G, c, a, b + 1), s11 = prefix2(G, c, a + 1, b + 1);
        F[q] = (1.0 - fa) * ((1.0 - fb) * s00 + fb * s01) + fa * ((1.0 - fb) * s10 + fb * s11);
        if (DERIV) {
            Fa[q] = free_a ? (1.0 - fb) * (s10 - s00) + fb * (s11 - s01) : 0.0;
            Fb[q] = free_b ? (1.0 - fa) * (s01 - s00) + fa * (s11 - s10) : 0.0;
        }
    }
}

// d[q] difference of a pixel's four corners: (i+1, j+1) - (i, j+1) - (i+1, j) + (i, j).
__device__ __forceinline__ double box(const double *F, int pi, int pj, int ncy) {
    const int q = pi * ncy + pj;
    return F[q + ncy + 1] - F[q + 1] - F[q + ncy] + F[q];
}

__global__ void __launch_bounds__(kBwFwdWarps * 32)
bw_forward_kernel(BWConsts c, const float4 *__restrict__ emit, double *__restrict__ acc,
                  int32_t *status) {
    __shared__ double sF[kBwFwdWarps][2][kBwWin * kBwWin];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t total = (int64_t)c.n_frames * c.n_emit;
    for (int64_t g = (int64_t)blockIdx.x * kBwFwdWarps + warp; g < total;
         g += (int64_t)gridDim.x * kBwFwdWarps) {
        const int f = (int)(g / c.n_emit), n = (int)(g - (int64_t)f * c.n_emit);
        const float4 e = emit[g];
        if (!(e.w != 0.f)) continue;
        const Emitter m = emitter_geometry(c, e, status, f, n);
        if (!m.ok || m.nx <= 0 || m.ny <= 0) continue;
        fill_corners<false>(c, m, m.slot0, sF[warp][0], nullptr, nullptr, lane);
        fill_corners<false>(c, m, m.slot1, sF[warp][1], nullptr, nullptr, lane);
        __syncwarp();
        const double w = (double)m.I * m.A * c.cnorm;
        const int ncy = m.ny + 1;
        double *out = acc + (int64_t)f * c.nw * c.nh;
        for (int q = lane; q < m.nx * m.ny; q += 32) {
            const int pi = q / m.ny, pj = q - (q / m.ny) * m.ny;
            const double B = (1.0 - m.t) * box(sF[warp][0], pi, pj, ncy) +
                             m.t * box(sF[warp][1], pi, pj, ncy);
            if (B != 0.0)
                atomicAdd(out + (int64_t)(m.i_lo + pi) * c.nh + (m.j_lo + pj), w * B);
        }
        __syncwarp();
    }
}

__global__ void bw_finish_kernel(const double *__restrict__ acc, const float *__restrict__ bg,
                                 int64_t per_frame, int n_frames, float *__restrict__ mu) {
    const int64_t total = per_frame * n_frames;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total;
         g += (int64_t)gridDim.x * blockDim.x)
        mu[g] = (float)(acc[g] + (double)bg[g / per_frame]);
}

__global__ void __launch_bounds__(kBwBwdWarps * 32)
bw_backward_kernel(BWConsts c, const float4 *__restrict__ emit, const float *__restrict__ gmu,
                   float4 *__restrict__ gemit, int32_t *status) {
    __shared__ double sF[kBwBwdWarps][2][3][kBwWin * kBwWin];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t total = (int64_t)c.n_frames * c.n_emit;
    for (int64_t g = (int64_t)blockIdx.x * kBwBwdWarps + warp; g < total;
         g += (int64_t)gridDim.x * kBwBwdWarps) {
        const int f = (int)(g / c.n_emit), n = (int)(g - (int64_t)f * c.n_emit);
        const float4 e = emit[g];
        const Emitter m = emitter_geometry(c, e, status, f, n);
        double gx = 0.0, gy = 0.0, gz = 0.0, gI = 0.0;
        if (m.ok && m.nx > 0 && m.ny > 0) {
            double(*S)[3][kBwWin * kBwWin] = sF[warp];
            fill_corners<true>(c, m, m.slot0, S[0][0], S[0][1], S[0][2], lane);
            fill_corners<true>(c, m, m.slot1, S[1][0], S[1][1], S[1][2], lane);
            __syncwarp();
            const int ncy = m.ny + 1;
            const double inv_res = 1.0 / c.res;
            const float *gm = gmu + (int64_t)f * c.nw * c.nh;
            for (int q = lane; q < m.nx * m.ny; q += 32) {
                const int pi = q / m.ny, pj = q - (q / m.ny) * m.ny;
                const double gp = (double)gm[(int64_t)(m.i_lo + pi) * c.nh + (m.j_lo + pj)];
                const double B0 = box(S[0][0], pi, pj, ncy), B1 = box(S[1][0], pi, pj, ncy);
                const double B = (1.0 - m.t) * B0 + m.t * B1;
                // dalpha / dx = -1 / res at every corner (x0 moves with x)
                const double Bx = -inv_res * ((1.0 - m.t) * box(S[0][1], pi, pj, ncy) +
                                              m.t * box(S[1][1], pi, pj, ncy));
                const double By = -inv_res * ((1.0 - m.t) * box(S[0][2], pi, pj, ncy) +
                                              m.t * box(S[1][2], pi, pj, ncy));
                const double Bz = (B1 - B0) * m.dt;
                gI += gp * m.A * c.cnorm * B;
                gx += gp * (double)m.I * m.A * c.cnorm * Bx;
                gy += gp * (double)m.I * m.A * c.cnorm * By;
                gz += gp * (double)m.I * c.cnorm * (m.dA * B + m.A * Bz);
            }
            __syncwarp();
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            gx += __shfl_xor_sync(0xffffffffu, gx, o);
            gy += __shfl_xor_sync(0xffffffffu, gy, o);
            gz += __shfl_xor_sync(0xffffffffu, gz, o);
            gI += __shfl_xor_sync(0xffffffffu, gI, o);
        }
        if (lane == 0)
            gemit[g] = make_float4((float)gx, (float)gy, (float)(gz * m.sgn), (float)gI);
    }
}

int bw_consts(const ScBWParams *p, const float *d_sat, BWConsts &c) {
    SC_REQUIRE(p != nullptr, "born-wolf image: params are NULL");
    SC_REQUIRE(p->nw > 0 && p->nh > 0 && p->n_frames > 0 && p->n_emit >= 0,
               "born-wolf image: %d x %d, %d frames, %d emitters", p->nw, p->nh, p->n_frames,
               p->n_emit);
    SC_REQUIRE(p->n_r >= 2 && p->sat_pitch >= p->n_r + 1 && p->key_hi >= 1,
               "born-wolf image: n_r=%d pitch=%d key_hi=%d", p->n_r, p->sat_pitch, p->key_hi);
    SC_REQUIRE(p->px > 0 && p->res > 0 && p->cnorm > 0, "born-wolf image: px, res, cnorm > 0");
    SC_REQUIRE(d_sat && p->d_key_slot, "born-wolf image: NULL tables or key slots");
    c.nw = p->nw;
    c.nh = p->nh;
    c.n_frames = p->n_frames;
    c.n_emit = p->n_emit;
    c.n_r = p->n_r;
    c.n_signal = 2 * p->n_r - 1;
    c.pitch = p->sat_pitch;
    c.key_hi = p->key_hi;
    c.table_stride = (int64_t)(p->n_r + 1) * p->sat_pitch;
    c.px = p->px;
    c.res = p->res;
    c.inv_pen = p->inv_pen;
    c.z_focal = p->z_focal;
    c.cnorm = p->cnorm;
    c.half_w = (double)p->nw * p->px * 0.5;
    c.half_h = (double)p->nh * p->px * 0.5;
    c.half_sig = p->res * (double)(c.n_signal - 1) * 0.5;
    SC_REQUIRE(ceil(p->res * c.n_signal / p->px) + 1 <= kBwWin - 1,
               "born-wolf image: pixels of %g m are too small for the %d-pixel footprint window",
               p->px, kBwWin - 1);
    c.sat = reinterpret_cast<const float2 *>(d_sat);
    c.key_slot = p->d_key_slot;
    return SC_OK;
}

int grid_of(int64_t items, int per_block) {
    int64_t g = (items + per_block - 1) / per_block;
    return (int)(g < 152 * 16 ? (g > 0 ? g : 1) : 152 * 16);
}

}  // namespace

extern "C" size_t sc_bw_work_bytes(const ScBWParams *p) {
    if (!p || p->nw <= 0 || p->nh <= 0 || p->n_frames <= 0) return 0;
    return sizeof(double) * (size_t)p->nw * p->nh * p->n_frames;
}

extern "C" int sc_bw_forward(const ScBWParams *p, const float *d_emit, const float *d_bg,
                             const float *d_sat, void *d_work, size_t work_bytes, float *d_mu,
                             int32_t *d_status, void *stream) {
    BWConsts c;
    int rc = bw_consts(p, d_sat, c);
    if (rc) return rc;
    SC_REQUIRE(d_bg && d_mu && (d_emit || p->n_emit == 0), "sc_bw_forward: NULL pointer");
    SC_REQUIRE_CAP(d_work && work_bytes >= sc_bw_work_bytes(p), "sc_bw_forward: work %zu < %zu",
                   work_bytes, sc_bw_work_bytes(p));
    cudaStream_t st = sc::as_stream(stream);
    double *acc = static_cast<double *>(d_work);
    rc = sc::cuda_status(cudaMemsetAsync(acc, 0, sc_bw_work_bytes(p), st), "sc_bw_forward");
    if (rc) return rc;
    const int64_t items = (int64_t)p->n_frames * p->n_emit;
    if (items > 0)
        bw_forward_kernel<<<grid_of(items, kBwFwdWarps), kBwFwdWarps * 32, 0, st>>>(
            c, reinterpret_cast<const float4 *>(d_emit), acc, d_status);
    const int64_t per_frame = (int64_t)p->nw * p->nh;
    bw_finish_kernel<<<grid_of(per_frame * p->n_frames, 256), 256, 0, st>>>(
        acc, d_bg, per_frame, p->n_frames, d_mu);
    return sc::launch_status("sc_bw_forward");
}

extern "C" int sc_bw_backward(const ScBWParams *p, const float *d_emit, const float *d_sat,
                              const float *d_grad_mu, float *d_grad_emit, int32_t *d_status,
                              void *stream) {
    BWConsts c;
    int rc = bw_consts(p, d_sat, c);
    if (rc) return rc;
    const int64_t items = (int64_t)p->n_frames * p->n_emit;
    if (items == 0) return SC_OK;
    SC_REQUIRE(d_emit && d_grad_mu && d_grad_emit, "sc_bw_backward: NULL pointer");
    bw_backward_kernel<<<grid_of(items, kBwBwdWarps), kBwBwdWarps * 32, 0,
                         sc::as_stream(stream)>>>(c, reinterpret_cast<const float4 *>(d_emit),
                                                  d_grad_mu,
                                                  reinterpret_cast<float4 *>(d_grad_emit),
                                                  d_status);
    return sc::launch_status("sc_bw_backward");
}
