// Differentiable expected image with the Gaussian PSF, and its adjoint.
//
// Model (the reference's Gaussian PSF path, _epifm.py:133-134 and :224-282,
// with the TIRF excitation of _epifm.py:1281-1289 as the depth dependence):
//   mu[f, i, j] = bg[f] + sum_e I_e A(z_e) Gx_e(i) Gy_e(j)
//   Gx_e(i) = Phi((u_i + px - x_e) / sigma) - Phi((u_i - x_e) / sigma),
//   u_i = i px - W px / 2 (pixel i's low edge), Phi the normal CDF,
//   A(z) = exp(-|z - z_focal| / d) (1 under EPI, d = inf).
// The reference samples the same Gaussian on a 1-nm grid and sums the
// samples over each pixel; here the pixel integral is analytic, so that it
// can be differentiated.  Each emitter covers a (2R+1)^2 pixel window around
// its centre pixel (R = half_win, about 5.5 sigma: the truncated tails are
// below 1e-7 of the emitter's photons).
//
// Forward: one splat record per emitter, binned by tile (sc_bin_steps); the
// tile kernel adds its emitters' separable windows into a tile buffer in
// list order, and a merge pass sums the buffers covering each pixel in a
// fixed order: deterministic.  Adjoint: each binned record gathers dL/dmu
// over its window from a copy of the tile's area in shared memory: sum g Gx
// Gy, sum g dGx Gy, sum g Gx dGy and the sigma terms, in a fixed order.
// Windows of up to 15 pixels (R <= 7) take the tile kernels below (a warp per
// tile, registers for the buffer); wider ones the per-pixel kernels (a warp
// per record, one lane per window column).
#include <math.h>

#include "sc_common.cuh"
#include "bin.cuh"

namespace {

constexpr float kInvSqrt2 = 0.70710678118654752f;
constexpr float kInvSqrt2Pi = 0.39894228040143268f;

// Phi(b) - Phi(a) for a <= b, without cancellation in either tail.
__device__ __forceinline__ float cdf_diff(float a, float b) {
    if (a >= 0.f) return 0.5f * (erfcf(a * kInvSqrt2) - erfcf(b * kInvSqrt2));
    if (b <= 0.f) return 0.5f * (erfcf(-b * kInvSqrt2) - erfcf(-a * kInvSqrt2));
    return 1.f - 0.5f * (erfcf(b * kInvSqrt2) + erfcf(-a * kInvSqrt2));
}

__device__ __forceinline__ float pdf(float t) { return kInvSqrt2Pi * __expf(-0.5f * t * t); }

struct GaussConsts {
    int nw, nh, n_frames, n_emit, R;
    double px, inv_pen, z_focal;
    float inv_hi, inv_lo;  // 1 / px as a double-float
    float mid_w, mid_h;    // nw / 2 and nh / 2 (exact)
};

// Window of one emitter along one axis: centre pixel ic and the fraction fx
// of the way across it, x_rel = (x + n px / 2) / px = x / px + n / 2 = ic + fx.
// x / px is formed as a double-float (about 44 bits), so fx is the FP32
// rounding of the exact fraction except in rare double-rounding cases; no
// FP64 instruction is needed.
__device__ __forceinline__ void axis_centre(float x, float inv_hi, float inv_lo, float mid, int &ic,
                                            float &fx) {
    const float p = x * inv_hi;
    const float pe = fmaf(x, inv_lo, fmaf(x, inv_hi, -p));  // x inv - p, to FP32
    const float s = p + mid;                                 // two-sum of p and mid
    const float bb = s - p;
    const float se = ((p - (s - bb)) + (mid - bb)) + pe;
    const float hi = s + se, lo = se - (hi - s);
    float fl = floorf(hi);
    float fr = (hi - fl) + lo;  // hi - fl is exact
    if (fr < 0.f) {
        fl -= 1.f;
        fr += 1.f;
    } else if (fr >= 1.f) {
        fl += 1.f;
        fr -= 1.f;
    }
    ic = (int)fminf(fmaxf(fl, -1e9f), 1e9f);
    fx = fr;
}

__device__ __forceinline__ float amplitude(const GaussConsts &c, float z) {
    return c.inv_pen > 0.0 ? __expf(-fabsf(z - (float)c.z_focal) * (float)c.inv_pen) : 1.f;
}

// One splat record per emitter (binned by the tile of its first pixel):
// i_start, n_i (bounds = pixels + 1), ax_hi = fx, ax_lo = i_start - ic, and
// the same along y; w = I A(z).  Emitters whose window misses the image get
// slot -1.  Each record is counted into its bin as it is written (count,
// rec_bin, rec_rank: the binning workspace's counts, bins and ranks).  The
// FP64 origin (x0, y0) of the footprint path is not written: nothing on this
// path reads it.
__global__ void gauss_records_kernel(GaussConsts c, const float4 *emit, ScStepRec *recs,
                                     sc::TileGeom g, int32_t *count, int32_t *rec_bin,
                                     int32_t *rec_rank) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= c.n_frames * c.n_emit) return;
    const float4 e = emit[r];
    ScStepRec rec;
    rec.box_off = 0;
    rec.x0 = rec.y0 = 0.0;
    rec.box = 1;
    rec.box_local = 0;
    rec.slot = -1;
    rec.i_start = rec.j_start = 0;
    rec.n_i = rec.n_j = 0;
    rec.ax_hi = rec.ax_lo = rec.ay_hi = rec.ay_lo = 0.f;
    rec.w = e.w * amplitude(c, e.z);
    int icx, icy;
    float fx, fy;
    axis_centre(e.x, c.inv_hi, c.inv_lo, c.mid_w, icx, fx);
    axis_centre(e.y, c.inv_hi, c.inv_lo, c.mid_h, icy, fy);
    const int i0 = max(icx - c.R, 0), i1 = min(icx + c.R, c.nw - 1);
    const int j0 = max(icy - c.R, 0), j1 = min(icy + c.R, c.nh - 1);
    if (i1 >= i0 && j1 >= j0 && isfinite(fx) && isfinite(fy)) {
        rec.slot = 0;
        rec.i_start = (int16_t)i0;
        rec.n_i = (int16_t)(i1 - i0 + 2);
        rec.j_start = (int16_t)j0;
        rec.n_j = (int16_t)(j1 - j0 + 2);
        rec.ax_hi = fx;
        rec.ax_lo = (float)(i0 - icx);
        rec.ay_hi = fy;
        rec.ay_lo = (float)(j0 - icy);
    }
    int4 *dst = reinterpret_cast<int4 *>(recs + r);
    const int4 *src = reinterpret_cast<const int4 *>(&rec);
    dst[0] = src[0];
    dst[1] = src[1];
    dst[3] = src[3];
    sc::bin_record(g, rec, r, count, rec_bin, rec_rank);
}

// Pixel integral of the unit Gaussian over pixel offset d (from the centre
// pixel) for an emitter at fraction f of its centre pixel; s = px / sigma.
__device__ __forceinline__ float gauss_pixel(int d, float f, float s) {
    return cdf_diff(((float)d - f) * s, ((float)d + 1.f - f) * s);
}

// Tile splat: warp m mod NW takes the m-th record of the tile's list.
template <int NW>
__global__ void __launch_bounds__(NW * 32)
gauss_splat_kernel(const ScStepRec *__restrict__ recs, const int32_t *__restrict__ tile_start,
                   const int32_t *__restrict__ items, sc::TileGeom g, const float *sigma_p,
                   double px, float *__restrict__ ws) {
    extern __shared__ float sm[];
    const int E = g.edge, EE = E * E;
    const int BS = (EE + 31) & ~31;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tile = blockIdx.x;
    const int t = tile % g.tiles_per_image;
    const int x0 = (t / g.tiles_y) * g.tile, y0 = (t % g.tiles_y) * g.tile;
    for (int i = threadIdx.x; i < NW * BS; i += blockDim.x) sm[i] = 0.f;
    __syncthreads();
    float *buf = sm + warp * BS;
    const float s = (float)(px / (double)*sigma_p);
    const int it0 = tile_start[tile], it1 = tile_start[tile + 1];
    for (int m = it0 + warp; m < it1; m += NW) {
        const ScStepRec &rec = recs[__ldg(items + m)];
        const int ni = rec.n_i - 1, nj = rec.n_j - 1;
        const int ox = rec.i_start - x0, oy = rec.j_start - y0;
        const float gx = lane < ni ? gauss_pixel((int)rec.ax_lo + lane, rec.ax_hi, s) : 0.f;
        const float gy = lane < nj ? rec.w * gauss_pixel((int)rec.ay_lo + lane, rec.ay_hi, s) : 0.f;
        if (ox < 0 || oy < 0 || ox + ni > E || oy + nj > E) continue;  // not produced by records
        for (int a = 0; a < ni; ++a) {
            const float gxa = __shfl_sync(0xffffffffu, gx, a);
            if (lane < nj) {
                float *d = buf + (ox + a) * E + oy + lane;
                *d = fmaf(gxa, gy, *d);
            }
        }
        __syncwarp();
    }
    __syncthreads();
    float *out = ws + (size_t)tile * EE;
    for (int p = threadIdx.x; p < EE; p += blockDim.x) {
        float sum = 0.f;
#pragma unroll
        for (int w = 0; w < NW; ++w) sum += sm[w * BS + p];
        out[p] = sum;
    }
}

// Per pixel: background plus the tile buffers that cover it, in a fixed order.
__global__ void gauss_merge_kernel(const float *__restrict__ ws, sc::TileGeom g,
                                   const float *__restrict__ bg, float *__restrict__ mu) {
    const int n = g.nw * g.nh, E = g.edge, EE = E * E;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < (int64_t)n * g.n_images;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int img = (int)(q / n);
        const int p = (int)(q - (int64_t)img * n);
        const int i = p / g.nh, j = p - (p / g.nh) * g.nh;
        const int tx = i / g.tile, ty = j / g.tile;
        const float *tiles = ws + (size_t)img * g.tiles_per_image * EE;
        float sum = 0.f;
        for (int a = 0; a <= tx; ++a) {
            const int li = i - (tx - a) * g.tile;
            if (li >= E) break;
            for (int b = 0; b <= ty; ++b) {
                const int lj = j - (ty - b) * g.tile;
                if (lj >= E) break;
                sum += tiles[(size_t)((tx - a) * g.tiles_y + (ty - b)) * EE + li * E + lj];
            }
        }
        mu[q] = (bg ? bg[img] : 0.f) + sum;
    }
}

// Pixel value, x derivative (per pixel offset, times -1/sigma later) and
// sigma derivative factors of one window pixel.
struct PixTerms {
    float g, dg, sg;  // G, (phi(b) - phi(a)), (b phi(b) - a phi(a))
};

__device__ __forceinline__ PixTerms pix_terms(int d, float f, float s) {
    const float a = ((float)d - f) * s, b = ((float)d + 1.f - f) * s;
    const float pa = pdf(a), pb = pdf(b);
    return PixTerms{cdf_diff(a, b), pb - pa, b * pb - a * pa};
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Adjoint: one warp per emitter.  With g = dL/dmu over the window,
//   S1 = sum g Gx Gy,  Sx = sum g (dGx/dx) Gy,  Sy = sum g Gx (dGy/dy),
//   Ss = sum g (dGx/dsigma Gy + Gx dGy/dsigma),
// dL/dx = c Sx, dL/dy = c Sy, dL/dI = A S1, dL/dz = I A'(z) S1 and the
// emitter's share of dL/dsigma is c Ss (c = I A(z)).
__global__ void gauss_backward_kernel(GaussConsts c, const float4 *__restrict__ emit,
                                      const float *sigma_p, const float *__restrict__ grad_mu,
                                      float4 *__restrict__ grad_emit, float *grad_sigma_e) {
    const int warps = blockDim.x >> 5;
    const int r = blockIdx.x * warps + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (r >= c.n_frames * c.n_emit) return;
    const int f = r / c.n_emit;
    const float4 e = emit[r];
    const float sigma = *sigma_p;
    const float s = (float)(c.px / (double)sigma);
    int icx, icy;
    float fx, fy;
    axis_centre(e.x, c.inv_hi, c.inv_lo, c.mid_w, icx, fx);
    axis_centre(e.y, c.inv_hi, c.inv_lo, c.mid_h, icy, fy);
    const int K = 2 * c.R + 1;
    const int i0 = icx - c.R, j0 = icy - c.R;
    // lane b: column j0 + b (window column terms); row terms go by shuffle
    const bool col_ok = lane < K && j0 + lane >= 0 && j0 + lane < c.nh && isfinite(fy);
    const PixTerms ty = lane < K ? pix_terms(lane - c.R, fy, s) : PixTerms{0.f, 0.f, 0.f};
    const PixTerms tx = lane < K ? pix_terms(lane - c.R, fx, s) : PixTerms{0.f, 0.f, 0.f};
    float acc_g = 0.f, acc_d = 0.f, acc_s = 0.f;
    const float *G = grad_mu + (size_t)f * c.nw * c.nh;
    for (int a = 0; a < K; ++a) {
        const float gx = __shfl_sync(0xffffffffu, tx.g, a);
        const float dgx = __shfl_sync(0xffffffffu, tx.dg, a);
        const float sgx = __shfl_sync(0xffffffffu, tx.sg, a);
        const int i = i0 + a;
        if (i < 0 || i >= c.nw || !col_ok) continue;
        const float gv = __ldg(G + (size_t)i * c.nh + j0 + lane);
        acc_g = fmaf(gv, gx, acc_g);
        acc_d = fmaf(gv, dgx, acc_d);
        acc_s = fmaf(gv, sgx, acc_s);
    }
    // fold the column terms
    const float S1 = warp_sum(acc_g * ty.g);
    const float Sdx = warp_sum(acc_d * ty.g);
    const float Sdy = warp_sum(acc_g * ty.dg);
    const float Ss = warp_sum(acc_s * ty.g + acc_g * ty.sg);
    if (lane == 0) {
        const float A = amplitude(c, e.z);
        const float cc = e.w * A;
        const float inv_sigma = 1.f / sigma;
        // d/dx Phi((u - x) / sigma) = -phi / sigma; d/dsigma = -t phi / sigma
        float4 gr;
        gr.x = -cc * inv_sigma * Sdx;
        gr.y = -cc * inv_sigma * Sdy;
        const float dz = e.z - (float)c.z_focal;
        gr.z = c.inv_pen > 0.0 ? -e.w * A * (float)c.inv_pen * (dz > 0.f ? 1.f : (dz < 0.f ? -1.f : 0.f)) * S1
                               : 0.f;
        gr.w = A * S1;
        grad_emit[r] = gr;
        if (grad_sigma_e) grad_sigma_e[r] = -cc * inv_sigma * Ss;
    }
}

// ---------------------------------------------------------------------------
// Tile kernels for windows of up to 15 pixels (R <= 7), one warp per tile.
//
// A window along one axis has K + 1 edges t_k = ((float)(lo + k) - f) s
// (lo: its first pixel's offset from the centre pixel); pixel k integrates
// to Phi(t_{k+1}) - Phi(t_k).  Each edge's erfc is evaluated once and shared
// by the two pixels on either side, and the difference is formed exactly as
// cdf_diff forms it, so pixel values equal the per-pixel kernels' bit for bit.

constexpr int kTileWarps = 4;

__device__ __forceinline__ float edge_t(int lo, int k, float f, float s) {
    return ((float)(lo + k) - f) * s;
}

__device__ __forceinline__ float edge_erfc(float t) { return erfcf(fabsf(t) * kInvSqrt2); }

__device__ __forceinline__ float pixel_from_edges(float ta, float tb, float va, float vb) {
    if (ta >= 0.f) return 0.5f * (va - vb);
    if (tb <= 0.f) return 0.5f * (vb - va);
    return 1.f - 0.5f * (vb + va);
}

// A record's x integrals into row[0 .. P) and its w * y integrals into
// row[P .. 2P): window pixel k at position o + k (the first n of the window;
// the rest of the window and everything outside it are 0).  The two axes
// run in one loop, two independent chains per step.
template <int K, int P>
__device__ __forceinline__ void stage_record(const ScStepRec &rec, int ox, int oy, int ni, int nj,
                                             float s, float *row) {
#pragma unroll
    for (int z = 0; z < P - K; ++z) {
        row[z < ox ? z : z + K] = 0.f;
        row[P + (z < oy ? z : z + K)] = 0.f;
    }
    const int lx = (int)rec.ax_lo, ly = (int)rec.ay_lo;
    const float fx = rec.ax_hi, fy = rec.ay_hi, w = rec.w;
    float tax = edge_t(lx, 0, fx, s), vax = edge_erfc(tax);
    float tay = edge_t(ly, 0, fy, s), vay = edge_erfc(tay);
    float *px_out = row + ox, *py_out = row + P + oy;
#pragma unroll 1
    for (int k = 0; k < K; ++k) {
        const float tbx = edge_t(lx, k + 1, fx, s), vbx = edge_erfc(tbx);
        const float tby = edge_t(ly, k + 1, fy, s), vby = edge_erfc(tby);
        px_out[k] = k < ni ? pixel_from_edges(tax, tbx, vax, vbx) : 0.f;
        py_out[k] = k < nj ? w * pixel_from_edges(tay, tby, vay, vby) : 0.f;
        tax = tbx;
        vax = vbx;
        tay = tby;
        vay = vby;
    }
}

// First pixel of a binned record relative to its tile, and its window sizes;
// a record that does not fit the tile buffer (not one the records kernel
// writes) contributes nothing.
template <int K>
__device__ __forceinline__ void tile_window(const ScStepRec &rec, int x0, int y0, int tile,
                                            int &ox, int &oy, int &ni, int &nj) {
    ox = rec.i_start - x0;
    oy = rec.j_start - y0;
    ni = rec.n_i - 1;
    nj = rec.n_j - 1;
    if (ox < 0 || oy < 0 || ox >= tile || oy >= tile || ni > K || nj > K) ox = oy = ni = nj = 0;
}

// Forward, output-stationary: the warp of a tile keeps the tile's (E x E,
// E <= P) buffer in registers, lane (lr, lc) owning rows lr*P/4 .. +P/4 and
// columns lc*P/8 .. +P/8.  Lanes stage 32 records at a time (lane l: record
// l's x integrals and w * y integrals, zero-padded to P), then every lane
// adds the records' outer products to its block in list order:
// deterministic, and one fused multiply-add per pixel per record.
template <int R, int P>
__global__ void __launch_bounds__(kTileWarps * 32)
gauss_tile_splat_kernel(const ScStepRec *__restrict__ recs, const int32_t *__restrict__ tile_start,
                        const int32_t *__restrict__ items, sc::TileGeom g, const float *sigma_p,
                        double px, float *__restrict__ ws) {
    constexpr int K = 2 * R + 1;
    constexpr int BR = P / 4, BC = P / 8;
    constexpr int STR = 2 * P + 2;  // staged record: x[P], w y[P]; 2-way store conflicts at most
    static_assert(BR % 2 == 0, "row blocks are read as float2");
    __shared__ __align__(16) float stage[kTileWarps][32 * STR];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tile = blockIdx.x * kTileWarps + warp;
    if (tile >= g.n_tiles) return;
    const int t = tile % g.tiles_per_image;
    const int x0 = (t / g.tiles_y) * g.tile, y0 = (t % g.tiles_y) * g.tile;
    const int E = g.edge;
    float *st = stage[warp];
    const float s = (float)(px / (double)*sigma_p);
    const int lr = lane >> 3, lc = lane & 7;
    float acc[BR][BC];
#pragma unroll
    for (int i = 0; i < BR; ++i)
#pragma unroll
        for (int j = 0; j < BC; ++j) acc[i][j] = 0.f;
    const int it0 = tile_start[tile], it1 = tile_start[tile + 1];
    for (int m0 = it0; m0 < it1; m0 += 32) {
        const int cnt = min(32, it1 - m0);
        if (lane < cnt) {
            const ScStepRec &rec = recs[__ldg(items + m0 + lane)];
            int ox, oy, ni, nj;
            tile_window<K>(rec, x0, y0, g.tile, ox, oy, ni, nj);
            stage_record<K, P>(rec, ox, oy, ni, nj, s, st + lane * STR);
        }
        __syncwarp();
        for (int r = 0; r < cnt; ++r) {
            const float *row = st + r * STR;
            float gx[BR], gy[BC];
#pragma unroll
            for (int i = 0; i < BR; i += 2) {
                const float2 v = *reinterpret_cast<const float2 *>(row + lr * BR + i);
                gx[i] = v.x;
                gx[i + 1] = v.y;
            }
#pragma unroll
            for (int j = 0; j < BC; ++j) gy[j] = row[P + lc * BC + j];
#pragma unroll
            for (int i = 0; i < BR; ++i)
#pragma unroll
                for (int j = 0; j < BC; ++j) acc[i][j] = fmaf(gx[i], gy[j], acc[i][j]);
        }
        __syncwarp();
    }
    float *out = ws + (size_t)tile * E * E;
#pragma unroll
    for (int i = 0; i < BR; ++i)
#pragma unroll
        for (int j = 0; j < BC; ++j) {
            const int pi = lr * BR + i, pj = lc * BC + j;
            if (pi < E && pj < E) out[pi * E + pj] = acc[i][j];
        }
}

// Adjoint, one thread per binned record: the warp of a tile copies dL/dmu
// over the tile's E x E buffer area into shared memory (0 outside the
// image), then each lane takes records l, l + 32, ... of the tile's list and
// forms, over its window,
//   h(a) = sum_b G[a][b] gy(b) (and with dgy, sgy),
//   S1 = sum_a gx(a) h(a), Sdx = sum_a dgx(a) h(a), Sdy = sum_a gx(a) hd(a),
//   Ss = sum_a sgx(a) h(a) + gx(a) hs(a),
// in a fixed order.  The y terms live in registers; the x terms are formed
// row by row from the running edge.
constexpr int kPatchStride = 40;  // 8 (mod 32): first pixels (ox, oy) spread over the banks
constexpr int kPatchRows = 16 + 2 * 7;

template <int R>
__global__ void __launch_bounds__(kTileWarps * 32)
gauss_tile_backward_kernel(GaussConsts c, const ScStepRec *__restrict__ recs,
                           const int32_t *__restrict__ tile_start,
                           const int32_t *__restrict__ items, sc::TileGeom g,
                           const float4 *__restrict__ emit, const float *sigma_p,
                           const float *__restrict__ grad_mu, float4 *__restrict__ grad_emit,
                           float *grad_sigma_e) {
    constexpr int K = 2 * R + 1;
    constexpr int S = kPatchStride;
    __shared__ float patch[kTileWarps][kPatchRows * S];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tile = blockIdx.x * kTileWarps + warp;
    if (tile >= g.n_tiles) return;
    const int img = tile / g.tiles_per_image;
    const int t = tile - img * g.tiles_per_image;
    const int x0 = (t / g.tiles_y) * g.tile, y0 = (t % g.tiles_y) * g.tile;
    const int E = g.edge;
    const int it0 = tile_start[tile], it1 = tile_start[tile + 1];
    if (it0 == it1) return;
    float *pt = patch[warp];
    const float *G = grad_mu + (size_t)img * c.nw * c.nh;
    const int j = y0 + lane;
    for (int a = 0; a < E; ++a) {
        const int i = x0 + a;
        if (lane < E) pt[a * S + lane] = (i < c.nw && j < c.nh) ? __ldg(G + (size_t)i * c.nh + j) : 0.f;
    }
    __syncwarp();
    const float sigma = *sigma_p;
    const float s = (float)(c.px / (double)sigma);
    for (int m = it0 + lane; m < it1; m += 32) {
        const int r = __ldg(items + m);
        const ScStepRec &rec = recs[r];
        int ox, oy, ni, nj;
        tile_window<K>(rec, x0, y0, g.tile, ox, oy, ni, nj);
        float gy[K], dgy[K], sgy[K];
        {
            const int lo = (int)rec.ay_lo;
            const float f = rec.ay_hi;
            float ta = edge_t(lo, 0, f, s), va = edge_erfc(ta), pa = pdf(ta);
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const float tb = edge_t(lo, k + 1, f, s), vb = edge_erfc(tb), pb = pdf(tb);
                const bool ok = k < nj;
                gy[k] = ok ? pixel_from_edges(ta, tb, va, vb) : 0.f;
                dgy[k] = ok ? pb - pa : 0.f;
                sgy[k] = ok ? tb * pb - ta * pa : 0.f;
                ta = tb;
                va = vb;
                pa = pb;
            }
        }
        float S1 = 0.f, Sdx = 0.f, Sdy = 0.f, Ss = 0.f;
        {
            const int lo = (int)rec.ax_lo;
            const float f = rec.ax_hi;
            const float *p0 = pt + ox * S + oy;
            float ta = edge_t(lo, 0, f, s), va = edge_erfc(ta), pa = pdf(ta);
#pragma unroll 1
            for (int a = 0; a < ni; ++a) {
                const float tb = edge_t(lo, a + 1, f, s), vb = edge_erfc(tb), pb = pdf(tb);
                const float gx = pixel_from_edges(ta, tb, va, vb);
                const float dgx = pb - pa, sgx = tb * pb - ta * pa;
                float hg = 0.f, hd = 0.f, hs = 0.f;
#pragma unroll
                for (int b = 0; b < K; ++b) {
                    const float gv = p0[a * S + b];
                    hg = fmaf(gv, gy[b], hg);
                    hd = fmaf(gv, dgy[b], hd);
                    hs = fmaf(gv, sgy[b], hs);
                }
                S1 = fmaf(gx, hg, S1);
                Sdx = fmaf(dgx, hg, Sdx);
                Sdy = fmaf(gx, hd, Sdy);
                Ss = fmaf(sgx, hg, fmaf(gx, hs, Ss));
                ta = tb;
                va = vb;
                pa = pb;
            }
        }
        const float4 e = emit[r];
        const float A = amplitude(c, e.z);
        const float cc = e.w * A;
        const float inv_sigma = 1.f / sigma;
        float4 gr;
        gr.x = -cc * inv_sigma * Sdx;
        gr.y = -cc * inv_sigma * Sdy;
        const float dz = e.z - (float)c.z_focal;
        gr.z = c.inv_pen > 0.0
                   ? -e.w * A * (float)c.inv_pen * (dz > 0.f ? 1.f : (dz < 0.f ? -1.f : 0.f)) * S1
                   : 0.f;
        gr.w = A * S1;
        grad_emit[r] = gr;
        if (grad_sigma_e) grad_sigma_e[r] = -cc * inv_sigma * Ss;
    }
}

template <int R>
void launch_tile_splat(int P, int grid, cudaStream_t st, const ScStepRec *recs,
                       const int32_t *tile_start, const int32_t *items, const sc::TileGeom &g,
                       const float *sigma, double px, float *ws) {
    if (P == 24)
        gauss_tile_splat_kernel<R, 24><<<grid, kTileWarps * 32, 0, st>>>(recs, tile_start, items,
                                                                         g, sigma, px, ws);
    else
        gauss_tile_splat_kernel<R, 32><<<grid, kTileWarps * 32, 0, st>>>(recs, tile_start, items,
                                                                         g, sigma, px, ws);
}

// Tile kernels take windows of R <= 7 on tiles of 8 or 16 pixels.
bool tile_path(const GaussConsts &c) { return c.R <= 7; }

constexpr int kSumThreads = 256;
constexpr int kSumChunk = 1024;    // values per CTA and pass
constexpr int kSumMaxParts = 1216; // CTAs per segment (8 on each of 152 SMs)

__device__ __forceinline__ double block_sum(double acc, double *part) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < kSumThreads / 32; ++w) t += part[w];
    return t;
}

// Part x of segment y: the chunks x, x + parts, ... of kSumChunk values,
// summed in FP64 in a fixed order into partial[y][x].
// With counts, the terms are the Poisson NLL mu - k log mu and grad gets
// 1 - k / mu.
__global__ void __launch_bounds__(kSumThreads)
partial_sum_kernel(const float *__restrict__ x, const float *__restrict__ counts, int64_t seg_len,
                   float *grad, double *partial) {
    __shared__ double part[kSumThreads / 32];
    const int parts = gridDim.x;
    const size_t base = (size_t)blockIdx.y * seg_len;
    double acc = 0.0;
    for (int64_t c0 = (int64_t)blockIdx.x * kSumChunk; c0 < seg_len; c0 += (int64_t)parts * kSumChunk) {
        const int64_t c1 = c0 + kSumChunk < seg_len ? c0 + kSumChunk : seg_len;
        for (int64_t q = c0 + threadIdx.x; q < c1; q += kSumThreads) {
            const float m = x[base + q];
            if (counts) {
                const float kk = counts[base + q];
                // logf is within an ulp; the FP64 accumulation is what a
                // sum over millions of pixels needs
                acc += sc::f2d_exact(m) - sc::f2d_exact(kk) * sc::f2d_exact(logf(m));
                if (grad) grad[base + q] = 1.f - kk / m;
            } else {
                acc += sc::f2d_exact(m);
            }
        }
    }
    const double t = block_sum(acc, part);
    if (threadIdx.x == 0) partial[(size_t)blockIdx.y * parts + blockIdx.x] = t;
}

// out[y] = sum of partial[y][0 .. parts), a warp per segment: lane l sums
// partials l, l + 32, ... in order, then a butterfly (the same bits on every
// lane and every run).
__global__ void finish_sum_kernel(const double *partial, int parts, int n_seg, double *out) {
    const int y = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (y >= n_seg) return;
    double t = 0.0;
    for (int k = lane; k < parts; k += 32) t += partial[(size_t)y * parts + k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) out[y] = t;
}

int sum_parts(int64_t seg_len) {
    int64_t parts = (seg_len + kSumChunk - 1) / kSumChunk;
    if (parts < 1) parts = 1;
    if (parts > kSumMaxParts) parts = kSumMaxParts;
    return (int)parts;
}

int launch_reduce(const float *x, const float *counts, int64_t seg_len, int n_seg, void *scratch,
                  size_t scratch_bytes, float *grad, double *out, cudaStream_t s) {
    SC_REQUIRE(seg_len >= 0 && n_seg >= 0, "negative size");
    if (n_seg == 0) return SC_OK;
    SC_REQUIRE(n_seg <= 65535, "n_seg=%d exceeds 65535", n_seg);
    SC_REQUIRE(out && (seg_len == 0 || x), "NULL pointer");
    const int parts = sum_parts(seg_len);
    SC_REQUIRE_CAP(scratch && scratch_bytes >= (size_t)parts * n_seg * sizeof(double),
               "reduction scratch %zu < %zu bytes", scratch_bytes,
               (size_t)parts * n_seg * sizeof(double));
    double *partial = static_cast<double *>(scratch);
    partial_sum_kernel<<<dim3((unsigned)parts, (unsigned)n_seg), kSumThreads, 0, s>>>(
        x, counts, seg_len, grad, partial);
    finish_sum_kernel<<<(n_seg + 3) / 4, 128, 0, s>>>(partial, parts, n_seg, out);
    return sc::launch_status("reduction");
}

int gauss_consts(const ScGaussParams *p, GaussConsts &c) {
    SC_REQUIRE(p != nullptr, "gauss params are NULL");
    SC_REQUIRE(p->nw > 0 && p->nh > 0 && p->nw < 32767 && p->nh < 32767, "image %dx%d", p->nw, p->nh);
    SC_REQUIRE(p->n_frames >= 1 && p->n_emit >= 0, "n_frames=%d n_emit=%d", p->n_frames, p->n_emit);
    SC_REQUIRE((int64_t)p->n_frames * p->n_emit < (1ll << 31), "too many emitters");
    SC_REQUIRE(p->half_win >= 1 && p->half_win <= 15, "half_win=%d must be in [1, 15]", p->half_win);
    SC_REQUIRE(p->tile == 8 || p->tile == 16, "tile=%d must be 8 or 16", p->tile);
    SC_REQUIRE(p->px > 0, "px must be positive");
    SC_REQUIRE(p->inv_pen >= 0, "inv_pen must be >= 0");
    c.nw = p->nw;
    c.nh = p->nh;
    c.n_frames = p->n_frames;
    c.n_emit = p->n_emit;
    c.R = p->half_win;
    c.px = p->px;
    const double inv = 1.0 / p->px;
    c.inv_hi = (float)inv;
    c.inv_lo = (float)(inv - (double)c.inv_hi);
    c.mid_w = 0.5f * (float)p->nw;
    c.mid_h = 0.5f * (float)p->nh;
    c.inv_pen = p->inv_pen;
    c.z_focal = p->z_focal;
    return SC_OK;
}

// Splat parameters of the forward: tiles of p->tile, halo 2R (a window spans
// 2R + 1 pixels from its first one), one image per frame.
ScSplatParams gauss_splat_params(const ScGaussParams *p) {
    ScSplatParams sp{};
    sp.nw = p->nw;
    sp.nh = p->nh;
    sp.tile = p->tile;
    sp.halo = 2 * p->half_win;
    sp.warps = 4;
    sp.tiles_x = (p->nw + p->tile - 1) / p->tile;
    sp.tiles_y = (p->nh + p->tile - 1) / p->tile;
    sp.n_images = p->n_frames;
    sp.rec_per_image = p->n_emit;
    return sp;
}

struct GaussWorkspace {
    ScStepRec *recs;
    int32_t *tile_start, *items;
    void *bin_ws;
    size_t bin_bytes;
    float *tiles;
    size_t total;
};

GaussWorkspace gauss_workspace(const ScGaussParams *p, void *base) {
    const ScSplatParams sp = gauss_splat_params(p);
    const int n_rec = p->n_frames * p->n_emit;
    const int n_tiles = sp.tiles_x * sp.tiles_y * sp.n_images;
    const int E = sp.tile + sp.halo;
    auto up = [](size_t v) { return (v + 255) & ~(size_t)255; };
    GaussWorkspace w{};
    char *b = static_cast<char *>(base);
    size_t off = 0;
    w.recs = reinterpret_cast<ScStepRec *>(b + off);
    off += up((size_t)(n_rec > 0 ? n_rec : 1) * sizeof(ScStepRec));
    w.tile_start = reinterpret_cast<int32_t *>(b + off);
    off += up((size_t)(2 * n_tiles + 1) * sizeof(int32_t));
    w.items = reinterpret_cast<int32_t *>(b + off);
    off += up((size_t)(n_rec > 0 ? n_rec : 1) * sizeof(int32_t));
    w.bin_ws = b + off;
    w.bin_bytes = sc_bin_workspace_bytes(n_rec > 0 ? n_rec : 1, n_tiles);
    off += up(w.bin_bytes);
    w.tiles = reinterpret_cast<float *>(b + off);
    off += up((size_t)n_tiles * E * E * sizeof(float));
    w.total = off;
    return w;
}

}  // namespace

extern "C" size_t sc_gauss_workspace_bytes(const ScGaussParams *p) {
    GaussConsts c;
    if (gauss_consts(p, c) != SC_OK) return 0;
    return gauss_workspace(p, nullptr).total;
}

extern "C" int sc_gauss_forward(const ScGaussParams *p, const float *d_emit, const float *d_sigma,
                                const float *d_bg, void *d_ws, size_t ws_bytes, float *d_mu,
                                int32_t *d_status, void *stream) {
    (void)d_status;  // no data check on this path writes a status word
    GaussConsts c;
    int rc = gauss_consts(p, c);
    if (rc) return rc;
    SC_REQUIRE(d_sigma && d_mu && d_ws, "sc_gauss_forward: NULL pointer");
    SC_REQUIRE(c.n_emit == 0 || d_emit, "sc_gauss_forward: emitters are NULL");
    const GaussWorkspace w = gauss_workspace(p, d_ws);
    SC_REQUIRE_CAP(ws_bytes >= w.total, "sc_gauss_forward: workspace %zu < %zu bytes", ws_bytes, w.total);
    cudaStream_t s = sc::as_stream(stream);
    const ScSplatParams sp = gauss_splat_params(p);
    sc::TileGeom g;
    rc = sc::tile_geom(&sp, g);
    if (rc) return rc;
    const int n_rec = c.n_frames * c.n_emit;
    if (n_rec > 0) {
        sc::BinLayout b;
        sc::bin_layout(g, n_rec, w.bin_ws, w.bin_bytes, b);
        rc = sc_bin_reset(&sp, w.bin_ws, w.bin_bytes, stream);
        if (rc) return rc;
        gauss_records_kernel<<<(n_rec + 255) / 256, 256, 0, s>>>(
            c, reinterpret_cast<const float4 *>(d_emit), w.recs, g, b.count, b.rec_bin,
            sc::rank_array(b));
        rc = sc_bin_finish(n_rec, &sp, w.bin_ws, w.bin_bytes, w.tile_start, w.items, stream);
        if (rc) return rc;
        if (tile_path(c)) {
            const int P = g.edge <= 24 ? 24 : 32;
            const int grid = (g.n_tiles + kTileWarps - 1) / kTileWarps;
            switch (c.R) {
#define SC_TILE_SPLAT(RR)                                                                   \
    case RR:                                                                                \
        launch_tile_splat<RR>(P, grid, s, w.recs, w.tile_start, w.items, g, d_sigma, c.px, \
                              w.tiles);                                                     \
        break;
                SC_TILE_SPLAT(1) SC_TILE_SPLAT(2) SC_TILE_SPLAT(3) SC_TILE_SPLAT(4)
                SC_TILE_SPLAT(5) SC_TILE_SPLAT(6) SC_TILE_SPLAT(7)
#undef SC_TILE_SPLAT
            }
        } else {
            const int E = g.edge, BS = (E * E + 31) & ~31;
            const size_t smem = (size_t)4 * BS * sizeof(float);
            SC_REQUIRE(smem <= 48 * 1024, "sc_gauss_forward: tile buffers need %zu bytes", smem);
            gauss_splat_kernel<4><<<g.n_tiles, 128, smem, s>>>(w.recs, w.tile_start, w.items, g,
                                                               d_sigma, c.px, w.tiles);
        }
    } else {
        rc = sc::cuda_status(
            cudaMemsetAsync(w.tiles, 0, (size_t)g.n_tiles * g.edge * g.edge * sizeof(float), s),
            "sc_gauss_forward");
        if (rc) return rc;
    }
    const int64_t n_px = (int64_t)c.nw * c.nh * c.n_frames;
    int grid = (int)((n_px + 255) / 256);
    if (grid > 152 * 16) grid = 152 * 16;
    gauss_merge_kernel<<<grid, 256, 0, s>>>(w.tiles, g, d_bg, d_mu);
    return sc::launch_status("sc_gauss_forward");
}

extern "C" int sc_gauss_backward(const ScGaussParams *p, const float *d_emit, const float *d_sigma,
                                 const void *d_ws, size_t ws_bytes, const float *d_grad_mu,
                                 float *d_grad_emit, float *d_grad_sigma_e, void *stream) {
    GaussConsts c;
    int rc = gauss_consts(p, c);
    if (rc) return rc;
    const int n_rec = c.n_frames * c.n_emit;
    if (n_rec == 0) return SC_OK;
    SC_REQUIRE(d_emit && d_sigma && d_grad_mu && d_grad_emit, "sc_gauss_backward: NULL pointer");
    cudaStream_t s = sc::as_stream(stream);
    if (!tile_path(c)) {
        gauss_backward_kernel<<<(n_rec + 7) / 8, 256, 0, s>>>(
            c, reinterpret_cast<const float4 *>(d_emit), d_sigma, d_grad_mu,
            reinterpret_cast<float4 *>(d_grad_emit), d_grad_sigma_e);
        return sc::launch_status("sc_gauss_backward");
    }
    // the records and bins sc_gauss_forward left in the workspace
    SC_REQUIRE(d_ws, "sc_gauss_backward: the forward's workspace is NULL");
    const GaussWorkspace w = gauss_workspace(p, const_cast<void *>(d_ws));
    SC_REQUIRE_CAP(ws_bytes >= w.total, "sc_gauss_backward: workspace %zu < %zu bytes", ws_bytes,
               w.total);
    const ScSplatParams sp = gauss_splat_params(p);
    sc::TileGeom g;
    rc = sc::tile_geom(&sp, g);
    if (rc) return rc;
    // records outside every tile (windows that miss the image) get zeros
    rc = sc::cuda_status(cudaMemsetAsync(d_grad_emit, 0, (size_t)n_rec * sizeof(float4), s),
                         "sc_gauss_backward");
    if (rc) return rc;
    if (d_grad_sigma_e) {
        rc = sc::cuda_status(cudaMemsetAsync(d_grad_sigma_e, 0, (size_t)n_rec * sizeof(float), s),
                             "sc_gauss_backward");
        if (rc) return rc;
    }
    const int grid = (g.n_tiles + kTileWarps - 1) / kTileWarps;
    const float4 *e4 = reinterpret_cast<const float4 *>(d_emit);
    float4 *g4 = reinterpret_cast<float4 *>(d_grad_emit);
    switch (c.R) {
#define SC_TILE_BWD(RR)                                                                        \
    case RR:                                                                                   \
        gauss_tile_backward_kernel<RR><<<grid, kTileWarps * 32, 0, s>>>(                       \
            c, w.recs, w.tile_start, w.items, g, e4, d_sigma, d_grad_mu, g4, d_grad_sigma_e); \
        break;
        SC_TILE_BWD(1) SC_TILE_BWD(2) SC_TILE_BWD(3) SC_TILE_BWD(4)
        SC_TILE_BWD(5) SC_TILE_BWD(6) SC_TILE_BWD(7)
#undef SC_TILE_BWD
    }
    return sc::launch_status("sc_gauss_backward");
}

extern "C" size_t sc_reduce_scratch_bytes(int64_t seg_len, int n_seg) {
    if (seg_len < 0 || n_seg <= 0) return 0;
    return (size_t)sum_parts(seg_len) * n_seg * sizeof(double);
}

extern "C" int sc_segment_sum(const float *d_x, int64_t seg_len, int n_seg, void *d_scratch,
                              size_t scratch_bytes, double *d_out, void *stream) {
    return launch_reduce(d_x, nullptr, seg_len, n_seg, d_scratch, scratch_bytes, nullptr, d_out,
                         sc::as_stream(stream));
}

extern "C" int sc_poisson_nll(const float *d_mu, const float *d_counts, int64_t seg_len, int n_seg,
                              void *d_scratch, size_t scratch_bytes, double *d_loss,
                              float *d_grad_mu, void *stream) {
    SC_REQUIRE(n_seg == 0 || d_counts, "sc_poisson_nll: counts are NULL");
    return launch_reduce(d_mu, d_counts, seg_len, n_seg, d_scratch, scratch_bytes, d_grad_mu,
                         d_loss, sc::as_stream(stream));
}
