// Per-record emitter physics shared by the trajectory-driven and the
// on-device-diffusion step kernels.
#pragma once

#include "sc_common.cuh"

namespace sc {

struct StepConsts {
    double px, res, depth_cutoff;
    double focal[3];
    int nw, nh, n_signal, n_sub, n_particles, max_key;
    double amplitude0, penetration, x_sec, qy, beer, norm_coeff;
    int bleaching, with_optinfo, box_p, box_nq;
    double half_w, half_h, half_sig, inv_res;
    float inv_px_f, inv_res_f;
    // double-float copies for the footprint arithmetic
    df half_w_df, half_h_df, half_sig_df, nhalf_sig_df, inv_px_df, px_df, inv_res_df;
    float cut_f;      // fl32(depth_cutoff + res)
    int focal_zero;   // focal point at the origin: depths and offsets need no subtraction
    int row_layout;   // sc_emitter_steps input rows (ScStepParams.row_layout)
};

int step_consts(const ScStepParams *p, StepConsts &c);

// n_emit = QY * (amplitude * x_sec * dt) * (1 - 10^-A)   (_epifm.py:1344-1360).
// Products that feed an addition use __dmul_rn throughout these kernels: a
// contracted fma would skip the product's rounding, which the reference (numpy,
// one rounded operation at a time) performs, and flip threshold decisions.
__device__ __forceinline__ double emit_photons(const StepConsts &c, double amplitude, double dt) {
    const double n_abs = __dmul_rn(__dmul_rn(amplitude, c.x_sec), dt);
    return __dmul_rn(__dmul_rn(c.qy, n_abs), c.beer);
}

// Footprint arithmetic.  The reference evaluates, in FP64,
//   origin = (half_len + coord) - half_sig,  top = (half_len + coord) + half_sig,
//   first pixel floor(origin / px), last ceil(top / px), bounds ceil((i px - origin) / res)
// (_epifm.py:233-258).  Here the same quantities are carried as double-floats
// (hi + lo, ~2^-46 relative, FP32 pipe; GB300 runs FP64 at ~1/64 of the FP32
// rate).  Every floor / ceil whose double-float argument lies within kDfMargin
// of an integer is re-evaluated with the reference's FP64 expression, so the
// pixel ranges, depth keys and box decisions are the reference's.
constexpr float kDfMargin = 1e-7f;  // absolute, on quotients below 2^22

// floor / ceil of a double-float with the exact fallback decided by the caller.
__device__ __forceinline__ bool df_floor(df q, int &v) {
    float r;
    const float d = df_round(q, r);
    v = (int)r - (d < 0.f ? 1 : 0);
    return fabsf(d) > kDfMargin;
}

__device__ __forceinline__ bool df_ceil(df q, int &v) {
    float r;
    const float d = df_round(q, r);
    v = (int)r + (d > 0.f ? 1 : 0);
    return fabsf(d) > kDfMargin;
}

// A coordinate as a double-float, an FP64 value and an FP32 value: exact
// conversions, on the FP64 pipe for an FP64 coordinate and with no FP64 work
// for an FP32 one (the native trajectories), so that a record built from an
// FP32 coordinate equals, bit for bit, the record built from its FP64 value.
__device__ __forceinline__ df df_of(double x) { return df_from(x); }
__device__ __forceinline__ df df_of(float x) { return df{x, 0.f}; }
__device__ __forceinline__ double as_d(double x) { return x; }
__device__ __forceinline__ double as_d(float x) { return f2d_exact(x); }
__device__ __forceinline__ float as_f(double x) { return __double2float_rn(x); }
__device__ __forceinline__ float as_f(float x) { return x; }
__device__ __forceinline__ double abs_of(double x) { return fabs(x); }
__device__ __forceinline__ float abs_of(float x) { return fabsf(x); }

// Footprint of one axis: first pixel, number of bounds, and the first bound's
// unrounded value a = (start px - origin) / res as a double-float.  Returns
// false when the footprint misses the image.
template <typename T>
__device__ __forceinline__ bool axis_footprint(const StepConsts &c, double half_len, df hl,
                                               T coord, int n_pix, int16_t &start,
                                               int16_t &count, float &a_hi, float &a_lo) {
    const df x = df_of(coord);
    const df centre = df_add(hl, x);
    const df org = df_add(centre, c.nhalf_sig_df);
    const df top = df_add(centre, c.half_sig_df);
    df qlo = df_mul(org, c.inv_px_df), qhi = df_mul(top, c.inv_px_df);
    // far outside the image (and beyond int range): nothing to splat
    if (!(qhi.hi > -4.f) || !(qlo.hi < (float)n_pix + 4.f)) return false;
    qlo.hi = fmaxf(qlo.hi, -8.f);  // only the clamped first pixel 0 matters below this
    qhi.hi = fminf(qhi.hi, (float)n_pix + 8.f);
    int lo, hi;
    if (!df_floor(qlo, lo)) lo = (int)floor(((half_len + as_d(coord)) - c.half_sig) / c.px);
    if (!df_ceil(qhi, hi)) hi = (int)ceil(((half_len + as_d(coord)) + c.half_sig) / c.px);
    const int i0 = max(lo, 0), i1 = min(hi, n_pix);
    if (i1 < i0) return false;
    start = (int16_t)i0;
    count = (int16_t)(i1 - i0 + 1);
    const df a = df_mul(df_add(df_mul_i(c.px_df, i0), df_neg(org)), c.inv_res_df);
    a_hi = a.hi;
    a_lo = a.lo;
    return true;
}

// The splat record of one emitter at one sub-step: depth key and table slot,
// footprint along x and y, box-table entry when the pixel bounds are a fixed
// stride apart, and the weight w = norm * res^2.  rel0..2 are the emitter's
// depth, x and y relative to the focal point.
// origins: also give box-path records their FP64 footprint origins (x0, y0),
// which the FP64 splat's exact bound decisions read.  T: double, or float for
// FP32 positions (the same record as for their FP64 values, with less FP64 work).
template <typename T>
__device__ __forceinline__ void make_record(const StepConsts &c, T rel0, T rel1, T rel2,
                                            double norm, const int32_t *key_slot,
                                            int32_t *status, int i, int s, ScStepRec &rec,
                                            bool origins = false) {
    rec.box_off = 0;
    rec.x0 = rec.y0 = 0.0;
    rec.ax_hi = rec.ax_lo = rec.ay_hi = rec.ay_lo = 0.f;
    rec.i_start = rec.j_start = 0;
    rec.n_i = rec.n_j = 0;
    rec.box = 0;
    rec.box_local = 0;
    rec.slot = -1;
    rec.w = 0.f;
    if (norm <= 0.0) return;  // overlay_signal returns early (_epifm.py:216-217)
    // a non-finite position or normalisation: the reference's math.floor
    // raises ValueError (_epifm.py:233); reported here (status bit 7)
    if (!isfinite(rel1) || !isfinite(rel2) || !isfinite(norm)) {
        flag_status(status, 7, i, s, 0);
        return;
    }
    // depth key: int(|depth| / res) inside depth_cutoff + res, else -1 (_epifm.py:76-88)
    const T depth = abs_of(rel0);
    const float df32 = as_f(depth);
    bool inside = df32 < c.cut_f * (1.f - 1e-6f);
    if (!(inside || df32 > c.cut_f * (1.f + 1e-6f))) inside = as_d(depth) < c.depth_cutoff + c.res;
    int key = -1;
    if (inside) {
        const float q = df32 * c.inv_res_f;  // three roundings: |error| < 2e-7 q
        const float r = rintf(q);
        key = fabsf(q - r) > 5e-7f * fmaxf(1.f, q) ? (int)floorf(q)
                                                   : (int)floor(as_d(depth) / c.res);
        if (key > c.max_key) {
            flag_status(status, 0, i, s, 0);
            return;
        }
    }
    const int idx = key >= 0 ? key : c.max_key + 1;
    const int slot = key_slot[idx];
    if (slot < 0) {
        flag_status(status, 1, i, s, key);
        return;
    }
    int16_t si = 0, ni = 0, sj = 0, nj = 0;
    float axh, axl, ayh, ayl;
    if (!axis_footprint(c, c.half_w, c.half_w_df, rel1, c.nw, si, ni, axh, axl)) return;
    if (!axis_footprint(c, c.half_h, c.half_h_df, rel2, c.nh, sj, nj, ayh, ayl)) return;
    if (ni < 2 || nj < 2) return;
    float rx, ry;
    const float dx = df_round(df{axh, axl}, rx), dy = df_round(df{ayh, ayl}, ry);
    // Box path: with an integer pitch of P grid rows, bound k is ceil(a) + P k
    // for every k unless a lies within 1e-9 of an integer (FP64 evaluation
    // noise is ~1e-12 here, the double-float a within 1e-9 of it); those
    // emitters keep the summed-area path, which needs the FP64 origins.
    if (c.box_p > 0 && fabsf(dx) > 1e-9f && fabsf(dy) > 1e-9f) {
        // entry of pixel (i_start, j_start) in the phase-major box table of the
        // key: first rows m = l0 + P >= 1 split as (m mod P, m div P), l0 = ceil(a)
        const int P = c.box_p, NQ = c.box_nq, NB = SC_BOX_BLOCK_FLOATS(NQ);
        const int mx = (int)rx + (dx > 0.f ? 1 : 0) + P, my = (int)ry + (dy > 0.f ? 1 : 0) + P;
        const int phase = (mx % P) * P + (my % P);
        rec.box = 1 + phase;
        rec.box_local = ((mx / P) << 16) | (my / P);
        rec.box_off = (int64_t)slot * ((int64_t)P * P * NB) + (int64_t)phase * NB +
                      (mx / P) * NQ + my / P;
        if (origins) {
            rec.x0 = (c.half_w + as_d(rel1)) - c.half_sig;
            rec.y0 = (c.half_h + as_d(rel2)) - c.half_sig;
        }
    } else {
        rec.x0 = (c.half_w + as_d(rel1)) - c.half_sig;
        rec.y0 = (c.half_h + as_d(rel2)) - c.half_sig;
    }
    rec.ax_hi = axh;
    rec.ax_lo = axl;
    rec.ay_hi = ayh;
    rec.ay_lo = ayl;
    rec.i_start = si;
    rec.n_i = ni;
    rec.j_start = sj;
    rec.n_j = nj;
    rec.slot = slot;
    rec.w = (float)(norm * (c.res * c.res));
}

}  // namespace sc
