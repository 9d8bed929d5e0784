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

// floor(x / d) and ceil(x / d) as the reference computes them (one correctly
// rounded FP64 division, then floor / ceil).  The quotient is estimated in
// FP32 (relative error < 2^-22); only when the estimate lies within 1e-3 of an
// integer -- where the rounding of the true division could decide the result
// -- is the FP64 division evaluated.  FP64 instructions run at 1/64 of the
// FP32 rate on this GPU; the estimate costs one conversion.
__device__ __forceinline__ double floor_div(double x, double d, float inv_d) {
    const float q = (float)x * inv_d;
    if (fabsf(q - rintf(q)) > 1e-3f * fmaxf(1.f, fabsf(q))) return (double)floorf(q);
    return floor(x / d);
}

__device__ __forceinline__ double ceil_div(double x, double d, float inv_d) {
    const float q = (float)x * inv_d;
    if (fabsf(q - rintf(q)) > 1e-3f * fmaxf(1.f, fabsf(q))) return (double)ceilf(q);
    return ceil(x / d);
}

// Footprint of one axis (_epifm.py:233-258): first pixel, number of bounds,
// the exact FP64 origin, and the first bound's unrounded value a as a
// double-float (a_hi + a_lo, ~1e-12 absolute).
__device__ __forceinline__ void axis_footprint(double half_len, double coord, double half_sig,
                                               double px, float inv_px, double inv_res,
                                               int n_pix, double &origin, int16_t &start,
                                               int16_t &count, float &a_hi, float &a_lo) {
    const double centre = half_len + coord;
    origin = centre - half_sig;
    const double lo = floor_div(origin, px, inv_px);
    const double hi = ceil_div(centre + half_sig, px, inv_px);
    const double lo_c = fmax(lo, 0.0);
    const double hi_c = fmin(hi, (double)n_pix);
    start = 0;
    count = 0;
    a_hi = a_lo = 0.f;
    if (!(hi_c >= lo_c)) return;
    const int i0 = (int)lo_c;
    const int n = (int)hi_c - i0 + 1;
    start = (int16_t)i0;
    count = (int16_t)n;
    const double a = (__dmul_rn((double)i0, px) - origin) * inv_res;
    a_hi = (float)a;
    a_lo = (float)(a - (double)a_hi);
}

// a - rint(a) from its double-float form (exact to ~1e-11 near zero).
__device__ __forceinline__ float frac_to_int(float a_hi, float a_lo, float &r) {
    r = rintf(a_hi);
    return (a_hi - r) + a_lo;
}

__device__ __forceinline__ void make_record(const StepConsts &c, double rel0, double rel1,
                                            double rel2, double norm, const int32_t *key_slot,
                                            int32_t *status, int i, int s, ScStepRec &rec) {
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
    const double depth = fabs(rel0);
    int key;
    if (depth < c.depth_cutoff + c.res) {
        const double kd = floor_div(depth, c.res, c.inv_res_f);  // int() of a non-negative
        if (kd > (double)c.max_key) {
            flag_status(status, 0, i, s, 0);
            return;
        }
        key = (int)kd;
    } else {
        key = -1;
    }
    const int idx = key >= 0 ? key : c.max_key + 1;
    const int slot = key_slot[idx];
    if (slot < 0) {
        flag_status(status, 1, i, s, key);
        return;
    }
    int16_t si, ni, sj, nj;
    float axh, axl, ayh, ayl;
    double x0, y0;
    axis_footprint(c.half_w, rel1, c.half_sig, c.px, c.inv_px_f, c.inv_res, c.nw, x0, si, ni, axh,
                   axl);
    axis_footprint(c.half_h, rel2, c.half_sig, c.px, c.inv_px_f, c.inv_res, c.nh, y0, sj, nj, ayh,
                   ayl);
    if (ni < 2 || nj < 2) return;
    float rx, ry;
    const float dx = frac_to_int(axh, axl, rx), dy = frac_to_int(ayh, ayl, ry);
    // Box path: with an integer pitch of P grid rows, bound k is ceil(a) + P k
    // for every k unless a lies within 1e-9 of an integer (FP64 evaluation
    // noise and the estimate of a are ~1e-12 here); those emitters keep the
    // summed-area path.
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
    }
    rec.x0 = x0;
    rec.y0 = y0;
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
