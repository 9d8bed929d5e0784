// Emitter physics per particle and exposure sub-step -> splat records.
//
// One thread owns one particle slot and walks the frame's sub-steps in order,
// so the photon budget (bleaching) and the true_data sums are accumulated in
// exactly the reference's sequence:
//   amplitude  = amplitude0 * exp(-|depth| / penetration)     _epifm.py:1281-1289
//   n_emit     = QY * (amplitude * x_sec * dt) * (1 - 10^-A)   _epifm.py:1344-1360
//   budget    -= n_emit; <= 0 -> p_state = 0                   _epifm.py:1294-1306
//   norm       = norm_coeff * (p_state * n_emit / 4 pi)        _epifm.py:1309-1315
//   depth key  = int(|depth| / res) or -1 past the cutoff      _epifm.py:76-88
//   footprint  = pixel range and grid origin along x and y    _epifm.py:224-258
// All of it is FP64 (a few dozen flops per record) so that keys, footprint
// bounds and bleaching decisions are the reference's.
#include "sc_common.cuh"
#include "steps.cuh"

namespace {

// One input row: depth, x, y and p_state (FP64 rows, or the FP32 rows of
// sc_diffuse_steps layout 1, converted exactly on the integer pipes).
struct Row {
    double d, x, y, state;
};

__device__ __forceinline__ Row load_row(const void *rows, int layout, size_t idx) {
    if (layout == 1) {
        const float4 v = static_cast<const float4 *>(rows)[idx];
        return Row{sc::f2d_exact(v.x), sc::f2d_exact(v.y), sc::f2d_exact(v.z), 1.0};
    }
    const double *q = static_cast<const double *>(rows) + idx * 5;
    return Row{q[0], q[1], q[2], q[4]};
}

// Pass 1, one thread per particle slot, sub-steps in order: excitation,
// emitted photons, the photon-budget chain and the normalisation.  The
// normalisation of each (sub-step, slot) is parked in its record's x0 field
// for pass 2 (0: nothing to splat).
__global__ void emitter_physics_kernel(sc::StepConsts c, const void *particles,
                                       const double *unit_time, const uint8_t *present,
                                       double *budget, double *optinfo, ScStepRec *recs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n_particles) return;
    double b = c.bleaching ? budget[i] : 0.0;
    double acc[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) acc[k] = 0.0;
    const bool epi = isinf(c.penetration);
    for (int s = 0; s < c.n_sub; ++s) {
        const size_t idx = (size_t)s * c.n_particles + i;
        if (present && !present[idx]) {
            recs[idx].x0 = 0.0;  // absent at this sub-step: no record, no state change
            continue;
        }
        const Row q = load_row(particles, c.row_layout, idx);
        const double ut = unit_time[s];
        double p_state = q.state;
        const double rel0 = q.d - c.focal[0];
        // amplitude0 * exp(-|depth| / inf) is amplitude0 exactly
        const double amp = epi ? c.amplitude0
                               : __dmul_rn(c.amplitude0, exp(-fabs(rel0) / c.penetration));
        const double n_emit = sc::emit_photons(c, amp, ut);
        if (c.bleaching) {
            double nb = b - n_emit;
            if (nb <= 0) {
                nb = 0;
                p_state = 0.0;
            }
            b = nb;
        }
        const double norm = __dmul_rn(c.norm_coeff, __dmul_rn(p_state, n_emit) / (4.0 * M_PI));
        recs[idx].x0 = norm;
        if (c.with_optinfo) {
            acc[0] += ut;
            acc[1] += __dmul_rn(ut, p_state);
            acc[2] += __dmul_rn(ut, q.x);
            acc[3] += __dmul_rn(ut, q.y);
            acc[4] += __dmul_rn(ut, q.x);
            acc[5] += __dmul_rn(ut, q.y);
            acc[6] += __dmul_rn(ut, rel0);
            acc[7] += norm;
        }
    }
    if (c.bleaching) budget[i] = b;
    if (c.with_optinfo) {
#pragma unroll
        for (int k = 0; k < 8; ++k) optinfo[(size_t)i * 8 + k] = acc[k];
    }
}

// Pass 2, one thread per (sub-step, slot): depth key and footprint.
__global__ void emitter_footprint_kernel(sc::StepConsts c, const void *particles,
                                         const int32_t *key_slot, ScStepRec *recs,
                                         double *norm_out, int32_t *status) {
    const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= (int64_t)c.n_sub * c.n_particles) return;
    const double norm = recs[idx].x0;
    if (norm_out) norm_out[idx] = norm;
    ScStepRec rec;
    const int i = (int)(idx % c.n_particles), s = (int)(idx / c.n_particles);
    if (c.row_layout == 1 && c.focal_zero) {
        // FP32 rows: the record from the FP32 values (as from their FP64 ones)
        const float4 v = static_cast<const float4 *>(particles)[idx];
        sc::make_record<float>(c, v.x, v.y, v.z, norm, key_slot, status, i, s, rec,
                               norm_out != nullptr);
        recs[idx] = rec;
        return;
    }
    const Row q = load_row(particles, c.row_layout, (size_t)idx);
    if (c.focal_zero)
        sc::make_record(c, q.d, q.x, q.y, norm, key_slot, status, i, s, rec,
                        norm_out != nullptr);
    else
        sc::make_record(c, q.d - c.focal[0], q.x - c.focal[1], q.y - c.focal[2], norm,
                        key_slot, status, i, s, rec,
                        norm_out != nullptr);
    recs[idx] = rec;
}

}  // namespace

namespace sc {

int step_consts(const ScStepParams *p, StepConsts &c) {
    SC_REQUIRE(p != nullptr, "step params are NULL");
    SC_REQUIRE(p->px > 0 && p->res > 0, "px and res must be positive");
    SC_REQUIRE(p->nw > 0 && p->nh > 0 && p->nw < 32767 && p->nh < 32767,
               "image size %dx%d out of range", p->nw, p->nh);
    SC_REQUIRE(p->n_signal >= 3, "n_signal=%d too small", p->n_signal);
    SC_REQUIRE(p->max_key >= 0, "max_key=%d", p->max_key);
    SC_REQUIRE(p->n_particles >= 0 && p->n_sub >= 0, "negative sizes");
    c.px = p->px;
    c.res = p->res;
    c.depth_cutoff = p->depth_cutoff;
    for (int k = 0; k < 3; ++k) c.focal[k] = p->focal[k];
    c.nw = p->nw;
    c.nh = p->nh;
    c.n_signal = p->n_signal;
    c.n_sub = p->n_sub;
    c.n_particles = p->n_particles;
    c.max_key = p->max_key;
    c.amplitude0 = p->amplitude0;
    c.penetration = p->penetration;
    c.x_sec = p->x_sec;
    c.qy = p->qy;
    c.beer = p->beer;
    c.norm_coeff = p->norm_coeff;
    c.bleaching = p->bleaching;
    c.with_optinfo = p->with_optinfo;
    c.box_p = p->box_p;
    c.box_nq = p->box_nq;
    SC_REQUIRE(p->box_p >= 0 && p->box_p < 16384, "box_p=%d out of range", p->box_p);
    SC_REQUIRE(p->box_p == 0 || p->box_nq == (p->n_signal + p->box_p - 1) / p->box_p + 1,
               "box_nq=%d inconsistent with box_p=%d", p->box_nq, p->box_p);
    c.half_w = (double)p->nw * p->px * 0.5;
    c.half_h = (double)p->nh * p->px * 0.5;
    c.half_sig = p->res * (double)(p->n_signal - 1) * 0.5;
    c.inv_res = 1.0 / p->res;
    c.inv_px_f = (float)(1.0 / p->px);
    c.inv_res_f = (float)(1.0 / p->res);
    auto split = [](double v) {
        const float h = (float)v;
        return df{h, (float)(v - (double)h)};
    };
    c.half_w_df = split(c.half_w);
    c.half_h_df = split(c.half_h);
    c.half_sig_df = split(c.half_sig);
    c.nhalf_sig_df = split(-c.half_sig);
    c.inv_px_df = split(1.0 / p->px);
    c.px_df = split(p->px);
    c.inv_res_df = split(c.inv_res);
    c.cut_f = (float)(p->depth_cutoff + p->res);
    c.focal_zero = p->focal[0] == 0.0 && p->focal[1] == 0.0 && p->focal[2] == 0.0;
    SC_REQUIRE(p->row_layout == 0 || p->row_layout == 1, "row_layout=%d", p->row_layout);
    c.row_layout = p->row_layout;
    return SC_OK;
}

}  // namespace sc

extern "C" int sc_emitter_steps(const ScStepParams *p, const double *d_particles,
                                const double *d_unit_time, const uint8_t *d_present,
                                const int32_t *d_key_slot,
                                double *d_budget, double *d_optinfo, ScStepRec *d_recs,
                                double *d_norm, int32_t *d_status, void *stream) {
    sc::StepConsts c;
    int rc = sc::step_consts(p, c);
    if (rc) return rc;
    if (c.n_particles == 0 || c.n_sub == 0) return SC_OK;
    SC_REQUIRE(d_particles && d_unit_time && d_key_slot && d_recs,
               "sc_emitter_steps: NULL input/output pointer");
    SC_REQUIRE(!c.bleaching || d_budget, "sc_emitter_steps: bleaching needs a budget array");
    SC_REQUIRE(!c.with_optinfo || d_optinfo, "sc_emitter_steps: optinfo output is NULL");
    cudaStream_t st = sc::as_stream(stream);
    emitter_physics_kernel<<<(c.n_particles + 127) / 128, 128, 0, st>>>(
        c, d_particles, d_unit_time, d_present, d_budget, d_optinfo, d_recs);
    const int64_t n_rec = (int64_t)c.n_sub * c.n_particles;
    emitter_footprint_kernel<<<(unsigned)((n_rec + 255) / 256), 256, 0, st>>>(
        c, d_particles, d_key_slot, d_recs, d_norm, d_status);
    return sc::launch_status("sc_emitter_steps");
}
