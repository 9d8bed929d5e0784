// Brownian trajectories on the device, one frame's sub-steps per launch.
//
// Reference: sample_inputs / move_points (src/scopyon/sampling.py:88-162):
// x_d += N(0, sqrt(2 D_d dt)) per particle and axis at every time step, no
// boundary; sampling2.__move_points (src/scopyon/sampling2.py:33-50) adds a
// periodic wrap.  One thread owns one particle and walks the sub-steps: it
// writes the formatted position of each sub-step ([depth, x, y, m_id,
// p_state] as EPIFMSimulator.__format_data builds it, base.py:61-110), then
// moves the particle.  Normals come from Philox4x32-10 (counter = particle,
// global step) or, for parity with the reference, from a caller array.
// Boundaries: none (reference), periodic (sampling2), reflecting (this engine).
#include "sc_common.cuh"
#include "steps.cuh"

namespace {

struct DiffConsts {
    int n, n_sub, ndim, boundary, n_class, identity;
    int64_t step0;
    const int64_t *frame;
    uint64_t seed;
    double lower[3], upper[3];
    double scale, origin[3], ux[3], uy[3], uz[3];
};

__device__ __forceinline__ double wrap_axis(double x, double lo, double hi, int boundary) {
    if (boundary == 1) {  // periodic: (x - lo) mod (hi - lo) + lo, result in [lo, hi)
        const double len = hi - lo;
        double r = fmod(x - lo, len);
        if (r < 0) r += len;
        return r + lo;
    }
    if (boundary == 2) {  // reflecting walls at lo and hi
        for (int it = 0; it < 64 && (x < lo || x > hi); ++it) x = x < lo ? 2 * lo - x : 2 * hi - x;
        return fmin(fmax(x, lo), hi);
    }
    return x;
}

// Formatted position [depth, x, y] of a sampling-frame point (base.py:61-110).
__device__ __forceinline__ void format_point(const DiffConsts &c, const double *p, double *q) {
    if (c.ndim == 2) {
        q[0] = 0.0;
        q[1] = __dmul_rn(p[0], c.scale);
        q[2] = __dmul_rn(p[1], c.scale);
    } else if (c.identity) {
        q[0] = p[2];
        q[1] = p[0];
        q[2] = p[1];
    } else {
        const double d0 = __dmul_rn(p[0], c.scale) - c.origin[0];
        const double d1 = __dmul_rn(p[1], c.scale) - c.origin[1];
        const double d2 = __dmul_rn(p[2], c.scale) - c.origin[2];
        // numpy.dot of a length-3 row: ((a0 b0 + a1 b1) + a2 b2)
        q[0] = (__dmul_rn(d0, c.uz[0]) + __dmul_rn(d1, c.uz[1])) + __dmul_rn(d2, c.uz[2]);
        q[1] = (__dmul_rn(d0, c.ux[0]) + __dmul_rn(d1, c.ux[1])) + __dmul_rn(d2, c.ux[2]);
        q[2] = (__dmul_rn(d0, c.uy[0]) + __dmul_rn(d1, c.uy[1])) + __dmul_rn(d2, c.uy[2]);
    }
}

// Standard normals for one particle and step: Box-Muller in FP32 on Philox
// words (24-bit uniforms); the positions themselves stay FP64.
__device__ __forceinline__ void philox_normals(const DiffConsts &c, int i, uint64_t g, float *nrm) {
    const sc::u4 r = sc::philox4x32_10({(uint32_t)i, (uint32_t)g, (uint32_t)(g >> 32), 0x5d1ff05eu},
                                       (uint32_t)c.seed, (uint32_t)(c.seed >> 32));
    const float u1 = sc::u01f(r.x), u2 = sc::u01f(r.y), u3 = sc::u01f(r.z), u4 = sc::u01f(r.w);
    const float ra = sqrtf(-2.f * __logf(u1)), rb = sqrtf(-2.f * __logf(u3));
    float sa, ca, sb, cb;
    sincospif(2.f * u2, &sa, &ca);
    sincospif(2.f * u4, &sb, &cb);
    nrm[0] = ra * ca;
    nrm[1] = ra * sa;
    nrm[2] = rb * cb;
}

// One thread per particle, sub-steps in order.  With physics (native frames)
// the thread also runs the emitter physics of each sub-step -- excitation,
// emitted photons, the photon-budget chain -- and parks the normalisation in
// the record's x0 field for the footprint pass (0: nothing to splat).
template <bool PHYSICS>
__global__ void diffuse_kernel(DiffConsts c, sc::StepConsts sc_, double *pos, const int32_t *klass,
                               const double *sigma, const double *normals, double *particles,
                               const double *unit_time, double *budget, ScStepRec *recs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    double p[3] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
    const int k = klass ? klass[i] : 0;
    const int64_t step0 = c.step0 + (c.frame ? *c.frame * c.n_sub : 0);
    double b = PHYSICS && sc_.bleaching ? budget[i] : 0.0;
    const bool epi = PHYSICS && isinf(sc_.penetration);
    for (int s = 0; s < c.n_sub; ++s) {
        const size_t idx = (size_t)s * c.n + i;
        double *q = particles + idx * 5;
        double f[3];
        format_point(c, p, f);
        q[0] = f[0];
        q[1] = f[1];
        q[2] = f[2];
        q[3] = (double)i;
        q[4] = 1.0;
        if (PHYSICS) {
            const double ut = unit_time[s];
            const double rel0 = f[0] - sc_.focal[0];
            double p_state = 1.0;
            const double amp = epi ? sc_.amplitude0
                                   : __dmul_rn(sc_.amplitude0, exp(-fabs(rel0) / sc_.penetration));
            const double n_emit = sc::emit_photons(sc_, amp, ut);
            if (sc_.bleaching) {
                double nb = b - n_emit;
                if (nb <= 0) {
                    nb = 0;
                    p_state = 0.0;
                }
                b = nb;
            }
            recs[idx].x0 = __dmul_rn(sc_.norm_coeff, __dmul_rn(p_state, n_emit) / (4.0 * M_PI));
        }
        // one Brownian step: x_d += sigma_d * n_d (the reference's 0.0 + sigma * gauss)
        const double *sg = sigma + ((size_t)s * c.n_class + k) * 3;
        if (normals) {
            const double *nv = normals + idx * c.ndim;
            for (int d = 0; d < c.ndim; ++d) p[d] += __dmul_rn(sg[d], nv[d]);
        } else {
            float nrm[3];
            philox_normals(c, i, (uint64_t)(step0 + s), nrm);
            for (int d = 0; d < c.ndim; ++d) p[d] += sg[d] * (double)nrm[d];
        }
        if (c.boundary)
            for (int d = 0; d < c.ndim; ++d) p[d] = wrap_axis(p[d], c.lower[d], c.upper[d], c.boundary);
    }
    pos[3 * i] = p[0];
    pos[3 * i + 1] = p[1];
    pos[3 * i + 2] = p[2];
    if (PHYSICS && sc_.bleaching) budget[i] = b;
}

}  // namespace

namespace {

int diff_consts(const ScDiffuseParams *p, DiffConsts &c) {
    SC_REQUIRE(p != nullptr, "sc_diffuse_steps: params are NULL");
    SC_REQUIRE(p->n_particles >= 0 && p->n_sub >= 0, "sc_diffuse_steps: negative sizes");
    SC_REQUIRE(p->ndim == 2 || p->ndim == 3, "sc_diffuse_steps: ndim=%d must be 2 or 3", p->ndim);
    SC_REQUIRE(p->boundary >= 0 && p->boundary <= 2, "sc_diffuse_steps: boundary=%d", p->boundary);
    SC_REQUIRE(p->n_class >= 1, "sc_diffuse_steps: n_class=%d", p->n_class);
    if (p->boundary)
        for (int d = 0; d < p->ndim; ++d)
            SC_REQUIRE(p->upper[d] > p->lower[d], "sc_diffuse_steps: empty box along axis %d", d);
    c.n = p->n_particles;
    c.n_sub = p->n_sub;
    c.ndim = p->ndim;
    c.boundary = p->boundary;
    c.n_class = p->n_class;
    c.step0 = p->step0;
    c.frame = p->d_frame;
    c.seed = p->seed;
    c.scale = p->scale;
    bool ident = p->scale == 1.0;
    const double ex[3] = {1, 0, 0}, ey[3] = {0, 1, 0}, ez[3] = {0, 0, 1};
    for (int d = 0; d < 3; ++d) {
        c.lower[d] = p->lower[d];
        c.upper[d] = p->upper[d];
        c.origin[d] = p->origin[d];
        c.ux[d] = p->unit_x[d];
        c.uy[d] = p->unit_y[d];
        c.uz[d] = p->unit_z[d];
        ident = ident && p->origin[d] == 0.0 && p->unit_x[d] == ex[d] && p->unit_y[d] == ey[d] &&
                p->unit_z[d] == ez[d];
    }
    c.identity = ident ? 1 : 0;
    return SC_OK;
}

}  // namespace

extern "C" int sc_diffuse_steps(const ScDiffuseParams *p, double *d_pos, const int32_t *d_class,
                                const double *d_sigma, const double *d_normals,
                                double *d_particles, void *stream) {
    DiffConsts c;
    int rc = diff_consts(p, c);
    if (rc) return rc;
    if (c.n == 0 || c.n_sub == 0) return SC_OK;
    SC_REQUIRE(d_pos && d_sigma && d_particles, "sc_diffuse_steps: NULL pointer");
    sc::StepConsts none{};
    const int block = 128;
    diffuse_kernel<false><<<(c.n + block - 1) / block, block, 0, sc::as_stream(stream)>>>(
        c, none, d_pos, d_class, d_sigma, d_normals, d_particles, nullptr, nullptr, nullptr);
    return sc::launch_status("sc_diffuse_steps");
}

extern "C" int sc_native_substeps(const ScDiffuseParams *p, const ScStepParams *sp,
                                  double *d_pos, const int32_t *d_class, const double *d_sigma,
                                  const double *d_normals, const double *d_unit_time,
                                  double *d_budget, double *d_particles, ScStepRec *d_recs,
                                  void *stream) {
    DiffConsts c;
    int rc = diff_consts(p, c);
    if (rc) return rc;
    sc::StepConsts k;
    rc = sc::step_consts(sp, k);
    if (rc) return rc;
    SC_REQUIRE(k.n_particles == c.n && k.n_sub == c.n_sub,
               "sc_native_substeps: diffusion and step sizes differ");
    if (c.n == 0 || c.n_sub == 0) return SC_OK;
    SC_REQUIRE(d_pos && d_sigma && d_particles && d_unit_time && d_recs,
               "sc_native_substeps: NULL pointer");
    SC_REQUIRE(!k.bleaching || d_budget, "sc_native_substeps: bleaching needs a budget array");
    const int block = 64;
    diffuse_kernel<true><<<(c.n + block - 1) / block, block, 0, sc::as_stream(stream)>>>(
        c, k, d_pos, d_class, d_sigma, d_normals, d_particles, d_unit_time, d_budget, d_recs);
    return sc::launch_status("sc_native_substeps");
}
