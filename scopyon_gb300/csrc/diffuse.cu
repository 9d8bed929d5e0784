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

namespace {

struct DiffConsts {
    int n, n_sub, ndim, boundary, n_class;
    int64_t step0;
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

__global__ void diffuse_kernel(DiffConsts c, double *pos, const int32_t *klass,
                               const double *sigma, const double *normals, double *particles) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    double p[3] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
    const int k = klass ? klass[i] : 0;
    for (int s = 0; s < c.n_sub; ++s) {
        // formatted position of this sub-step
        double *q = particles + ((size_t)s * c.n + i) * 5;
        if (c.ndim == 3) {
            const double d0 = __dmul_rn(p[0], c.scale) - c.origin[0];
            const double d1 = __dmul_rn(p[1], c.scale) - c.origin[1];
            const double d2 = __dmul_rn(p[2], c.scale) - c.origin[2];
            // numpy.dot of a length-3 row: ((a0 b0 + a1 b1) + a2 b2)
            q[0] = (__dmul_rn(d0, c.uz[0]) + __dmul_rn(d1, c.uz[1])) + __dmul_rn(d2, c.uz[2]);
            q[1] = (__dmul_rn(d0, c.ux[0]) + __dmul_rn(d1, c.ux[1])) + __dmul_rn(d2, c.ux[2]);
            q[2] = (__dmul_rn(d0, c.uy[0]) + __dmul_rn(d1, c.uy[1])) + __dmul_rn(d2, c.uy[2]);
        } else {
            q[0] = 0.0;
            q[1] = __dmul_rn(p[0], c.scale);
            q[2] = __dmul_rn(p[1], c.scale);
        }
        q[3] = (double)i;
        q[4] = 1.0;
        // one Brownian step: x_d += sigma_d * n_d (the reference's 0.0 + sigma * gauss)
        const double *sg = sigma + ((size_t)s * c.n_class + k) * 3;
        if (normals) {
            const double *nv = normals + ((size_t)s * c.n + i) * c.ndim;
            for (int d = 0; d < c.ndim; ++d) p[d] += __dmul_rn(sg[d], nv[d]);
        } else {
            const uint64_t g = (uint64_t)(c.step0 + s);
            sc::u4 r = sc::philox4x32_10({(uint32_t)i, (uint32_t)g, (uint32_t)(g >> 32), 0x5d1ff05eu},
                                         (uint32_t)c.seed, (uint32_t)(c.seed >> 32));
            // Box-Muller on two 53-bit uniforms -> two normals, a third from the next draw
            const double u1 = sc::u01d(r.x, r.y), u2 = sc::u01d(r.z, r.w);
            const double rad = sqrt(-2.0 * log(u1));
            double sn, cs;
            sincospi(2.0 * u2, &sn, &cs);
            double nrm[3] = {rad * cs, rad * sn, 0.0};
            if (c.ndim == 3) {
                sc::u4 r2 = sc::philox4x32_10({(uint32_t)i, (uint32_t)g, (uint32_t)(g >> 32), 0x5d1ff05fu},
                                              (uint32_t)c.seed, (uint32_t)(c.seed >> 32));
                const double v1 = sc::u01d(r2.x, r2.y), v2 = sc::u01d(r2.z, r2.w);
                nrm[2] = sqrt(-2.0 * log(v1)) * cospi(2.0 * v2);
            }
            for (int d = 0; d < c.ndim; ++d) p[d] += sg[d] * nrm[d];
        }
        if (c.boundary)
            for (int d = 0; d < c.ndim; ++d) p[d] = wrap_axis(p[d], c.lower[d], c.upper[d], c.boundary);
    }
    pos[3 * i] = p[0];
    pos[3 * i + 1] = p[1];
    pos[3 * i + 2] = p[2];
}

}  // namespace

extern "C" int sc_diffuse_steps(const ScDiffuseParams *p, double *d_pos, const int32_t *d_class,
                                const double *d_sigma, const double *d_normals,
                                double *d_particles, void *stream) {
    SC_REQUIRE(p != nullptr, "sc_diffuse_steps: params are NULL");
    SC_REQUIRE(p->n_particles >= 0 && p->n_sub >= 0, "sc_diffuse_steps: negative sizes");
    SC_REQUIRE(p->ndim == 2 || p->ndim == 3, "sc_diffuse_steps: ndim=%d must be 2 or 3", p->ndim);
    SC_REQUIRE(p->boundary >= 0 && p->boundary <= 2, "sc_diffuse_steps: boundary=%d", p->boundary);
    SC_REQUIRE(p->n_class >= 1, "sc_diffuse_steps: n_class=%d", p->n_class);
    if (p->n_particles == 0 || p->n_sub == 0) return SC_OK;
    SC_REQUIRE(d_pos && d_sigma && d_particles, "sc_diffuse_steps: NULL pointer");
    if (p->boundary)
        for (int d = 0; d < p->ndim; ++d)
            SC_REQUIRE(p->upper[d] > p->lower[d], "sc_diffuse_steps: empty box along axis %d", d);
    DiffConsts c;
    c.n = p->n_particles;
    c.n_sub = p->n_sub;
    c.ndim = p->ndim;
    c.boundary = p->boundary;
    c.n_class = p->n_class;
    c.step0 = p->step0;
    c.seed = p->seed;
    c.scale = p->scale;
    for (int d = 0; d < 3; ++d) {
        c.lower[d] = p->lower[d];
        c.upper[d] = p->upper[d];
        c.origin[d] = p->origin[d];
        c.ux[d] = p->unit_x[d];
        c.uy[d] = p->unit_y[d];
        c.uz[d] = p->unit_z[d];
    }
    const int block = 128;
    diffuse_kernel<<<(c.n + block - 1) / block, block, 0, sc::as_stream(stream)>>>(
        c, d_pos, d_class, d_sigma, d_normals, d_particles);
    return sc::launch_status("sc_diffuse_steps");
}
