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
#include "bin.cuh"
#include "steps.cuh"

namespace {

struct DiffConsts {
    int n, n_sub, ndim, boundary, n_class, identity, layout;
    int n_sig;  // FP32 sigma table entries staged in shared memory (0: none)
    int64_t step0;
    const int64_t *frame;
    uint64_t seed;
    double lower[3], upper[3];
    float lower_f[3], upper_f[3];
    double scale, origin[3], ux[3], uy[3], uz[3];
    const double *class_box;  // [n_class][6] lower xyz, upper xyz (optional)
    const double *trans;      // [n_sub][n_class][n_class] cumulative transitions (optional)
    const double *uniforms;   // [n_sub][n] injected transition uniforms (optional)
};

// Wall box of a particle's class: the class table's entry, else the common box.
__device__ __forceinline__ void class_walls(const DiffConsts &c, int cls, int d, double &lo,
                                            double &hi) {
    if (c.class_box) {
        lo = c.class_box[cls * 6 + d];
        hi = c.class_box[cls * 6 + 3 + d];
    } else {
        lo = c.lower[d];
        hi = c.upper[d];
    }
}

// a < b as the FP64 compare gives it, from the order keys ka, kb: two zeros
// are equal whatever their signs (NaN aside, which the clamp below handles).
__device__ __forceinline__ bool key_less(long long ka, long long kb, double a, double b) {
    return ka < kb &&
           ((__double_as_longlong(a) | __double_as_longlong(b)) & 0x7fffffffffffffffLL) != 0;
}

// Reflecting walls at lo and hi: a point inside is returned as it is; one
// outside is mirrored in the wall it crossed until it is inside (at most 64
// times), then clamped.  The compares run on the integer pipes (order keys):
// GB300 issues FP64 instructions at about 1/64 of the FP32 rate, and a
// predicated-off FP64 instruction costs as much as an executed one, so the
// only FP64 work is one fused multiply-add per reflection and the clamp.
__device__ __forceinline__ double reflect_walls(double x, double lo, double hi) {
    const long long klo = sc::order_key(lo), khi = sc::order_key(hi);
    long long kx = sc::order_key(x);
    bool below = key_less(kx, klo, x, lo), above = key_less(khi, kx, hi, x);
    if (!below && !above) return x;
    for (int it = 0; it < 64 && (below || above); ++it) {
        const double wall = below ? lo : hi;
        x = 2 * wall - x;
        kx = sc::order_key(x);
        below = key_less(kx, klo, x, lo);
        above = key_less(khi, kx, hi, x);
    }
    return fmin(fmax(x, lo), hi);
}

__device__ __forceinline__ double wrap_axis(double x, double lo, double hi, int boundary) {
    if (boundary == 1) {  // periodic: (x - lo) mod (hi - lo) + lo, result in [lo, hi)
        const double len = hi - lo;
        if (!(len > 0.0)) return lo;  // a flat axis stays on its wall (sampling2.py:44-48)
        double r = fmod(x - lo, len);
        if (r < 0) r += len;
        return r + lo;
    }
    if (boundary == 2) return reflect_walls(x, lo, hi);
    return x;
}

// ------------------------------------------------ native moves in FP32
// With Philox normals (native mode) a particle's position is an FP32 value,
// held exactly in the FP64 state and rows: a move is x = fma(sigma, n, x) in
// FP32, then the walls in FP32.  GB300 issues FP64 at about 1/64 of the FP32
// rate, so the FP64 move cost as much as the rest of a sub-step; the FP32
// position resolves 2^-24 of its value (0.004 nm at 40 um), and a trajectory
// of 20,000 sub-steps drifts by well under a nanometre from an FP64 one.
// Positions that enter a launch as FP64 values are rounded to FP32 first.
// Exact mode (the caller's normals) keeps the FP64 moves above, bit for bit
// the reference's.

// Reflecting walls in FP32: mirrored in the wall crossed until inside (at
// most 64 times), then clamped.
__device__ __forceinline__ float reflect_walls_f(float x, float lo, float hi) {
    if (x >= lo && x <= hi) return x;
    for (int it = 0; it < 64 && !(x >= lo && x <= hi); ++it)
        x = fmaf(2.f, x < lo ? lo : hi, -x);
    return fminf(fmaxf(x, lo), hi);
}

__device__ __forceinline__ float wrap_axis_f(float x, float lo, float hi, int boundary) {
    if (boundary == 1) {  // periodic, as wrap_axis
        const float len = hi - lo;
        if (!(len > 0.f)) return lo;
        float r = fmodf(x - lo, len);
        if (r < 0.f) r += len;
        return r + lo;
    }
    if (boundary == 2) return reflect_walls_f(x, lo, hi);
    return x;
}

// The FP32 walls of class cls on every axis.
__device__ __forceinline__ void class_walls_f(const DiffConsts &c, int cls, float *lo, float *hi) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (c.class_box) {
            lo[d] = __double2float_rn(c.class_box[cls * 6 + d]);
            hi[d] = __double2float_rn(c.class_box[cls * 6 + 3 + d]);
        } else {
            lo[d] = c.lower_f[d];
            hi[d] = c.upper_f[d];
        }
    }
}

// FP32 sigma of (sub-step s, class cls, axis d): from the block's shared copy
// of the launch's table (kSig), else converted from the FP64 table.  The
// choice is a template parameter: as a run-time test the compiler predicates
// the conversion into every sub-step, and a predicated-off FP64 instruction
// occupies GB300's FP64 pipe as long as an executed one.
template <bool kSig>
__device__ __forceinline__ float sigma_f(const DiffConsts &c, const float *s_sig,
                                         const double *sigma, int s, int cls, int d) {
    const int e = (s * c.n_class + cls) * 3 + d;
    if (kSig) return s_sig[e];
    return __double2float_rn(sigma[e]);
}

// Stages the launch's sigma table in shared memory as FP32 (all threads).
__device__ __forceinline__ void stage_sigma(const DiffConsts &c, const double *sigma, float *s_sig) {
    for (int e = threadIdx.x; e < c.n_sig; e += blockDim.x) s_sig[e] = __double2float_rn(sigma[e]);
}

// Largest sigma table (floats) staged in shared memory.
constexpr int kSigMax = 6144;

// Formatted position [depth, x, y] of a sampling-frame point (base.py:61-110).
__device__ __forceinline__ void format_point(const DiffConsts &c, const double *p, double *q) {
    if (c.ndim == 2) {
        q[0] = 0.0;
        q[1] = c.scale == 1.0 ? p[0] : __dmul_rn(p[0], c.scale);
        q[2] = c.scale == 1.0 ? p[1] : __dmul_rn(p[1], c.scale);
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
    // radii sqrt(-2 ln u) as x rsqrt(x) (relative error a few 1e-7); x is
    // kept above 0, since u01f rounds its largest values to 1 and x rsqrt(x)
    // of 0 is 0 * inf
    const float xa = fmaxf(-2.f * __logf(u1), 1e-30f), xb = fmaxf(-2.f * __logf(u3), 1e-30f);
    const float ra = xa * rsqrtf(xa), rb = xb * rsqrtf(xb);
    float sa, ca, sb, cb;
    sc::sincos_2pi(u2, &sa, &ca);
    sc::sincos_2pi(u4, &sb, &cb);
    nrm[0] = ra * ca;
    nrm[1] = ra * sa;
    nrm[2] = rb * cb;
}

// Uniform in [0, 1) with 53 random bits for the class transition of
// particle i at global step g: Philox4x32-10, counter (i, g, 0x7a5e1f0b).
__device__ __forceinline__ double philox_uniform(const DiffConsts &c, int i, uint64_t g) {
    const sc::u4 r = sc::philox4x32_10({(uint32_t)i, (uint32_t)g, (uint32_t)(g >> 32), 0x7a5e1f0bu},
                                       (uint32_t)c.seed, (uint32_t)(c.seed >> 32));
    return ((double)(r.x >> 5) * 67108864.0 + (double)(r.y >> 6)) * (1.0 / 9007199254740992.0);
}

// Class after a move: the first b with cumulative probability row[b] >= u
// (numpy.searchsorted side 'left', sampling2.py:63-66); the last class when
// rounding leaves u above every entry.
__device__ __forceinline__ int next_class(const double *row, int n_class, double u) {
    int b = 0;
    while (b < n_class - 1 && row[b] < u) ++b;
    return b;
}

// The class transition of particle i after sub-step s (global step g).
__device__ __forceinline__ int transition(const DiffConsts &c, int cls, int i, int s, uint64_t g) {
    const double u = c.uniforms ? c.uniforms[(size_t)s * c.n + i] : philox_uniform(c, i, g);
    return next_class(c.trans + ((size_t)s * c.n_class + cls) * c.n_class, c.n_class, u);
}

// One sub-step of one axis d of a particle: x += sigma_d * n_d (the
// reference's 0.0 + sigma * gauss; the normal from the caller's nv, else the
// FP32 Philox normal), then the walls of the particle's class on that axis.
// kInjected selects the normals at compile time: as a run-time test the
// compiler predicates both forms, and the FP64 pipe (about 1/64 of the FP32
// rate on GB300) then issues the injected form's multiply and add as well.
template <bool kInjected>
__device__ __forceinline__ double move_axis(const DiffConsts &c, double x, int d, int cls,
                                            double sg, double nv, float nrm) {
    if (kInjected) x += __dmul_rn(sg, nv);
    else x = fma(sg, sc::f2d_exact(nrm), x);
    if (c.boundary) {
        double lo, hi;
        class_walls(c, cls, d, lo, hi);
        x = wrap_axis(x, lo, hi, c.boundary);
    }
    return x;
}

// One sub-step of a particle on every axis.  The axes are independent, so
// moving and wrapping one axis at a time equals moving all, then wrapping.
// The loop runs over a fixed 3 (ndim is 2 or 3) so that p stays in registers.
template <bool kInjected>
__device__ __forceinline__ void move_point(const DiffConsts &c, double *p, int cls,
                                           const double *sg, const double *nv, const float *nrm) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (d >= c.ndim) break;
        p[d] = move_axis<kInjected>(c, p[d], d, cls, sg[d], kInjected ? nv[d] : 0.0,
                                    kInjected ? 0.f : nrm[d]);
    }
}

constexpr int kDiffThreads = 128;

// Exact mode (the caller's normals, FP64 moves): one thread per particle,
// sub-steps in order.  Each warp stages its 32 rows of a sub-step ([depth,
// x, y, id, state], 40 B each) in shared memory and writes the 1280
// contiguous bytes with five coalesced 8-byte stores per lane: 40 full
// sectors per warp and sub-step, where a row per lane would touch 32 sectors
// with each of its five stores.  particles NULL: no rows.
__global__ void __launch_bounds__(kDiffThreads)
diffuse_exact_kernel(DiffConsts c, double *pos, int32_t *klass, const double *sigma,
                     const double *normals, double *particles) {
    __shared__ double rows[kDiffThreads * 5];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const int first = i - lane;  // this warp's first particle
    if (first >= c.n) return;    // whole warps only: the staging below is warp-wide
    const bool live = i < c.n;
    const int n_rows = min(32, c.n - first);
    double *stage = rows + (threadIdx.x - lane) * 5;
    double p[3] = {0.0, 0.0, 0.0};
    int k = 0;
    if (live) {
        p[0] = pos[3 * i];
        p[1] = pos[3 * i + 1];
        p[2] = pos[3 * i + 2];
        k = klass ? klass[i] : 0;
    }
    const int64_t step0 = c.step0 + (c.frame ? *c.frame * c.n_sub : 0);
    const double id = (double)i;
    for (int s = 0; s < c.n_sub; ++s) {
        const size_t idx = (size_t)s * c.n + i;
        if (particles) {
            double f[3];
            format_point(c, p, f);
            double *q = stage + lane * 5;
            q[0] = f[0];
            q[1] = f[1];
            q[2] = f[2];
            q[3] = id;
            q[4] = 1.0;
            __syncwarp();
            double *dst = particles + ((size_t)s * c.n + first) * 5;
#pragma unroll
            for (int r = 0; r < 5; ++r) {
                const int e = lane + 32 * r;
                if (e < n_rows * 5) dst[e] = stage[e];
            }
            __syncwarp();
        }
        if (!live) continue;
        // one Brownian step
        const double *sg = sigma + ((size_t)s * c.n_class + k) * 3;
        move_point<true>(c, p, k, sg, normals + idx * c.ndim, nullptr);
        if (c.trans) k = transition(c, k, i, s, (uint64_t)(step0 + s));
    }
    if (!live) return;
    pos[3 * i] = p[0];
    pos[3 * i + 1] = p[1];
    pos[3 * i + 2] = p[2];
    if (c.trans) klass[i] = k;
}

// The formatted row of an FP32 position (as format_point on its FP64 value):
// with the identity transform a permutation, converted on the integer pipes.
__device__ __forceinline__ void format_point_f(const DiffConsts &c, const float *p, double *f) {
    if (c.identity && c.ndim == 3) {
        f[0] = sc::f2d_exact(p[2]);
        f[1] = sc::f2d_exact(p[0]);
        f[2] = sc::f2d_exact(p[1]);
    } else if (c.ndim == 2 && c.scale == 1.0) {
        f[0] = 0.0;
        f[1] = sc::f2d_exact(p[0]);
        f[2] = sc::f2d_exact(p[1]);
    } else {
        const double q[3] = {sc::f2d_exact(p[0]), sc::f2d_exact(p[1]), sc::f2d_exact(p[2])};
        format_point(c, q, f);
    }
}

// Native mode (Philox normals, FP32 moves): one thread per particle,
// sub-steps in order.  LAYOUT 0 writes the rows of diffuse_exact_kernel
// (staged per warp, coalesced); LAYOUT 1 writes one 16-byte row (depth, x, y,
// 0) as FP32 per particle and sub-step -- the formatted position exactly,
// which the identity transform keeps FP32 -- a warp's 32 rows one 512-byte
// coalesced store; LAYOUT 2 writes no rows (the positions only advance).
template <int LAYOUT, bool kSig>
__global__ void __launch_bounds__(kDiffThreads)
diffuse_native_kernel(DiffConsts c, double *pos, int32_t *klass, const double *sigma,
                      void *particles) {
    extern __shared__ float s_sig[];  // [n_sub][n_class][3] FP32 when kSig
    __shared__ double rows[LAYOUT == 0 ? kDiffThreads * 5 : 1];
    if (kSig) {
        stage_sigma(c, sigma, s_sig);
        __syncthreads();
    }
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const int first = i - lane;
    if (first >= c.n) return;
    const bool live = i < c.n;
    const int n_rows = min(32, c.n - first);
    double *stage = rows + (LAYOUT == 0 ? (threadIdx.x - lane) * 5 : 0);
    float p[3] = {0.f, 0.f, 0.f};
    int k = 0;
    if (live) {
        p[0] = __double2float_rn(pos[3 * i]);
        p[1] = __double2float_rn(pos[3 * i + 1]);
        p[2] = __double2float_rn(pos[3 * i + 2]);
        k = klass ? klass[i] : 0;
    }
    float lo[3], hi[3];
    class_walls_f(c, k, lo, hi);
    const int64_t step0 = c.step0 + (c.frame ? *c.frame * c.n_sub : 0);
    const double id = (double)i;
    for (int s = 0; s < c.n_sub; ++s) {
        if (LAYOUT == 0) {
            double f[3];
            format_point_f(c, p, f);
            double *q = stage + lane * 5;
            q[0] = f[0];
            q[1] = f[1];
            q[2] = f[2];
            q[3] = id;
            q[4] = 1.0;
            __syncwarp();
            double *dst = static_cast<double *>(particles) + ((size_t)s * c.n + first) * 5;
#pragma unroll
            for (int r = 0; r < 5; ++r) {
                const int e = lane + 32 * r;
                if (e < n_rows * 5) dst[e] = stage[e];
            }
            __syncwarp();
        } else if (LAYOUT == 1) {
            if (live)
                static_cast<float4 *>(particles)[(size_t)s * c.n + i] =
                    make_float4(c.ndim == 3 ? p[2] : 0.f, p[0], p[1], 0.f);
        }
        if (!live) continue;
        float nrm[3];
        philox_normals(c, i, (uint64_t)(step0 + s), nrm);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            if (d >= c.ndim) break;
            const float x = fmaf(sigma_f<kSig>(c, s_sig, sigma, s, k, d), nrm[d], p[d]);
            p[d] = c.boundary ? wrap_axis_f(x, lo[d], hi[d], c.boundary) : x;
        }
        if (c.trans) {
            const int k1 = transition(c, k, i, s, (uint64_t)(step0 + s));
            if (k1 != k && c.class_box) class_walls_f(c, k1, lo, hi);
            k = k1;
        }
    }
    if (!live) return;
    pos[3 * i] = sc::f2d_exact(p[0]);
    pos[3 * i + 1] = sc::f2d_exact(p[1]);
    pos[3 * i + 2] = sc::f2d_exact(p[2]);
    if (c.trans) klass[i] = k;
}

// Native frame records for 32 particles per CTA, in phases per chunk of up to
// 32 sub-steps:
//   1. all warps draw the Philox normals of every (sub-step, particle); when
//      the excitation does not depend on the particle (EPI, or a flat field
//      whose depth is always 0) the last warp computes the emitted photons
//      and the normalisation of each sub-step once;
//   2. the position chains, in sub-step order with the operations of
//      diffuse_kernel, one lane per particle, storing each sub-step's
//      position in shared memory.  Without class transitions the axes are
//      independent chains and warp d runs axis d; with transitions warp 0
//      runs all axes and the class.  When the excitation is uniform the last
//      warp runs the photon-budget chains meanwhile (one subtraction per
//      sub-step), zeroing the normalisation of the sub-steps at which a
//      particle is bleached;
//   3. otherwise (TIRF with depth) all warps, a warp per sub-step and a lane
//      per particle, evaluate the excitation, the emitted photons and the
//      normalisation of every (sub-step, particle): the FP64 exponentials and
//      divisions, independent of one another, run on every warp instead of
//      on a chain; then, with bleaching, warp 0 runs the budget chains;
//   4. all warps build the records, a warp per sub-step and a lane per
//      particle (32 consecutive records, coalesced stores).
// The records equal those of sc_diffuse_steps followed by sc_emitter_steps bit
// for bit: every quantity is formed by the same FP64 expression as there.
// FP64 work runs with full warps only (GB300's FP64 rate is ~1/64 of FP32, so
// a warp with a few active lanes wastes it).
#ifndef SC_REC_WARPS
#define SC_REC_WARPS 4
#endif
constexpr int kRecWarps = SC_REC_WARPS;
static_assert(kRecWarps >= 4, "the chain phase takes warps 0-2 and the last warp");

// Shared memory of one CTA for `chunk` sub-steps: positions [chunk][32][3] and
// normalisations [chunk][32] (FP64), per-sub-step photons and normalisation
// [chunk] (FP64), normals [chunk][32][3] (FP32).  The emitted photons of each
// (sub-step, particle) [chunk][32] (FP64, phase 3) reuse the normals' space,
// which the position chains have consumed by then.
inline size_t rec_shared_bytes(int chunk) {
    return (size_t)chunk * (32 * 3 * sizeof(double) + 32 * sizeof(double) + 2 * sizeof(double) +
                            32 * 3 * sizeof(float));
}

#ifndef SC_REC_MIN_BLOCKS
#define SC_REC_MIN_BLOCKS 6
#endif
// kF32: native records from the FP32 positions (focal point at the origin,
// identity transform); a template parameter, so that each instance holds one
// form of the record arithmetic (a smaller kernel for the instruction cache).
template <bool kInjected, bool kSig, bool kF32>
__global__ void __launch_bounds__(kRecWarps * 32, SC_REC_MIN_BLOCKS)
native_records_kernel(DiffConsts c, sc::StepConsts k, int chunk, double *pos,
                      int32_t *klass, const double *sigma, const double *normals,
                      const double *unit_time, double *budget, const int32_t *key_slot,
                      ScStepRec *recs, sc::TileGeom g, sc::BinLayout bl, int32_t *status) {
    extern __shared__ double rec_smem[];
    double *s_pos = rec_smem;
    double *s_norm = s_pos + chunk * 32 * 3;
    double *s_emit = s_norm + chunk * 32;
    double *s_norm1 = s_emit + chunk;
    float *s_nrm = reinterpret_cast<float *>(s_norm1 + chunk);
    double *s_e = s_norm1 + chunk;  // [chunk][32], over the normals after phase 2
    float *s_sig = s_nrm + chunk * 32 * 3;  // native: the FP32 sigma table when c.n_sig
    if (!kInjected && kSig) {
        stage_sigma(c, sigma, s_sig);
        __syncthreads();
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = blockIdx.x * 32 + lane;  // this lane's particle
    // native mode keeps the sub-steps' positions as FP32 values ([chunk][32][3]
    // floats over the start of s_pos), exact mode as FP64
    float *s_posf = reinterpret_cast<float *>(s_pos);
    auto pos_d = [&](int j, double *q) {
        if (kInjected) {
            const double *ps = s_pos + (j * 32 + lane) * 3;
            q[0] = ps[0];
            q[1] = ps[1];
            q[2] = ps[2];
        } else {
            const float *ps = s_posf + (j * 32 + lane) * 3;
            q[0] = sc::f2d_exact(ps[0]);
            q[1] = sc::f2d_exact(ps[1]);
            q[2] = sc::f2d_exact(ps[2]);
        }
    };
    // native records from the FP32 positions directly (no FP64 conversions)
    constexpr bool f32_records = !kInjected && kF32;
    const bool live = i < c.n;
    const int64_t step0 = c.step0 + (c.frame ? *c.frame * c.n_sub : 0);
    // the excitation is the same for every particle: EPI, or a flat field
    // (format_point gives depth 0.0, so the depth offset is -focal[0])
    const bool epi = isinf(k.penetration);
    const bool uniform = epi || c.ndim == 2;
    const bool axis_chains = c.trans == nullptr;
    const int budget_warp = uniform ? kRecWarps - 1 : 0;
    // chain state: axis `warp` (axis chains) or every axis and the class (warp
    // 0 otherwise); the photon budget on budget_warp
    double p[3] = {0.0, 0.0, 0.0}, b = 0.0;
    float pf[3] = {0.f, 0.f, 0.f};  // native mode: the FP32 positions (see diffuse_native_kernel)
    float lo[3], hi[3];
    int cls = 0;
    if (live) {
        if (axis_chains && warp < c.ndim) {
            p[0] = pos[3 * i + warp];  // an axis chain keeps its coordinate in p[0]
            cls = klass ? klass[i] : 0;
        } else if (!axis_chains && warp == 0) {
            p[0] = pos[3 * i];
            p[1] = pos[3 * i + 1];
            p[2] = pos[3 * i + 2];
            cls = klass[i];
        }
        if (!kInjected) {
            pf[0] = __double2float_rn(p[0]);
            pf[1] = __double2float_rn(p[1]);
            pf[2] = __double2float_rn(p[2]);
        }
        if (warp == budget_warp && k.bleaching) b = budget[i];
    }
    if (!kInjected) class_walls_f(c, cls, lo, hi);
    for (int s0 = 0; s0 < c.n_sub; s0 += chunk) {
        const int ns = min(chunk, c.n_sub - s0);
        // 1. normals; per-sub-step photons and normalisation when uniform
        if (!kInjected) {
            for (int j = warp; j < ns; j += kRecWarps) {
                float nrm[3] = {0.f, 0.f, 0.f};
                if (live) philox_normals(c, i, (uint64_t)(step0 + s0 + j), nrm);
                float *d = s_nrm + (j * 32 + lane) * 3;
                d[0] = nrm[0];
                d[1] = nrm[1];
                d[2] = nrm[2];
            }
        }
        if (uniform && warp == kRecWarps - 1) {
            const double amp =
                epi ? k.amplitude0
                    : __dmul_rn(k.amplitude0, exp(-fabs(0.0 - k.focal[0]) / k.penetration));
            for (int j = lane; j < ns; j += 32) {
                const double n_emit = sc::emit_photons(k, amp, unit_time[s0 + j]);
                s_emit[j] = n_emit;
                // p_state = 1: __dmul_rn(1.0, n_emit) is n_emit
                s_norm1[j] = __dmul_rn(k.norm_coeff, n_emit / (4.0 * M_PI));
            }
        }
        __syncthreads();
        // 2. the position chains (and the budget chains when uniform)
        if (live) {
            if (!kInjected && axis_chains && warp < c.ndim) {
                const int d = warp;
                float x = pf[0];
                for (int j = 0; j < ns; ++j) {
                    const int s = s0 + j;
                    s_posf[(j * 32 + lane) * 3 + d] = x;
                    x = fmaf(sigma_f<kSig>(c, s_sig, sigma, s, cls, d),
                             s_nrm[(j * 32 + lane) * 3 + d], x);
                    if (c.boundary) x = wrap_axis_f(x, lo[d], hi[d], c.boundary);
                }
                pf[0] = x;
            } else if (!kInjected && !axis_chains && warp == 0) {
                for (int j = 0; j < ns; ++j) {
                    const int s = s0 + j;
                    float *ps = s_posf + (j * 32 + lane) * 3;
                    ps[0] = pf[0];
                    ps[1] = pf[1];
                    ps[2] = pf[2];
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        if (d >= c.ndim) break;
                        const float x = fmaf(sigma_f<kSig>(c, s_sig, sigma, s, cls, d),
                                             s_nrm[(j * 32 + lane) * 3 + d], pf[d]);
                        pf[d] = c.boundary ? wrap_axis_f(x, lo[d], hi[d], c.boundary) : x;
                    }
                    const int k1 = transition(c, cls, i, s, (uint64_t)(step0 + s));
                    if (k1 != cls && c.class_box) class_walls_f(c, k1, lo, hi);
                    cls = k1;
                }
            } else if (axis_chains && warp < c.ndim) {
                const int d = warp;
                double x = p[0];
                const double *sgd = sigma + (size_t)cls * 3 + d;
                const size_t sg_step = (size_t)c.n_class * 3;
                // the next sub-step's sigma and normal are loaded a step ahead
                double sg = sgd[(size_t)s0 * sg_step];
                double nv = kInjected ? normals[((size_t)s0 * c.n + i) * c.ndim + d] : 0.0;
                float nr = kInjected ? 0.f : s_nrm[lane * 3 + d];
                for (int j = 0; j < ns; ++j) {
                    const int s = s0 + j;
                    s_pos[(j * 32 + lane) * 3 + d] = x;
                    double sg_n = 0.0, nv_n = 0.0;
                    float nr_n = 0.f;
                    if (j + 1 < ns) {
                        sg_n = sgd[(size_t)(s + 1) * sg_step];
                        if (kInjected) nv_n = normals[((size_t)(s + 1) * c.n + i) * c.ndim + d];
                        else nr_n = s_nrm[((j + 1) * 32 + lane) * 3 + d];
                    }
                    x = move_axis<kInjected>(c, x, d, cls, sg, nv, nr);
                    sg = sg_n;
                    nv = nv_n;
                    nr = nr_n;
                }
                p[0] = x;
            } else if (!axis_chains && warp == 0) {
                for (int j = 0; j < ns; ++j) {
                    const int s = s0 + j;
                    double *ps = s_pos + (j * 32 + lane) * 3;
                    ps[0] = p[0];
                    ps[1] = p[1];
                    ps[2] = p[2];
                    const double *sg = sigma + ((size_t)s * c.n_class + cls) * 3;
                    move_point<kInjected>(
                        c, p, cls, sg, kInjected ? normals + ((size_t)s * c.n + i) * c.ndim : nullptr,
                        s_nrm + (j * 32 + lane) * 3);
                    cls = transition(c, cls, i, s, (uint64_t)(step0 + s));
                }
            }
            if (uniform && warp == kRecWarps - 1) {
                // p_state = 0 gives norm_coeff * (0 / 4 pi) = 0: no record
                for (int j = 0; j < ns; ++j) {
                    double norm = s_norm1[j];
                    if (k.bleaching) {
                        double nb = b - s_emit[j];
                        if (nb <= 0) {
                            nb = 0;
                            norm = 0.0;
                        }
                        b = nb;
                    }
                    s_norm[j * 32 + lane] = norm;
                }
            }
        }
        __syncthreads();
        // 3. excitation, photons and normalisation of every (sub-step,
        // particle) when they depend on its depth; then the budget chains
        if (!uniform) {
            if (live) {
                for (int j = warp; j < ns; j += kRecWarps) {
                    double q[3];
                    pos_d(j, q);
                    double f[3];
                    format_point(c, q, f);
                    const double rel0 = f[0] - k.focal[0];
                    const double amp = __dmul_rn(k.amplitude0, exp(-fabs(rel0) / k.penetration));
                    const double n_emit = sc::emit_photons(k, amp, unit_time[s0 + j]);
                    s_e[j * 32 + lane] = n_emit;
                    s_norm[j * 32 + lane] = __dmul_rn(k.norm_coeff, n_emit / (4.0 * M_PI));
                }
            }
            if (k.bleaching) {
                __syncthreads();
                if (warp == 0 && live) {
                    for (int j = 0; j < ns; ++j) {
                        double nb = b - s_e[j * 32 + lane];
                        if (nb <= 0) {
                            nb = 0;
                            s_norm[j * 32 + lane] = 0.0;
                        }
                        b = nb;
                    }
                }
                __syncthreads();
            } else {
                __syncwarp();  // phase 4 reads what phase 3 of the same warp wrote
            }
        }
        // 4. records: warp w takes sub-steps w, w + kRecWarps, ...
        if (live) {
            for (int j = warp; j < ns; j += kRecWarps) {
                const int s = s0 + j;
                const double norm = s_norm[j * 32 + lane];
                ScStepRec rec;
                if (f32_records) {
                    const float *ps = s_posf + (j * 32 + lane) * 3;
                    sc::make_record<float>(k, c.ndim == 3 ? ps[2] : 0.f, ps[0], ps[1], norm,
                                           key_slot, status, i, s, rec);
                } else {
                    double q[3];
                    pos_d(j, q);
                    if (c.ndim != 3) q[2] = 0.0;
                    double f[3];
                    format_point(c, q, f);
                    if (k.focal_zero)
                        sc::make_record<double>(k, f[0], f[1], f[2], norm, key_slot, status, i, s,
                                                rec);
                    else
                        sc::make_record<double>(k, f[0] - k.focal[0], f[1] - k.focal[1],
                                                f[2] - k.focal[2], norm, key_slot, status, i, s,
                                                rec);
                }
                recs[(size_t)s * c.n + i] = rec;
                if (bl.count) sc::bin_record(g, rec, s * c.n + i, bl.count, bl.rec_bin, sc::rank_array(bl));
            }
        }
        __syncthreads();
    }
    if (live) {
        if (!kInjected) {
            p[0] = sc::f2d_exact(pf[0]);
            p[1] = sc::f2d_exact(pf[1]);
            p[2] = sc::f2d_exact(pf[2]);
        }
        if (axis_chains) {
            if (warp < c.ndim) pos[3 * i + warp] = p[0];
        } else if (warp == 0) {
            pos[3 * i] = p[0];
            pos[3 * i + 1] = p[1];
            pos[3 * i + 2] = p[2];
            klass[i] = cls;
        }
        if (warp == budget_warp && k.bleaching) budget[i] = b;
    }
}

}  // namespace

namespace {

int diff_consts(const ScDiffuseParams *p, DiffConsts &c) {
    SC_REQUIRE(p != nullptr, "sc_diffuse_steps: params are NULL");
    SC_REQUIRE(p->n_particles >= 0 && p->n_sub >= 0, "sc_diffuse_steps: negative sizes");
    SC_REQUIRE(p->ndim == 2 || p->ndim == 3, "sc_diffuse_steps: ndim=%d must be 2 or 3", p->ndim);
    SC_REQUIRE(p->boundary >= 0 && p->boundary <= 2, "sc_diffuse_steps: boundary=%d", p->boundary);
    SC_REQUIRE(p->n_class >= 1, "sc_diffuse_steps: n_class=%d", p->n_class);
    if (p->boundary && !p->d_class_box)
        for (int d = 0; d < p->ndim; ++d)
            SC_REQUIRE(p->upper[d] > p->lower[d] || (p->boundary == 1 && p->upper[d] == p->lower[d]),
                       "sc_diffuse_steps: empty box along axis %d", d);
    c.n = p->n_particles;
    c.n_sub = p->n_sub;
    c.ndim = p->ndim;
    c.boundary = p->boundary;
    c.n_class = p->n_class;
    c.step0 = p->step0;
    c.frame = p->d_frame;
    c.class_box = p->d_class_box;
    c.trans = p->d_trans;
    c.uniforms = p->d_uniforms;
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
    for (int d = 0; d < 3; ++d) {
        c.lower_f[d] = (float)p->lower[d];
        c.upper_f[d] = (float)p->upper[d];
    }
    SC_REQUIRE(p->layout >= 0 && p->layout <= 1, "sc_diffuse_steps: layout=%d", p->layout);
    c.layout = p->layout;
    const int64_t n_sig = (int64_t)p->n_sub * p->n_class * 3;
    c.n_sig = n_sig <= kSigMax ? (int)n_sig : 0;
    return SC_OK;
}

}  // namespace

extern "C" int sc_diffuse_steps(const ScDiffuseParams *p, double *d_pos, int32_t *d_class,
                                const double *d_sigma, const double *d_normals,
                                double *d_particles, void *stream) {
    DiffConsts c;
    int rc = diff_consts(p, c);
    if (rc) return rc;
    if (c.n == 0 || c.n_sub == 0) return SC_OK;
    SC_REQUIRE(d_pos && d_sigma, "sc_diffuse_steps: NULL pointer");
    SC_REQUIRE(!p->d_trans || d_class, "sc_diffuse_steps: transitions need the class array");
    SC_REQUIRE(c.layout == 0 || (!d_normals && (c.ndim == 3 ? c.identity : c.scale == 1.0)),
               "sc_diffuse_steps: FP32 rows (layout 1) need native draws and the identity "
               "transform");
    const int block = kDiffThreads;
    const int grid = (c.n + block - 1) / block;
    cudaStream_t st = sc::as_stream(stream);
    if (d_normals) {
        diffuse_exact_kernel<<<grid, block, 0, st>>>(c, d_pos, d_class, d_sigma, d_normals,
                                                     d_particles);
    } else {
        const size_t smem = (size_t)c.n_sig * sizeof(float);
        const int lay = !d_particles ? 2 : c.layout;
#define SC_DIFF_LAUNCH(L)                                                                       \
    if (c.n_sig)                                                                                \
        diffuse_native_kernel<L, true><<<grid, block, smem, st>>>(c, d_pos, d_class, d_sigma,   \
                                                                  d_particles);                 \
    else                                                                                        \
        diffuse_native_kernel<L, false><<<grid, block, 0, st>>>(c, d_pos, d_class, d_sigma,     \
                                                                d_particles);
        if (lay == 2) {
            SC_DIFF_LAUNCH(2)
        } else if (lay == 1) {
            SC_DIFF_LAUNCH(1)
        } else {
            SC_DIFF_LAUNCH(0)
        }
#undef SC_DIFF_LAUNCH
    }
    return sc::launch_status("sc_diffuse_steps");
}

extern "C" int sc_native_records(const ScDiffuseParams *p, const ScStepParams *sp, double *d_pos,
                                 int32_t *d_class, const double *d_sigma,
                                 const double *d_normals, const double *d_unit_time,
                                 double *d_budget, const int32_t *d_key_slot, ScStepRec *d_recs,
                                 const ScSplatParams *bin_p, void *d_bin_ws, size_t bin_ws_bytes,
                                 int32_t *d_status, void *stream) {
    DiffConsts c;
    int rc = diff_consts(p, c);
    if (rc) return rc;
    sc::StepConsts k;
    rc = sc::step_consts(sp, k);
    if (rc) return rc;
    SC_REQUIRE(k.n_particles == c.n && k.n_sub == c.n_sub,
               "sc_native_records: diffusion and step sizes differ");
    if (c.n == 0 || c.n_sub == 0) return SC_OK;
    SC_REQUIRE(d_pos && d_sigma && d_unit_time && d_key_slot && d_recs,
               "sc_native_records: NULL pointer");
    SC_REQUIRE(!k.bleaching || d_budget, "sc_native_records: bleaching needs a budget array");
    SC_REQUIRE(!p->d_trans || d_class, "sc_native_records: transitions need the class array");
    sc::TileGeom g{};
    sc::BinLayout bl{nullptr, nullptr, nullptr, nullptr, nullptr};
    if (bin_p) {
        rc = sc::tile_geom(bin_p, g);
        if (rc) return rc;
        const int64_t n_rec = (int64_t)c.n * c.n_sub;
        SC_REQUIRE(n_rec < (1ll << 31), "sc_native_records: %lld records", (long long)n_rec);
        SC_REQUIRE(g.n_images == 1 && g.nw == k.nw && g.nh == k.nh,
                   "sc_native_records: bin geometry is not the frame's");
        SC_REQUIRE_CAP(d_bin_ws && bin_ws_bytes >= sc_bin_workspace_bytes((int)n_rec, g.n_tiles),
                   "sc_native_records: bin workspace %zu < %zu bytes", bin_ws_bytes,
                   sc_bin_workspace_bytes((int)n_rec, g.n_tiles));
        sc::bin_layout(g, (int)n_rec, d_bin_ws, bin_ws_bytes, bl);
    }
    const int chunk = c.n_sub < 32 ? c.n_sub : 32;
    const bool sig = !d_normals && c.n_sig > 0;
    const size_t smem = rec_shared_bytes(chunk) + (sig ? (size_t)c.n_sig * sizeof(float) : 0);
    // native records from FP32 positions when the formatted position is a
    // permutation of them and the focal point is the origin
    const bool f32 = !d_normals && k.focal_zero && (c.ndim == 3 ? c.identity != 0 : c.scale == 1.0);
    auto kern = d_normals ? native_records_kernel<true, false, false>
                : sig ? (f32 ? native_records_kernel<false, true, true>
                             : native_records_kernel<false, true, false>)
                      : (f32 ? native_records_kernel<false, false, true>
                             : native_records_kernel<false, false, false>);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return sc::cuda_status(e, "sc_native_records: smem attribute");
    }
    kern<<<(c.n + 31) / 32, kRecWarps * 32, smem, sc::as_stream(stream)>>>(
        c, k, chunk, d_pos, d_class, d_sigma, d_normals, d_unit_time, d_budget, d_key_slot, d_recs,
        g, bl, d_status);
    return sc::launch_status("sc_native_records");
}
