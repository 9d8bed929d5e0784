// Shared device helpers for the scopyon_gb300 kernels: error reporting,
// double-float (hi + lo FP32 pair) arithmetic, and the Philox4x32-10
// counter-based generator (Salmon, Moraes, Dror, Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC'11).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#include "../../include/scopyon_gb300.h"

namespace sc {

// ------------------------------------------------------------------ errors
void set_error(const char *fmt, ...);
int cuda_status(cudaError_t err, const char *what);
int launch_status(const char *what);

#define SC_REQUIRE(cond, ...)            \
    do {                                 \
        if (!(cond)) {                   \
            ::sc::set_error(__VA_ARGS__); \
            return SC_ERR_ARG;           \
        }                                \
    } while (0)

// A caller buffer (workspace, scratch) smaller than the call needs.
#define SC_REQUIRE_CAP(cond, ...)        \
    do {                                 \
        if (!(cond)) {                   \
            ::sc::set_error(__VA_ARGS__); \
            return SC_ERR_CAPACITY;      \
        }                                \
    } while (0)

// Blocks for a grid-stride kernel: `want` blocks, at most one full wave of
// resident blocks on the current device (occupancy of `fn` at `block`
// threads and `smem` dynamic bytes), so that no block starts a second wave.
int resident_grid(const void *fn, int block, size_t smem, int64_t want);

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// status word helpers (device): first error wins the index slots
__device__ __forceinline__ void flag_status(int32_t *status, int bit, int a, int b, int c) {
    if (status == nullptr) return;
    int old = atomicOr(status, 1 << bit);
    if (old == 0) {
        status[1] = a;
        status[2] = b;
        status[3] = c;
    }
}

// Bounds-checked build (-DSC_BOUNDS_CHECK): in_range(i, n, ...) is false for
// an index outside [0, n) and records it (status bit 8; the index, the bound
// and the check's site in words 1..3), and the caller then skips the access.
// In the normal build it is the constant true and the checks compile away.
// Sites: 1 a splat warp's tile buffer, 2 its block-copy ring, 3 the tile
// buffers a pixel's merge reads, 4 a record's place in the bin lists, 5 its
// bin, 6 the register splat's tile buffer.
constexpr int kBoundsBit = 8;
#ifdef SC_BOUNDS_CHECK
__device__ __forceinline__ bool in_range(int64_t i, int64_t n, int32_t *status, int site) {
    if (i >= 0 && i < n) return true;
    flag_status(status, kBoundsBit, (int)i, (int)n, site);
    return false;
}
#else
__device__ __forceinline__ bool in_range(int64_t, int64_t, int32_t *, int) { return true; }
#endif

// ------------------------------------------------------------ double-float
// A value v is held as hi + lo with hi = fl32(v) and lo = fl32(v - hi).
struct df {
    float hi, lo;
};

// Error-free sum of two floats (Knuth TwoSum).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// hi + lo of a double, on the device (three FP64-pipe conversions and one add).
__device__ __forceinline__ df df_from(double x) {
    const float h = __double2float_rn(x);
    return df{h, __double2float_rn(x - (double)h)};
}

// (s, e) with |e| small against s -> normalised pair (Fast2Sum).
__device__ __forceinline__ df df_norm(float s, float e) {
    const float h = s + e;
    return df{h, e - (h - s)};
}

__device__ __forceinline__ df df_add(df a, df b) {
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    e += a.lo + b.lo;
    return df_norm(s, e);
}

__device__ __forceinline__ df df_neg(df a) { return df{-a.hi, -a.lo}; }

// Product with an error-free FMA for hi * hi; relative error ~2^-46.
__device__ __forceinline__ df df_mul(df a, df b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return df_norm(p, e);
}

// a * k for an integer |k| < 2^24 (exact as a float).
__device__ __forceinline__ df df_mul_i(df a, int k) {
    const float kf = (float)k;
    const float p = a.hi * kf;
    float e = fmaf(a.hi, kf, -p);
    e = fmaf(a.lo, kf, e);
    return df_norm(p, e);
}

// Nearest integer r of a = hi + lo and the remainder a - r (exact to ~2^-46 |a|).
__device__ __forceinline__ float df_round(df a, float &r) {
    r = rintf(a.hi);
    return (a.hi - r) + a.lo;
}

// acc += sign * (hi + lo), keeping acc as an unnormalised (s, e) pair.
__device__ __forceinline__ void df_acc(float &s, float &e, float hi, float lo, float sign) {
    float t, err;
    two_sum(s, sign * hi, t, err);
    s = t;
    e += err + sign * lo;
}

// ------------------------------------------- FP64 work on the integer pipes
// GB300 runs FP64 instructions (arithmetic, compares, conversions) at about
// 1/64 of the FP32 rate; these two replace a conversion and a compare that
// the Brownian sub-step loops would otherwise issue to the FP64 pipe.

// float -> double on the integer pipes: sign, the exponent rebiased by
// 1023 - 127 = 896, the 23 fraction bits moved to the top of the 52.
// Subnormals are normalised (top set bit t of the fraction: exponent field
// t + 874); zeros and infinities keep their sign; a NaN becomes a quiet NaN
// with its payload.  Equal, bit for bit, to the conversion instruction for
// every non-NaN float.
__device__ __forceinline__ double f2d_exact(float f) {
    const uint32_t u = __float_as_uint(f);
    const uint32_t e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
    const uint64_t sign = (uint64_t)(u >> 31) << 63;
    uint64_t bits;
    if (e == 0u) {
        if (m == 0u) {
            bits = sign;
        } else {
            const int t = 31 - __clz((int)m);
            bits = sign | ((uint64_t)(t + 874) << 52) |
                   (((uint64_t)m << (52 - t)) & 0xfffffffffffffull);
        }
    } else if (e == 0xffu) {
        bits = sign | (0x7ffull << 52) | ((uint64_t)(m ? (m | 0x400000u) : 0u) << 29);
    } else {
        bits = sign | ((uint64_t)(e + 896u) << 52) | ((uint64_t)m << 29);
    }
    return __longlong_as_double((long long)bits);
}

// A signed integer that orders doubles as their values do, except that -0.0
// comes before +0.0 and NaNs fall outside [-inf, +inf]: so key(lo) <= key(x) <=
// key(hi) implies lo <= x <= hi (the converse fails only for signed zeros and
// NaN, which callers send down their FP64 path).
__device__ __forceinline__ long long order_key(double x) {
    const long long b = __double_as_longlong(x);
    return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}

// ------------------------------------------------------------------ Philox
struct u4 {
    uint32_t x, y, z, w;
};

__device__ __forceinline__ u4 philox4x32_10(u4 ctr, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(M0, ctr.x), lo0 = M0 * ctr.x;
        uint32_t hi1 = __umulhi(M1, ctr.z), lo1 = M1 * ctr.z;
        u4 n;
        n.x = hi1 ^ ctr.y ^ k0;
        n.y = lo1;
        n.z = hi0 ^ ctr.w ^ k1;
        n.w = lo0;
        ctr = n;
        k0 += W0;
        k1 += W1;
    }
    return ctr;
}

// (sin, cos) of 2 pi u for u in (0, 1), the Box-Muller angle: the hardware's
// approximate sine and cosine of 2 pi (u - 1/2), in [-pi, pi) where their
// absolute error is about 5e-7, negated.  All on the FP32 and SFU pipes (the
// angle needs no more accuracy than this for standard normals).
__device__ __forceinline__ void sincos_2pi(float u, float *s, float *c) {
    float sn, cs;
    __sincosf(6.28318530718f * (u - 0.5f), &sn, &cs);
    *s = -sn;
    *c = -cs;
}

// uniform in (0, 1) from 32 bits
__device__ __forceinline__ float u01f(uint32_t x) {
    return (float)(x >> 8) * (1.0f / 16777216.0f) + (0.5f / 16777216.0f);
}

// uniform in (0, 1) from 64 bits, double precision
__device__ __forceinline__ double u01d(uint32_t a, uint32_t b) {
    uint64_t v = ((uint64_t)a << 21) ^ (uint64_t)(b >> 11);
    return ((double)(v & ((1ull << 53) - 1)) + 0.5) * (1.0 / 9007199254740992.0);
}

// A stream of Philox outputs for one (key, counter) pair: counter.w advances.
struct rng_stream {
    uint32_t k0, k1;
    u4 ctr;
    u4 buf;
    int left;
    __device__ rng_stream(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2)
        : k0((uint32_t)seed), k1((uint32_t)(seed >> 32)), left(0) {
        ctr.x = c0;
        ctr.y = c1;
        ctr.z = c2;
        ctr.w = 0;
    }
    __device__ uint32_t next() {
        if (left == 0) {
            buf = philox4x32_10(ctr, k0, k1);
            ctr.w += 1;
            left = 4;
        }
        uint32_t v = left == 4 ? buf.x : left == 3 ? buf.y : left == 2 ? buf.z : buf.w;
        --left;
        return v;
    }
    __device__ float uniform() { return u01f(next()); }
    __device__ double uniform_d() {
        uint32_t a = next();
        return u01d(a, next());
    }
    // standard normal, Box-Muller on two uniforms (u1 >= 2^-25: the
    // approximate logarithm's relative error, ~2^-22, is far below what any
    // test of the draws resolves)
    __device__ float normal() {
        float u1 = uniform(), u2 = uniform();
        float r = sqrtf(-2.0f * __logf(u1));
        float s, c;
        sincos_2pi(u2, &s, &c);
        return r * c;
    }
};

}  // namespace sc
