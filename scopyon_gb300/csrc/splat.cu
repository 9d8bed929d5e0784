// Tile splat of emitter footprints onto the pixel grid.
//
// Reference: PointSpreadingFunction.overlay_signal_ (src/scopyon/_epifm.py:224-282).
// For each particle and sub-step it adds, to every pixel (i, j) of the
// footprint, norm * res^2 * sum(P[a0:a1, b0:b1]) where P is the 1-nm
// cartesian PSF grid and the bounds are ceil((i*px - x0) / res).
//
// Records are filed under the tile of their first pixel (bin.cu).  One CTA per
// tile sums the whole footprints of its records into a (tile + halo)^2 buffer
// in shared memory, one FP32 copy per half-warp, then stores the sum over the
// copies to the workspace; a merge pass adds, per pixel, the up to
// (1 + halo/tile)^2 buffers that cover it, in a fixed order.  No atomics, and
// every record is read and processed exactly once.
//
// Pixel sums come from one of two tables of the record's depth key:
//  * box path (integer pixel pitch P, generic positions): the box table holds
//    each pixel's rectangle sum directly, so a footprint is one contiguous
//    block of FP32 values;
//  * summed-area path (everything else): the footprint bounds are recomputed
//    (an FP32 double-float estimate, with the reference's FP64 expression
//    evaluated exactly whenever the estimate is within 1e-6 of an integer),
//    and each pixel's sum folds onto at most 3 x 3 quadrant-table entries of
//    the mirror-symmetric grid, held as double-float pairs (~2^-48 relative).
#include <climits>

#include "sc_common.cuh"
#include "bin.cuh"
#include "fold.cuh"
#include "camera.cuh"


namespace {

struct SplatConsts {
    int tiles_per_image, tiles_y, tile, halo, edge, nw, nh, n_r, n_signal, pitch;
    int64_t table_stride;  // float2 entries per quadrant table
    double px, res;
    float b_hi, b_lo;  // px / res as a double-float
    const float *box;  // box tables (NULL when px / res is not an integer)
    int box_nq;        // rows and columns of a box table block
    int box_p;         // grid rows per pixel of the box tables
    int64_t box_floats;  // floats held in the box tables (every slot)
    uint32_t first_wait_tries;  // polls of each bulk-copy warp's first wait
};

// Footprint bound k of one axis: ceil(((start + k) * px - origin) / res) with
// the first bound clamped at 0 and the last at n_signal (_epifm.py:238-258).
__device__ __forceinline__ int axis_bound(int k, int n, int start, float a_hi, float a_lo,
                                          double origin, const SplatConsts &c) {
    const float kf = (float)k;
    const float p = kf * c.b_hi;
    const float pe = fmaf(kf, c.b_hi, -p);
    float s, e2;
    sc::two_sum(a_hi, p, s, e2);
    const float low = a_lo + (kf * c.b_lo + (pe + e2));
    const float r = rintf(s);
    const float d = (s - r) + low;
    int v;
    if (fabsf(d) >= 1e-6f) {
        v = (int)r + (d > 0.f ? 1 : 0);
    } else {
        // the reference's FP64 sequence; __dmul_rn keeps the product rounded
        // (a contracted fma would skip that rounding and can flip the ceil)
        const double t = (__dmul_rn((double)(start + k), c.px) - origin) / c.res;
        v = (int)ceil(t);
    }
    if (k == 0) v = max(v, 0);
    if (k == n - 1) v = min(v, c.n_signal);
    return v;
}


// One summed-area-path record over its whole footprint, by a whole warp:
// bounds from the exact footprint arithmetic (bx, by: per-warp scratch), each
// pixel from folded quadrant-table sums.
__device__ void splat_sat_record(const ScStepRec &rec, int base, const float2 *__restrict__ sat,
                                 const SplatConsts &c, int *bx, int *by, float *my_acc, int lane) {
    const int i_start = rec.i_start, n_i = rec.n_i, j_start = rec.j_start, n_j = rec.n_j;
    const double x0 = rec.x0, y0 = rec.y0;
    const float axh = rec.ax_hi, axl = rec.ax_lo, ayh = rec.ay_hi, ayl = rec.ay_lo;
    const float w = rec.w;
    for (int b = lane; b < n_i + n_j; b += 32) {
        if (b < n_i) bx[b] = axis_bound(b, n_i, i_start, axh, axl, x0, c);
        else by[b - n_i] = axis_bound(b - n_i, n_j, j_start, ayh, ayl, y0, c);
    }
    __syncwarp();
    const float2 *G = sat + (int64_t)rec.slot * c.table_stride;
    const int ni = n_i - 1, nj = n_j - 1;
    for (int q = lane; q < ni * nj; q += 32) {
        const int a = q / nj, bj = q - (q / nj) * nj;
        int a0 = bx[a], a1 = bx[a + 1], b0 = by[bj], b1 = by[bj + 1];
        sc::slice_bounds(a0, a1, c.n_signal);
        sc::slice_bounds(b0, b1, c.n_signal);
        if (a1 <= a0 || b1 <= b0) continue;
        int uu[3], vv[3];
        float us[3], vs[3];
        const int nu = sc::fold(a0, a1, c.n_r, uu, us);
        const int nv = sc::fold(b0, b1, c.n_r, vv, vs);
        float s = 0.f, e = 0.f;
        for (int iu = 0; iu < nu; ++iu) {
            const float2 *row = G + (int64_t)uu[iu] * c.pitch;
            for (int iv = 0; iv < nv; ++iv) {
                const float2 gv = __ldg(row + vv[iv]);
                sc::df_acc(s, e, gv.x, gv.y, us[iu] * vs[iv]);
            }
        }
        const float val = s + e;
        if (val > 0.f) my_acc[base + a * c.edge + bj] += w * val;
    }
    __syncwarp();
}

// Tile geometry of a CTA; false (after flagging) when a footprint does not
// fit its tile buffer.
__device__ __forceinline__ bool in_buffer(int ox, int oy, int ni, int nj, int E) {
    return ox >= 0 && oy >= 0 && ox + ni <= E && oy + nj <= E;
}

// Box path.  Sums are plain FP32: one warp buffer receives at most a few
// dozen footprints per pixel, and a pixel's value is then the sum of NW warp
// buffers and of at most (1 + halo/tile)^2 tile buffers, so each chain of
// roundings is short (about 1e-6 relative at the densities the engine
// targets; the tests hold 1e-5).
//
// Record m of the tile's box list goes to warp m mod NW, so the warps of a
// CTA finish together.  A warp stages the 32-byte heads of its next 32
// records in shared memory, then takes them one at a time: lane (row0 =
// lane / 16, col = lane % 16) loads rows row0, row0 + 2, ... of footprint
// column col (eight loads in flight), reads the eight buffer values, then
// writes the eight sums.  Footprints wider or taller than 16 pixels take
// further passes.
template <int NW>
__global__ void __launch_bounds__(NW * 32, 32 / NW)
splat_box_kernel(const ScStepRec *__restrict__ recs, const int32_t *__restrict__ tile_start,
                 const int32_t *__restrict__ items, SplatConsts c, float *__restrict__ ws,
                 int32_t *status) {
    extern __shared__ float sm[];
    const int E = c.edge, EE = c.edge * c.edge;
    const int BS = (EE + 31) & ~31;
    float *acc = sm;                                          // [NW][BS]
    int4 *heads = reinterpret_cast<int4 *>(acc + NW * BS);    // [NW][32][2]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tile = blockIdx.x;
    const int t = tile % c.tiles_per_image;
    const int x0 = (t / c.tiles_y) * c.tile, y0 = (t % c.tiles_y) * c.tile;
    for (int i = threadIdx.x; i < NW * BS; i += blockDim.x) sm[i] = 0.f;
    __syncthreads();
    float *my_acc = acc + warp * BS;
    int4 *my_heads = heads + warp * 64;
    const int col = lane & 15, row0 = lane >> 4;
    const int nq = c.box_nq;
    const int it0 = tile_start[tile], it1 = tile_start[tile + 1];
    for (int base = it0 + warp; base < it1; base += NW * 32) {
        const int mine = base + NW * lane;
        if (mine < it1) {
            const int4 *src = reinterpret_cast<const int4 *>(recs + __ldg(items + mine));
            my_heads[2 * lane] = __ldg(src);
            my_heads[2 * lane + 1] = __ldg(src + 1);
        }
        __syncwarp();
        const int cnt = min(32, (it1 - base + NW - 1) / NW);
        for (int k = 0; k < cnt; ++k) {
            const int4 ha = my_heads[2 * k], hb = my_heads[2 * k + 1];
            const int i_start = (int)(int16_t)(ha.z & 0xffff), ni = (ha.z >> 16) - 1;
            const int j_start = (int)(int16_t)(ha.w & 0xffff), nj = (ha.w >> 16) - 1;
            const int ox = i_start - x0, oy = j_start - y0;
            if (!in_buffer(ox, oy, ni, nj, E)) {
                if (lane == 0) sc::flag_status(status, 2, i_start, j_start, tile);
                continue;
            }
            const float w = __int_as_float(hb.x);
            // pixel (i_start + a, j_start + b) is entry box_off + a * NQ + b
            const int64_t off = ((int64_t)ha.y << 32) | (uint32_t)ha.x;
            if (off < 0 || off + (int64_t)(ni - 1) * nq + nj > c.box_floats) {
                if (lane == 0) sc::flag_status(status, 2, (int)(off >> 32), (int)off, tile);
                continue;
            }
            const float *B = c.box + off;
            float *D = my_acc + ox * E + oy;
            for (int cb = 0; cb < nj; cb += 16) {
                const int b = cb + col;
                const bool cok = b < nj;
                for (int a0 = row0; a0 < ni; a0 += 16) {
                    const float *src = B + a0 * nq + b;
                    float *dst = D + a0 * E + b;
                    float v[8], o[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u)
                        v[u] = (cok && a0 + 2 * u < ni) ? __ldg(src + 2 * u * nq) : 0.f;
#pragma unroll
                    for (int u = 0; u < 8; ++u)
                        o[u] = (cok && a0 + 2 * u < ni) ? dst[2 * u * E] : 0.f;
#pragma unroll
                    for (int u = 0; u < 8; ++u)
                        if (cok && a0 + 2 * u < ni) dst[2 * u * E] = fmaf(w, v[u], o[u]);
                }
            }
        }
        __syncwarp();
    }
    __syncthreads();
    float *out = ws + (size_t)tile * EE;
    for (int p = threadIdx.x; p < EE; p += blockDim.x) {
        float sum = 0.f;
#pragma unroll
        for (int w = 0; w < NW; ++w) sum += acc[w * BS + p];
        out[p] = sum;
    }
}

// ---------------------------------------------------------------------------
// Box path, bulk-copy form.
//
// A box record's pixel sums are one contiguous phase block of the box table
// (NQ x NQ floats, 16-byte aligned), and every entry of the block outside the
// footprint is zero as well (those pixels do not meet the PSF grid).  One
// cp.async.bulk moves the block into shared memory; the warp then adds it into
// its tile buffer: block row q goes to buffer row q + dr, block column v to
// buffer column v + dc (dr = ox - qx0, dc = oy - qy0 for a footprint whose
// first pixel, entry (qx0, qy0) of the block, sits at (ox, oy) in the buffer).
// A lane owns block column lane % 16 (lanes >= NQ idle) of the rows of parity
// lane / 16.
//
// The tile buffer has a guard row and column before it, and the stage
// buffers a zero row when NQ is odd, so a footprint whose block starts at
// most one row and column before its first pixel -- every footprint not
// clipped by the image's low edges -- is added as NQ / 2 unconditional row
// pairs.  The others visit only the rows and columns that land in the buffer.
// The buffer keeps even and odd rows in two halves 16 banks apart, so the
// two rows a warp instruction touches never share a bank.
//
// Each warp runs a ring of `stages` block buffers with one mbarrier each; the
// lane that decoded a record issues its copy, `stages` records ahead, so an SM
// holds about warps x stages blocks of HBM reads in flight.  Record m of the
// tile's list is taken by warp m mod NW; the NW buffers are summed at the end.

constexpr uint32_t kWaitTries = 4096;      // polls per wait, each suspending up to:
constexpr uint32_t kSuspendNs = 500000;    // 0.5 ms (a copy lands in microseconds)
// Tile-buffer half row stride: 32 floats, with the odd half 16 floats (mod 32)
// after the even one, so the two rows a warp instruction touches -- (even,
// odd) at equal half-row index or (odd, even) one index apart -- are 16 banks
// apart either way.
constexpr int kBulkBsr = 32;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}

// Waits until the phase of this parity has completed: at most max_tries
// polls, each suspending the thread until completion or kSuspendNs.  The
// result is uniform across the warp.
__device__ __forceinline__ bool warp_wait(uint64_t *bar, uint32_t parity,
                                          uint32_t max_tries = kWaitTries) {
    uint32_t ok = 0;
    for (uint32_t tries = 0; tries < max_tries && !ok; ++tries) {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(smem_u32(bar)), "r"(parity), "r"(kSuspendNs)
            : "memory");
    }
    return __all_sync(0xffffffffu, ok != 0);
}

// One lane: global [src, src + bytes) -> shared dst, completion on bar.
// src, dst and bytes are multiples of 16 bytes.
__device__ __forceinline__ void bulk_copy(void *dst, const void *src, uint32_t bytes,
                                          uint64_t *bar) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// Splat descriptor of one record, decoded by the lane that loaded it:
// (w, (dr + 128) | (dc + 128) << 8, rows [qlo, qhi) as qlo | qhi << 8,
// bit 0: splat it, bit 1: the unconditional path applies).
template <int NQ>
__device__ __forceinline__ int4 decode_record(const ScStepRec *recs, const int32_t *items, int m,
                                              bool valid, int x0, int y0, const SplatConsts &c,
                                              int64_t table_floats, int nb, const float *&src,
                                              int32_t *status, int tile) {
    src = c.box;
    if (!valid) return make_int4(0, 0, 0, 0);
    const int4 *hp = reinterpret_cast<const int4 *>(recs + __ldg(items + m));
    const int4 a = __ldg(hp), b = __ldg(hp + 1);
    const int i_start = (int)(int16_t)(a.z & 0xffff), ni = (a.z >> 16) - 1;
    const int j_start = (int)(int16_t)(a.w & 0xffff), nj = (a.w >> 16) - 1;
    const int ox = i_start - x0, oy = j_start - y0;
    const int qx0 = b.w >> 16, qy0 = b.w & 0xffff;
    const int64_t off = ((int64_t)a.y << 32) | (uint32_t)a.x;
    const int64_t blk = off - ((int64_t)qx0 * NQ + qy0);
    bool ok = in_buffer(ox, oy, ni, nj, c.edge);
    if (!ok) sc::flag_status(status, 2, i_start, j_start, tile);
    if (blk < 0 || blk + nb > table_floats || (blk & 3) != 0) {
        sc::flag_status(status, 2, (int)(blk >> 32), (int)blk, tile);
        ok = false;
    } else {
        src = c.box + blk;
    }
    const int dr = ox - qx0, dc = oy - qy0;
    const int qlo = max(0, -dr), qhi = min(NQ, c.edge - dr);
    const int flags = (ok ? 1 : 0) | (ok && dr >= -1 && dc >= -1 ? 2 : 0);
    return make_int4(b.x, (dr + 128) | ((dc + 128) << 8), qlo | (qhi << 8), flags);
}

// One tile's box-path records through the calling warp's ring of block
// copies (`stages` buffers with one mbarrier each): the warp takes records
// it0 + warp + NW k of the tile's list.  Every copy a call issues is waited
// for before it returns, so the ring is empty between calls; `phase` holds
// each buffer's next wait parity (bit b for buffer b) and carries over.
// Returns false when a wait ran out (after draining the copies in flight).
template <int NW, int NQ>
__device__ __forceinline__ bool bulk_tile_records(
    const ScStepRec *__restrict__ recs, const int32_t *__restrict__ tile_start,
    const int32_t *__restrict__ items, const SplatConsts &c, int stages, int HB,
    int64_t table_floats, int tile, int x0, int y0, float *my_acc, int4 *my_desc,
    float *my_stage, uint64_t *my_bars, uint32_t &phase, uint32_t first_tries,
    int32_t *status) {
    constexpr int BSR = kBulkBsr;
    constexpr int PAIRS = (NQ + 1) / 2, SB = (2 * PAIRS * NQ + 3) & ~3;
    constexpr int NB = SC_BOX_BLOCK_FLOATS(NQ);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int it0 = tile_start[tile], it1 = tile_start[tile + 1];
    // records of this warp: m_k = it0 + warp + NW k, k < K
    const int K = it1 - it0 > warp ? (it1 - it0 - warp + NW - 1) / NW : 0;
    // the block's values, rounded up to 16 bytes (the padding after them is not read)
    constexpr uint32_t bytes = ((NQ * NQ + 3) & ~3) * 4u;
    const int col = lane & 15, rsel = lane >> 4;

    // lane l decodes records 32 q + l of chunks q (cur) and q + 1 (nxt); the
    // descriptors go to shared memory, the block addresses stay in registers
    const float *cur_src, *nxt_src;
    my_desc[lane] = decode_record<NQ>(recs, items, it0 + warp + NW * lane, lane < K, x0, y0, c,
                                      table_floats, NB, cur_src, status, tile);
    my_desc[32 + lane] =
        decode_record<NQ>(recs, items, it0 + warp + NW * (32 + lane), 32 + lane < K, x0, y0, c,
                          table_floats, NB, nxt_src, status, tile);
    __syncwarp();
    if (lane < min(stages, K)) bulk_copy(my_stage + lane * SB, cur_src, bytes, my_bars + lane);
    int s = 0;
    int k = 0;
    for (; k < K; ++k) {
        if (k > 0 && (k & 31) == 0) {
            // chunk k / 32 + 1 replaces chunk k / 32 - 1, whose records are all done
            cur_src = nxt_src;
            const int kk = k + 32 + lane;
            my_desc[(((k >> 5) + 1) & 1) * 32 + lane] =
                decode_record<NQ>(recs, items, it0 + warp + NW * kk, kk < K, x0, y0, c,
                                  table_floats, NB, nxt_src, status, tile);
            __syncwarp();
        }
        if (!warp_wait(my_bars + s, (phase >> s) & 1u, k == 0 ? first_tries : kWaitTries)) {
            if (lane == 0) sc::flag_status(status, 5, k, warp, tile);
            break;
        }
        const int4 d = my_desc[((k >> 5) & 1) * 32 + (k & 31)];
        if (d.w & 1) {
            const float w = __int_as_float(d.x);
            const int dr = (d.y & 0xff) - 128, dc = ((d.y >> 8) & 0xff) - 128;
            // this lane's rows q = 2 i + rsel land in buffer rows dr + q
            const int R = dr + 1 + rsel;
            const float *B = my_stage + s * SB + rsel * NQ + col;
            float *D = my_acc + (R & 1) * HB + (R >> 1) * BSR + dc + 1 + col;
            // bounds-checked build: the warp's tile buffer and stage ring
            const int d0 = (int)(D - my_acc), b0 = (int)(B - my_stage);
            const int acc_floats = (2 * HB + 31) & ~31, stage_floats = stages * SB;
            if (d.w & 2) {
                if (col < NQ && sc::in_range(d0, acc_floats, status, 1) &&
                    sc::in_range(d0 + (PAIRS - 1) * BSR, acc_floats, status, 1) &&
                    sc::in_range(b0 + 2 * (PAIRS - 1) * NQ, stage_floats, status, 2)) {
#pragma unroll
                    for (int i = 0; i < PAIRS; ++i)
                        D[i * BSR] = fmaf(w, B[2 * i * NQ], D[i * BSR]);
                }
            } else {
                const int qlo = d.z & 0xff, qhi = (d.z >> 8) & 0xff;
                if (col < NQ && col + dc >= 0) {
#pragma unroll
                    for (int i = 0; i < PAIRS; ++i) {
                        const int q = 2 * i + rsel;
                        if (q >= qlo && q < qhi && sc::in_range(d0 + i * BSR, acc_floats, status, 1) &&
                            sc::in_range(b0 + 2 * i * NQ, stage_floats, status, 2))
                            D[i * BSR] = fmaf(w, B[2 * i * NQ], D[i * BSR]);
                    }
                }
            }
        }
        __syncwarp();
        // refill this buffer with record k + stages: its own lane issues
        const int kn = k + stages;
        if (kn < K && lane == (kn & 31))
            bulk_copy(my_stage + s * SB, ((kn >> 5) == (k >> 5)) ? cur_src : nxt_src, bytes,
                      my_bars + s);
        phase ^= 1u << s;
        if (++s == stages) s = 0;
    }
    if (k < K) {
        // a wait ran out: wait (bounded) for every copy still in flight before
        // the CTA's shared memory is released
        const int last = min(K, k + stages);
        for (int j = k; j < last; ++j) {
            const int bj = j % stages;
            warp_wait(my_bars + bj, (phase >> bj) & 1u);
        }
        return false;
    }
    return true;
}

// At most 64 registers: the box records' loop needs about 54; the tile's
// summed-area records, rare, take what spills there are.
template <int NW, int NQ>
__global__ void __launch_bounds__(NW * 32, 32 / NW)
splat_box_bulk_kernel(const ScStepRec *__restrict__ recs, const int32_t *__restrict__ tile_start,
                      const int32_t *__restrict__ items, const float2 *__restrict__ sat,
                      SplatConsts c, int sat_tiles, int stages, int half_rows,
                      int64_t table_floats, float *__restrict__ ws, int32_t *status) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int BSR = kBulkBsr;
    constexpr int PAIRS = (NQ + 1) / 2, SB = (2 * PAIRS * NQ + 3) & ~3;  // stage buffer floats
    const int E = c.edge, EE = c.edge * c.edge;
    const int HB = half_rows * BSR + 16;  // odd half starts 16 banks after the even half
    const int BS = (2 * HB + 31) & ~31;
    const int SBS = (EE + 31) & ~31;  // summed-area buffers (E-stride), in the same space
    float *acc = reinterpret_cast<float *>(smem_raw);                   // [NW][BS]
    int4 *descs = reinterpret_cast<int4 *>(acc + NW * BS);              // [NW][2][32]
    float *stage = reinterpret_cast<float *>(descs + NW * 64);          // [NW][stages][SB]
    uint64_t *bars = reinterpret_cast<uint64_t *>(stage + NW * stages * SB);  // [NW][stages]
    int *bnd = reinterpret_cast<int *>(bars + NW * stages);  // [NW][2][E + 2] when sat_tiles
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tile = blockIdx.x;
    const int t = tile % c.tiles_per_image;
    const int x0 = (t / c.tiles_y) * c.tile, y0 = (t % c.tiles_y) * c.tile;
    for (int i = threadIdx.x; i < NW * BS; i += blockDim.x) acc[i] = 0.f;
    for (int i = threadIdx.x; i < NW * stages * SB; i += blockDim.x) stage[i] = 0.f;
    if (threadIdx.x < NW * stages) mbar_init(bars + threadIdx.x, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    __syncthreads();

    // buffer (r, c) is half (r + 1) & 1, entry ((r + 1) >> 1) * BSR + c + 1
    uint32_t phase = 0;
    bulk_tile_records<NW, NQ>(recs, tile_start, items, c, stages, HB, table_floats, tile, x0, y0,
                              acc + warp * BS, descs + warp * 64, stage + warp * stages * SB,
                              bars + warp * stages, phase, c.first_wait_tries, status);
    __syncthreads();
    float *out = ws + (size_t)tile * EE;
    for (int p = threadIdx.x; p < EE; p += blockDim.x) {
        const int r = p / E, cc = p - (p / E) * E;
        const int off = ((r + 1) & 1) * HB + ((r + 1) >> 1) * BSR + cc + 1;
        float sum = 0.f;
#pragma unroll
        for (int w = 0; w < NW; ++w) sum += acc[w * BS + off];
        out[p] = sum;
    }
    // the tile's summed-area records (bin sat_tiles + tile), added as
    // splat_sat_kernel adds them, with no launch of their own
    if (sat_tiles == 0) return;
    const int s0 = tile_start[sat_tiles + tile], s1 = tile_start[sat_tiles + tile + 1];
    if (s1 == s0) return;
    __syncthreads();
    for (int i = threadIdx.x; i < NW * SBS; i += blockDim.x) acc[i] = 0.f;
    __syncthreads();
    int *bx = bnd + warp * 2 * (E + 2);
    int *by = bx + (E + 2);
    for (int m = s0 + warp; m < s1; m += NW) {
        const ScStepRec &rec = recs[__ldg(items + m)];
        const int ni = rec.n_i - 1, nj = rec.n_j - 1;
        const int ox = rec.i_start - x0, oy = rec.j_start - y0;
        if (!in_buffer(ox, oy, ni, nj, E)) {
            if (lane == 0) sc::flag_status(status, 2, rec.i_start, rec.j_start, tile);
            continue;
        }
        splat_sat_record(rec, ox * E + oy, sat, c, bx, by, acc + warp * SBS, lane);
    }
    __syncthreads();
    for (int p = threadIdx.x; p < EE; p += blockDim.x) {
        float sum = 0.f;
#pragma unroll
        for (int w = 0; w < NW; ++w) sum += acc[w * SBS + p];
        out[p] = out[p] + sum;
    }
}

// Bulk-copy box launch for block size NQ; done stays false when the geometry
// does not fit it (the direct kernel then runs).
template <int NW, int NQ>
int launch_bulk(const ScStepRec *recs, const int32_t *tile_start, const int32_t *items,
                const float2 *sat, const SplatConsts &c, int n_tiles, int n_slots,
                int want_stages, float *ws, int32_t *status, cudaStream_t s, bool &done,
                bool &sat_done) {
    done = sat_done = false;
    constexpr int PAIRS = (NQ + 1) / 2, SB = (2 * PAIRS * NQ + 3) & ~3;
    constexpr int NB = SC_BOX_BLOCK_FLOATS(NQ);
    // buffer rows -1 .. tile + 2 PAIRS - 2 and columns -1 .. tile + 14 are reachable
    if (n_slots <= 0 || c.box_nq != NQ || c.tile + 15 > kBulkBsr || c.edge + 1 > kBulkBsr)
        return SC_OK;
    const int rows = max(c.edge, c.tile + 2 * PAIRS - 1) + 1;
    const int half_rows = ((rows + 1) / 2 + 3) & ~3;  // multiple of 4: halves 16 banks apart
    const int64_t table_floats = (int64_t)n_slots * c.box_p * c.box_p * NB;
    const int bs = (2 * (half_rows * kBulkBsr + 16) + 31) & ~31;
    // the summed-area records go in the same kernel when their E-stride
    // buffers fit the box buffers' space
    const bool fuse_sat = ((c.edge * c.edge + 31) & ~31) <= bs;
    const size_t fixed = (size_t)NW * bs * sizeof(float) + (size_t)NW * 64 * sizeof(int4) +
                         (fuse_sat ? (size_t)NW * 2 * (c.edge + 2) * sizeof(int) : 0);
    auto bulk_smem = [&](int st) {
        return fixed + (size_t)NW * st * SB * sizeof(float) + (size_t)NW * st * sizeof(uint64_t);
    };
    int stages = want_stages > 0 ? want_stages : 4;
    while (stages > 1 && bulk_smem(stages) > 160 * 1024) --stages;
    const size_t smem = bulk_smem(stages);
    if (smem > 160 * 1024) return SC_OK;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(splat_box_bulk_kernel<NW, NQ>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return sc::cuda_status(e, "sc_splat: smem attribute");
    }
    splat_box_bulk_kernel<NW, NQ><<<n_tiles, NW * 32, smem, s>>>(
        recs, tile_start, items, sat, c, fuse_sat ? n_tiles : 0, stages, half_rows, table_floats,
        ws, status);
    done = true;
    sat_done = fuse_sat;
    return sc::launch_status("sc_splat bulk-copy box");
}

// ------------------------------------------------ register-path box splat
// The same box-path records as splat_box_bulk_kernel, with the blocks moved
// by ordinary 16-byte loads: lane l holds the block's floats 4l .. 4l + 3 and,
// when there are more than 128, 128 + 4l .. 128 + 4l + 3.  Float f of the
// block (row f / NQ, column f % NQ) is added into the warp's tile buffer at a
// lane-constant offset from the record's corner; the buffer is row-major
// with row stride S (chosen on the host so that a warp's 32 adds touch each
// bank at most twice) and one margin row and column.  Each warp loads its
// next record's block before it adds the current one, and the SM's many
// resident warps (no staging buffers: about 3 KB of shared memory per warp)
// keep enough blocks in flight to cover the DRAM latency of random reads.
// Record m of the tile's box list goes to warp m mod NW, in list order, so a
// pixel's sums are formed in the same order as in the bulk-copy kernel.
template <int NQ>
struct RegRec {
    float4 a, b;  // the block's values this lane holds
    float w;
    int dd;       // (dr + 128) | (dc + 128) << 8
    int flags;    // bit 0 splat it, bit 1 the unconditional path applies
};

#ifndef SC_REG_WARPS_PER_SM
#define SC_REG_WARPS_PER_SM 32
#endif
template <int NW, int NQ>
__global__ void __launch_bounds__(NW * 32, SC_REG_WARPS_PER_SM / NW)
splat_box_reg_kernel(const ScStepRec *__restrict__ recs, const int32_t *__restrict__ tile_start,
                     const int32_t *__restrict__ items, SplatConsts c, int S, int rows,
                     int64_t table_floats, float *__restrict__ ws, int32_t *status) {
    extern __shared__ __align__(16) float smem_reg[];
    constexpr int NF = NQ * NQ;
    constexpr int NB = SC_BOX_BLOCK_FLOATS(NQ);
    constexpr int N1 = (NB - 128) / 4;  // lanes that hold a second float4
    static_assert(NB > 128 && NB <= 256 && NB % 4 == 0, "block of 129 .. 256 floats");
    const int E = c.edge, EE = c.edge * c.edge;
    const int BS = (rows * S + 31) & ~31;
    float *acc = smem_reg;  // [NW][BS]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tile = blockIdx.x;
    const int t = tile % c.tiles_per_image;
    const int x0 = (t / c.tiles_y) * c.tile, y0 = (t % c.tiles_y) * c.tile;
    for (int i = threadIdx.x; i < NW * BS; i += blockDim.x) acc[i] = 0.f;
    __syncthreads();
    float *my = acc + warp * BS;
    // offsets of this lane's floats from the record's corner; the padding
    // floats after NF (zero in the table) land in the margin rows below
    int off[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int f = (j < 4 ? 4 * lane + j : 128 + 4 * lane + j - 4);
        off[j] = (f / NQ) * S + f % NQ;
    }
    const int it0 = tile_start[tile], it1 = tile_start[tile + 1];
    const int K = it1 - it0 > warp ? (it1 - it0 - warp + NW - 1) / NW : 0;
    // lane l keeps the decoded descriptor of record 32 q + l of chunk q
    int chunk = -1;
    int4 my_desc = make_int4(0, 0, 0, 0);
    const float *my_src = c.box;
    auto fetch = [&](int k, RegRec<NQ> &r) {
        if ((k >> 5) != chunk) {
            chunk = k >> 5;
            const int kk = 32 * chunk + lane;
            my_desc = decode_record<NQ>(recs, items, it0 + warp + NW * kk, kk < K, x0, y0, c,
                                        table_floats, NB, my_src, status, tile);
        }
        const int src_lane = k & 31;
        r.w = __int_as_float(__shfl_sync(0xffffffffu, my_desc.x, src_lane));
        r.dd = __shfl_sync(0xffffffffu, my_desc.y, src_lane);
        r.flags = __shfl_sync(0xffffffffu, my_desc.w, src_lane);
        const uint64_t sp = __shfl_sync(0xffffffffu, (unsigned long long)(uintptr_t)my_src, src_lane);
        const float4 *src = reinterpret_cast<const float4 *>((uintptr_t)sp);
        r.a = make_float4(0.f, 0.f, 0.f, 0.f);
        r.b = r.a;
        if (r.flags & 1) {
            r.a = __ldg(src + lane);
            if (lane < N1) r.b = __ldg(src + 32 + lane);
        }
    };
    RegRec<NQ> cur, nxt;
    if (K > 0) fetch(0, cur);
    for (int k = 0; k < K; ++k) {
        if (k + 1 < K) fetch(k + 1, nxt);
        if (cur.flags & 1) {
            const int dr = (cur.dd & 0xff) - 128, dc = ((cur.dd >> 8) & 0xff) - 128;
            const float v[8] = {cur.a.x, cur.a.y, cur.a.z, cur.a.w, cur.b.x, cur.b.y, cur.b.z, cur.b.w};
            float *D = my + (dr + 1) * S + dc + 1;
            const int d0 = (int)(D - my);  // bounds-checked build: the warp's buffer
            if (cur.flags & 2) {
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (sc::in_range(d0 + off[j], BS, status, 6))
                        D[off[j]] = fmaf(cur.w, v[j], D[off[j]]);
                if (lane < N1) {
#pragma unroll
                    for (int j = 4; j < 8; ++j)
                        if (sc::in_range(d0 + off[j], BS, status, 6))
                            D[off[j]] = fmaf(cur.w, v[j], D[off[j]]);
                }
            } else {
                // clipped by the image's low edges: rows and columns from 0,
                // rows below the tile buffer's edge
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int f = (j < 4 ? 4 * lane + j : 128 + 4 * lane + j - 4);
                    const int r = dr + f / NQ, cc = dc + f % NQ;
                    if ((j < 4 || lane < N1) && f < NF && r >= 0 && r < E && cc >= 0 &&
                        sc::in_range(d0 + off[j], BS, status, 6))
                        D[off[j]] = fmaf(cur.w, v[j], D[off[j]]);
                }
            }
        }
        cur = nxt;
    }
    __syncthreads();
    float *out = ws + (size_t)tile * EE;
    for (int p = threadIdx.x; p < EE; p += blockDim.x) {
        const int r = p / E, cc = p - (p / E) * E;
        const int o = (r + 1) * S + cc + 1;
        float sum = 0.f;
#pragma unroll
        for (int w = 0; w < NW; ++w) sum += acc[w * BS + o];
        out[p] = sum;
    }
}

// Row stride of the register kernel's tile buffers: at least `min_s`, the
// smallest with the fewest shared-memory bank conflicts over the lanes' adds.
inline int reg_row_stride(int nq, int min_s) {
    const int nb = SC_BOX_BLOCK_FLOATS(nq);
    int best = min_s, best_cost = INT_MAX;
    for (int S = min_s; S < min_s + 48; ++S) {
        int cost = 0;
        for (int part = 0; part < 2; ++part)
            for (int j = 0; j < 4; ++j) {
                int count[32] = {0};
                int worst = 0;
                for (int l = 0; l < 32; ++l) {
                    const int f = part * 128 + 4 * l + j;
                    if (f >= nb) continue;
                    const int bank = ((f / nq) * S + f % nq) & 31;
                    worst = worst > ++count[bank] ? worst : count[bank];
                }
                cost += worst;
            }
        if (cost < best_cost) {
            best_cost = cost;
            best = S;
        }
    }
    return best;
}

template <int NW, int NQ>
int launch_reg(const ScStepRec *recs, const int32_t *tile_start, const int32_t *items,
               const SplatConsts &c, int n_tiles, int n_slots, float *ws, int32_t *status,
               cudaStream_t s, bool &done) {
    done = false;
    if (n_slots <= 0 || c.box_nq != NQ) return SC_OK;
    // buffer rows and columns -1 .. tile + NQ (the padding floats land at row NQ)
    const int span = max(c.edge, c.tile + NQ) + 2;
    const int S = reg_row_stride(NQ, span);
    const int rows = span + 1;
    const int64_t table_floats = (int64_t)n_slots * c.box_p * c.box_p * SC_BOX_BLOCK_FLOATS(NQ);
    const size_t smem = (size_t)NW * ((rows * S + 31) & ~31) * sizeof(float);
    if (smem > 160 * 1024) return SC_OK;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(splat_box_reg_kernel<NW, NQ>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return sc::cuda_status(e, "sc_splat: smem attribute");
    }
    splat_box_reg_kernel<NW, NQ><<<n_tiles, NW * 32, smem, s>>>(recs, tile_start, items, c, S, rows,
                                                                table_floats, ws, status);
    done = true;
    return sc::launch_status("sc_splat register box");
}

// Summed-area path: the tile's second bin.  Adds into the tile buffer the box
// kernel wrote (accumulate = 1) or writes it (accumulate = 0, no box tables).
template <int NW>
__global__ void __launch_bounds__(NW * 32)
splat_sat_kernel(const ScStepRec *__restrict__ recs, const int32_t *__restrict__ tile_start,
                 const int32_t *__restrict__ items, const float2 *__restrict__ sat,
                 SplatConsts c, int n_tiles, int accumulate, float *__restrict__ ws,
                 int32_t *status) {
    extern __shared__ float sm[];
    const int E = c.edge, EE = c.edge * c.edge;
    const int BS = (EE + 31) & ~31;
    const int tile = blockIdx.x;
    const int it0 = tile_start[n_tiles + tile], it1 = tile_start[n_tiles + tile + 1];
    float *out = ws + (size_t)tile * EE;
    if (it0 == it1) {
        if (!accumulate)
            for (int p = threadIdx.x; p < EE; p += blockDim.x) out[p] = 0.f;
        return;
    }
    float *acc = sm;
    int *bnd = reinterpret_cast<int *>(acc + NW * BS);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t = tile % c.tiles_per_image;
    const int x0 = (t / c.tiles_y) * c.tile, y0 = (t % c.tiles_y) * c.tile;
    for (int i = threadIdx.x; i < NW * BS; i += blockDim.x) sm[i] = 0.f;
    __syncthreads();
    float *my_acc = acc + warp * BS;
    int *bx = bnd + warp * 2 * (E + 2);
    int *by = bx + (E + 2);
    for (int m = it0 + warp; m < it1; m += NW) {
        const ScStepRec &rec = recs[__ldg(items + m)];
        const int ni = rec.n_i - 1, nj = rec.n_j - 1;
        const int ox = rec.i_start - x0, oy = rec.j_start - y0;
        if (!in_buffer(ox, oy, ni, nj, E)) {
            if (lane == 0) sc::flag_status(status, 2, rec.i_start, rec.j_start, tile);
            continue;
        }
        splat_sat_record(rec, ox * E + oy, sat, c, bx, by, my_acc, lane);
    }
    __syncthreads();
    for (int p = threadIdx.x; p < EE; p += blockDim.x) {
        float sum = 0.f;
#pragma unroll
        for (int w = 0; w < NW; ++w) sum += acc[w * BS + p];
        out[p] = accumulate ? out[p] + sum : sum;
    }
}

// FP64 splat (injected-draws parity mode): a warp per record, no bins.  The
// footprint bounds are axis_bound's (the reference's ceil decisions), each
// pixel's slice sum is the signed quadrant-table combination with every hi
// and lo term taken in FP64, and the pixel gets (sum * res^2) * norm by an
// FP64 atomic add when the sum is positive (_epifm.py:277-282).
__global__ void splat_fp64_kernel(const ScStepRec *__restrict__ recs,
                                  const double *__restrict__ norm, int n_rec,
                                  const float2 *__restrict__ sat, SplatConsts c, int n_images,
                                  int rec_per_image, int n_slots, int max_bounds,
                                  double *__restrict__ image, int32_t *status) {
    extern __shared__ int bnd64[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int *bx = bnd64 + warp * 2 * max_bounds;
    int *by = bx + max_bounds;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    const double unit_area = c.res * c.res;
    for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n_rec; r += warps) {
        const ScStepRec rec = recs[r];
        const double w = norm[r];
        if (rec.n_i < 2 || rec.n_j < 2 || rec.slot < 0 || !(w > 0.0)) continue;
        const int img = rec_per_image > 0 ? r / rec_per_image : 0;
        if (rec.n_i > max_bounds || rec.n_j > max_bounds || rec.slot >= n_slots ||
            img >= n_images || rec.i_start < 0 || rec.j_start < 0 ||
            rec.i_start + rec.n_i - 1 > c.nw || rec.j_start + rec.n_j - 1 > c.nh) {
            if (lane == 0) sc::flag_status(status, 2, r, rec.i_start, rec.j_start);
            continue;
        }
        for (int b = lane; b < rec.n_i + rec.n_j; b += 32) {
            if (b < rec.n_i)
                bx[b] = axis_bound(b, rec.n_i, rec.i_start, rec.ax_hi, rec.ax_lo, rec.x0, c);
            else
                by[b - rec.n_i] = axis_bound(b - rec.n_i, rec.n_j, rec.j_start, rec.ay_hi,
                                             rec.ay_lo, rec.y0, c);
        }
        __syncwarp();
        const float2 *G = sat + (int64_t)rec.slot * c.table_stride;
        const int ni = rec.n_i - 1, nj = rec.n_j - 1;
        double *out = image + (int64_t)img * c.nw * c.nh;
        for (int q = lane; q < ni * nj; q += 32) {
            const int a = q / nj, bj = q - (q / nj) * nj;
            int a0 = bx[a], a1 = bx[a + 1], b0 = by[bj], b1 = by[bj + 1];
            sc::slice_bounds(a0, a1, c.n_signal);
            sc::slice_bounds(b0, b1, c.n_signal);
            if (a1 <= a0 || b1 <= b0) continue;
            int uu[3], vv[3];
            float us[3], vs[3];
            const int nu = sc::fold(a0, a1, c.n_r, uu, us);
            const int nv = sc::fold(b0, b1, c.n_r, vv, vs);
            double sum = 0.0;
            for (int iu = 0; iu < nu; ++iu) {
                const float2 *row = G + (int64_t)uu[iu] * c.pitch;
                for (int iv = 0; iv < nv; ++iv) {
                    const float2 gv = __ldg(row + vv[iv]);
                    sum += (double)(us[iu] * vs[iv]) * ((double)gv.x + (double)gv.y);
                }
            }
            const double photons = sum * unit_area;
            if (photons > 0.0)
                atomicAdd(out + (int64_t)(rec.i_start + a) * c.nh + (rec.j_start + bj),
                          photons * w);
        }
        __syncwarp();
    }
}

// Per pixel: the tile buffers that cover it, summed in a fixed order.
__global__ void splat_merge_kernel(const float *__restrict__ ws, SplatConsts c, int n_images,
                                   float *__restrict__ image) {
    const int n = c.nw * c.nh;
    const int E = c.edge, EE = c.edge * c.edge;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < (int64_t)n * n_images;
         g += (int64_t)gridDim.x * blockDim.x) {
        const int img = (int)(g / n);
        const int p = (int)(g - (int64_t)img * n);
        const int i = p / c.nh, j = p - (p / c.nh) * c.nh;
        const int tx = i / c.tile, ty = j / c.tile;
        const float *tiles = ws + (size_t)img * c.tiles_per_image * EE;
        float sum = 0.f;
        for (int a = 0; a <= tx; ++a) {
            const int li = i - (tx - a) * c.tile;
            if (li >= E) break;
            for (int b = 0; b <= ty; ++b) {
                const int lj = j - (ty - b) * c.tile;
                if (lj >= E) break;
                sum += tiles[(size_t)((tx - a) * c.tiles_y + (ty - b)) * EE + li * E + lj];
            }
        }
        image[g] = sum;
    }
}

template <int NW>
int launch_splat(const ScStepRec *recs, const int32_t *tile_start, const int32_t *items,
                 const float2 *sat, const SplatConsts &c, int n_tiles, int n_slots, int stages,
                 int box_kernel, bool box, float *ws, int32_t *status, cudaStream_t s) {
    const int ee = c.edge * c.edge;
    const int bs = (ee + 31) & ~31;
    if (box && box_kernel == 1) {
        // register kernel for blocks of 12..16 rows
        bool done = false;
        int rc = SC_OK;
        switch (c.box_nq) {
            case 12: rc = launch_reg<NW, 12>(recs, tile_start, items, c, n_tiles, n_slots, ws, status, s, done); break;
            case 13: rc = launch_reg<NW, 13>(recs, tile_start, items, c, n_tiles, n_slots, ws, status, s, done); break;
            case 14: rc = launch_reg<NW, 14>(recs, tile_start, items, c, n_tiles, n_slots, ws, status, s, done); break;
            case 15: rc = launch_reg<NW, 15>(recs, tile_start, items, c, n_tiles, n_slots, ws, status, s, done); break;
            case 16: rc = launch_reg<NW, 16>(recs, tile_start, items, c, n_tiles, n_slots, ws, status, s, done); break;
            default: break;
        }
        if (rc) return rc;
        if (done) box = false;  // the summed-area pass below accumulates
    }
    if (box) {
        // bulk-copy kernel for blocks of 12..16 rows (pixels of 134..181 grid rows)
        bool done = false, sat_done = false;
        int rc = SC_OK;
        switch (c.box_nq) {
            case 12: rc = launch_bulk<NW, 12>(recs, tile_start, items, sat, c, n_tiles, n_slots, stages, ws, status, s, done, sat_done); break;
            case 13: rc = launch_bulk<NW, 13>(recs, tile_start, items, sat, c, n_tiles, n_slots, stages, ws, status, s, done, sat_done); break;
            case 14: rc = launch_bulk<NW, 14>(recs, tile_start, items, sat, c, n_tiles, n_slots, stages, ws, status, s, done, sat_done); break;
            case 15: rc = launch_bulk<NW, 15>(recs, tile_start, items, sat, c, n_tiles, n_slots, stages, ws, status, s, done, sat_done); break;
            case 16: rc = launch_bulk<NW, 16>(recs, tile_start, items, sat, c, n_tiles, n_slots, stages, ws, status, s, done, sat_done); break;
            default: break;
        }
        if (rc) return rc;
        if (sat_done) return SC_OK;  // the kernel added the summed-area records too
        if (done) box = false;       // the summed-area pass below accumulates
    }
    const bool staged = !box && c.box != nullptr;
    if (box) {
        const size_t smem = (size_t)NW * bs * sizeof(float) + (size_t)NW * 64 * sizeof(int4);
        SC_REQUIRE(smem <= 227 * 1024, "sc_splat: tile %d + halo %d needs %zu bytes of shared "
                   "memory with %d warps", c.tile, c.halo, smem, NW);
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(splat_box_kernel<NW>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return sc::cuda_status(e, "sc_splat: smem attribute");
        }
        splat_box_kernel<NW><<<n_tiles, NW * 32, smem, s>>>(recs, tile_start, items, c, ws, status);
        int rc = sc::launch_status("sc_splat box");
        if (rc) return rc;
    }
    const size_t smem = (size_t)NW * bs * sizeof(float) + (size_t)NW * 2 * (c.edge + 2) * sizeof(int);
    SC_REQUIRE(smem <= 227 * 1024, "sc_splat: tile %d + halo %d needs %zu bytes of shared memory "
               "with %d warps", c.tile, c.halo, smem, NW);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(splat_sat_kernel<NW>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return sc::cuda_status(e, "sc_splat: smem attribute");
    }
    splat_sat_kernel<NW><<<n_tiles, NW * 32, smem, s>>>(recs, tile_start, items, sat, c, n_tiles,
                                                        (box || staged) ? 1 : 0, ws, status);
    return sc::launch_status("sc_splat summed-area");
}

// ------------------------------------------------- persistent batched frame
struct BatchPlanDev {
    const int32_t *work, *tile_field_off, *tile_field, *field, *chunk;
    int32_t *counters;  // [0] next work entry, [1] stop, [2 + f] tiles done of field f
    int n_work, n_fields, n_chunks, chunk_pixels;
    uint32_t spin_limit;
    int target_extra, blocks_per_sm;
};

struct BatchCam {
    sc::cam::CamConsts c;
    const void *ptab;
    const float *offset_f, *inv_gain_f, *sigma;
    const double *table_value, *table_cdf;
    float *expect, *adc32;
};

__device__ __forceinline__ int ld_acquire(const int32_t *p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Canvas pixel (i, j): the tile buffers that cover it, summed in
// splat_merge_kernel's order (read through L2: they were written by other
// blocks of the same launch).
__device__ __forceinline__ float merge_pixel(const float *ws, const SplatConsts &c, int i, int j) {
    const int E = c.edge, EE = c.edge * c.edge;
    const int tx = i / c.tile, ty = j / c.tile;
    float sum = 0.f;
    for (int a = 0; a <= tx; ++a) {
        const int li = i - (tx - a) * c.tile;
        if (li >= E) break;
        for (int b = 0; b <= ty; ++b) {
            const int lj = j - (ty - b) * c.tile;
            if (lj >= E) break;
            sum += __ldcg(ws + (size_t)((tx - a) * c.tiles_y + (ty - b)) * EE + li * E + lj);
        }
    }
    return sum;
}

// The merge and the native camera in one pass: a thread takes a pixel pair,
// sums the tile buffers that cover each of its pixels in splat_merge_kernel's
// order, and draws the pair's camera as camera_native_kernel does, so the
// expectation and the ADC counts equal those of sc_splat (with its merge)
// followed by sc_camera, bit for bit, without the photon image's write and
// read and one launch.
// merge_pixel with at most MT covering tiles per axis, all loads issued
// together: a tile that does not cover the pixel adds +0, which leaves the
// sum as merge_pixel forms it, bit for bit (the buffers hold sums of
// non-negative terms, so the running sum is never -0).
template <int MT>
__device__ __forceinline__ float merge_pixel_mt(const float *ws, const SplatConsts &c, int i,
                                                int j, int32_t *status) {
    const int E = c.edge, EE = c.edge * c.edge;
    const int tx = i / c.tile, ty = j / c.tile;
    const int li0 = i - tx * c.tile, lj0 = j - ty * c.tile;
    float v[MT][MT];
#pragma unroll
    for (int a = 0; a < MT; ++a)
#pragma unroll
        for (int b = 0; b < MT; ++b) {
            const int li = li0 + a * c.tile, lj = lj0 + b * c.tile;
            const bool ok = a <= tx && li < E && b <= ty && lj < E;
            const int64_t o = (int64_t)((tx - a) * c.tiles_y + (ty - b)) * EE + li * E + lj;
            v[a][b] = ok && sc::in_range(o, (int64_t)c.tiles_per_image * EE, status, 3)
                          ? __ldcg(ws + o) : 0.f;
        }
    float sum = 0.f;
#pragma unroll
    for (int a = 0; a < MT; ++a)
#pragma unroll
        for (int b = 0; b < MT; ++b) sum += v[a][b];
    return sum;
}

template <int CAM, int MT>
__global__ void __launch_bounds__(256)
merge_camera_kernel(const float *__restrict__ ws, SplatConsts c, sc::cam::CamConsts cc,
                    const void *__restrict__ ptab, const float *__restrict__ offset_f,
                    const float *__restrict__ inv_gain_f, const float *__restrict__ sigma,
                    const double *__restrict__ table_value, const double *__restrict__ table_cdf,
                    float *__restrict__ expect, float *__restrict__ adc32, int32_t *status) {
    using namespace sc::cam;
    const PoisTab t = pois_tab(ptab);
    const uint64_t counter = cc.counter + (cc.frame ? (uint64_t)*cc.frame : 0);
    const uint32_t c0 = (uint32_t)counter, c1 = (uint32_t)(counter >> 32);
    const int n = cc.n, n_pairs = (n + 1) >> 1;
    const bool scmos = CAM == SC_CAM_SCMOS && sigma;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n_pairs;
         q += gridDim.x * blockDim.x) {
        const PairDraws d = pair_draws<CAM>(cc, q, c0, c1);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int p = 2 * q + h;
            if (p >= n) break;
            const int i = p / c.nh, j = p - (p / c.nh) * c.nh;
            const float ph = MT > 0 ? merge_pixel_mt<(MT > 0 ? MT : 1)>(ws, c, i, j, status)
                                    : merge_pixel(ws, c, i, j);
            const float e = cc.qe_f * (ph + cc.background_f);
            const float sg = scmos ? __ldg(sigma + p) : cc.readout_f;
            const float g = inv_gain_f ? __ldg(inv_gain_f + p) : cc.inv_gain0_f;
            const float o = offset_f ? __ldg(offset_f + p) : cc.offset0_f;
            const float v = pixel_adc<CAM>(cc, t, p, e, sg, g, o, d, h, c0, c1, table_value,
                                           table_cdf, status);
            if (expect) expect[p] = e;
            adc32[p] = v;
        }
    }
}

// Resident blocks take work entries in plan order from b.counters[0] until
// the list is done.  An entry is claimed only when the block is free to work
// on it (claiming the next one ahead would let a block hold a tile that other
// blocks' chunks wait for while it is busy, measured 4x slower).  Tile entry: the tile's box records through each warp's
// copy ring (the ring and its mbarriers live for the whole launch), the
// buffer written, then the tile's summed-area records added (both sums as
// splat_box_bulk_kernel and splat_sat_kernel form them), then the tile
// counters of the fields that read it advanced.  Chunk entry: thread 0 polls
// the field's counter (bounded; running out sets status bit 5 and stops the
// launch), then every thread merges, images and draws its pixels.
template <int NW, int NQ>
__global__ void __launch_bounds__(NW * 32, 20 / NW)
batch_frame_kernel(const ScStepRec *__restrict__ recs, const int32_t *__restrict__ tile_start,
                   const int32_t *__restrict__ items, const float2 *__restrict__ sat,
                   SplatConsts c, int n_tiles, int stages, int half_rows, int64_t table_floats,
                   float *__restrict__ ws, BatchPlanDev b, BatchCam bc, int32_t *status) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int sh_work, sh_stop;
    constexpr int BSR = kBulkBsr;
    constexpr int PAIRS = (NQ + 1) / 2, SB = (2 * PAIRS * NQ + 3) & ~3;
    const int E = c.edge, EE = c.edge * c.edge;
    const int HB = half_rows * BSR + 16;
    const int BS = (2 * HB + 31) & ~31;
    const int SBS = (EE + 31) & ~31;  // summed-area buffers (E-stride), in the same space
    float *acc = reinterpret_cast<float *>(smem_raw);                         // [NW][BS]
    int4 *descs = reinterpret_cast<int4 *>(acc + NW * BS);                    // [NW][2][32]
    float *stage = reinterpret_cast<float *>(descs + NW * 64);                // [NW][stages][SB]
    uint64_t *bars = reinterpret_cast<uint64_t *>(stage + NW * stages * SB);  // [NW][stages]
    int *bnd = reinterpret_cast<int *>(bars + NW * stages);                   // [NW][2][E + 2]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < NW * stages * SB; i += blockDim.x) stage[i] = 0.f;
    if (threadIdx.x < NW * stages) mbar_init(bars + threadIdx.x, 1);
    if (threadIdx.x == 0) sh_stop = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    __syncthreads();
    uint32_t phase = 0;
    for (;;) {
        if (threadIdx.x == 0) {
            int w = atomicAdd(b.counters, 1);
            if (w < b.n_work && ld_acquire(b.counters + 1)) w = b.n_work;  // stopped
            sh_work = w < b.n_work ? b.work[w] : INT_MIN;
        }
        __syncthreads();
        const int w = sh_work;
        __syncthreads();
        if (w == INT_MIN) break;
        if (w >= 0) {
            const int tile = w;
            const int t = tile % c.tiles_per_image;
            const int x0 = (t / c.tiles_y) * c.tile, y0 = (t % c.tiles_y) * c.tile;
            for (int i = threadIdx.x; i < NW * BS; i += blockDim.x) acc[i] = 0.f;
            __syncthreads();
            if (!bulk_tile_records<NW, NQ>(recs, tile_start, items, c, stages, HB, table_floats,
                                           tile, x0, y0, acc + warp * BS, descs + warp * 64,
                                           stage + warp * stages * SB, bars + warp * stages,
                                           phase, kWaitTries, status))
                sh_stop = 1;
            __syncthreads();
            float *out = ws + (size_t)tile * EE;
            for (int p = threadIdx.x; p < EE; p += blockDim.x) {
                const int r = p / E, cc = p - (p / E) * E;
                const int off = ((r + 1) & 1) * HB + ((r + 1) >> 1) * BSR + cc + 1;
                float sum = 0.f;
#pragma unroll
                for (int v = 0; v < NW; ++v) sum += acc[v * BS + off];
                out[p] = sum;
            }
            const int s0 = tile_start[n_tiles + tile], s1 = tile_start[n_tiles + tile + 1];
            if (s1 > s0 && !sh_stop) {
                __syncthreads();
                for (int i = threadIdx.x; i < NW * SBS; i += blockDim.x) acc[i] = 0.f;
                __syncthreads();
                int *bx = bnd + warp * 2 * (E + 2);
                int *by = bx + (E + 2);
                for (int m = s0 + warp; m < s1; m += NW) {
                    const ScStepRec &rec = recs[__ldg(items + m)];
                    const int ni = rec.n_i - 1, nj = rec.n_j - 1;
                    const int ox = rec.i_start - x0, oy = rec.j_start - y0;
                    if (!in_buffer(ox, oy, ni, nj, E)) {
                        if (lane == 0) sc::flag_status(status, 2, rec.i_start, rec.j_start, tile);
                        continue;
                    }
                    splat_sat_record(rec, ox * E + oy, sat, c, bx, by, acc + warp * SBS, lane);
                }
                __syncthreads();
                for (int p = threadIdx.x; p < EE; p += blockDim.x) {
                    float sum = 0.f;
#pragma unroll
                    for (int v = 0; v < NW; ++v) sum += acc[v * SBS + p];
                    out[p] = out[p] + sum;
                }
            }
            __threadfence();
            __syncthreads();
            if (sh_stop) {
                if (threadIdx.x == 0) atomicExch(b.counters + 1, 1);
                break;
            }
            if (threadIdx.x == 0)
                for (int q = b.tile_field_off[tile]; q < b.tile_field_off[tile + 1]; ++q)
                    atomicAdd(b.counters + 2 + b.tile_field[q], 1);
        } else {
            const int k = -w - 1;
            const int f = b.chunk[2 * k], first = b.chunk[2 * k + 1];
            const int i0 = b.field[4 * f], j0 = b.field[4 * f + 1], edge = b.field[4 * f + 2];
            if (threadIdx.x == 0) {
                const int target = b.field[4 * f + 3] + b.target_extra;
                uint32_t it = 0;
                bool ok = true;
                while (ld_acquire(b.counters + 2 + f) < target) {
                    if (++it > b.spin_limit) {
                        ok = false;
                        break;
                    }
                    __nanosleep(256);
                }
                if (!ok) {
                    sc::flag_status(status, 5, k, f, -1);
                    atomicExch(b.counters + 1, 1);
                }
                sh_stop = ok ? 0 : 1;
                __threadfence();
            }
            __syncthreads();
            if (sh_stop) break;
            // the merged photons of the chunk's pixels, into the expectation
            // buffer; batch_camera_kernel turns them into the expectation and
            // the ADC counts at full occupancy
            const int last = min(first + b.chunk_pixels, edge * edge);
            for (int q = first + threadIdx.x; q < last; q += blockDim.x) {
                const int li = q / edge;
                const int i = i0 + li, j = j0 + (q - li * edge);
                bc.expect[i * c.nh + j] = merge_pixel(ws, c, i, j);
            }
        }
    }
}

// The camera of the fields' pixels: a block per chunk, the photons the
// persistent kernel merged (in the expectation buffer) turned into the
// expectation and the ADC counts.
template <int CAM>
__global__ void __launch_bounds__(256)
batch_camera_kernel(BatchPlanDev b, BatchCam bc, int nh, int32_t *status) {
    if (*(volatile const int32_t *)(b.counters + 1)) return;  // the frame was stopped
    const sc::cam::PoisTab ptab = sc::cam::pois_tab(bc.ptab);
    const uint64_t counter = bc.c.counter + (bc.c.frame ? (uint64_t)*bc.c.frame : 0);
    for (int k = blockIdx.x; k < b.n_chunks; k += gridDim.x) {
        const int f = b.chunk[2 * k], first = b.chunk[2 * k + 1];
        const int i0 = b.field[4 * f], j0 = b.field[4 * f + 1], edge = b.field[4 * f + 2];
        const int last = min(first + b.chunk_pixels, edge * edge);
        for (int q = first + threadIdx.x; q < last; q += blockDim.x) {
            const int li = q / edge;
            const int p = (i0 + li) * nh + j0 + (q - li * edge);
            const float ef = bc.c.qe_f * (bc.expect[p] + bc.c.background_f);
            bc.expect[p] = ef;
            const float sg =
                (CAM == SC_CAM_SCMOS && bc.sigma) ? __ldg(bc.sigma + p) : bc.c.readout_f;
            const float g = bc.inv_gain_f ? __ldg(bc.inv_gain_f + p) : bc.c.inv_gain0_f;
            const float o = bc.offset_f ? __ldg(bc.offset_f + p) : bc.c.offset0_f;
            bc.adc32[p] = sc::cam::native_adc<CAM>(bc.c, ptab, p, ef, sg, g, o, counter,
                                                   bc.table_value, bc.table_cdf, status);
        }
    }
}

template <int NW, int NQ>
int launch_batch(const ScStepRec *recs, const int32_t *tile_start, const int32_t *items,
                 const float2 *sat, const SplatConsts &c, int n_tiles, int n_slots,
                 int want_stages, float *ws, const BatchPlanDev &b, const BatchCam &bc,
                 int32_t *status, cudaStream_t s) {
    constexpr int PAIRS = (NQ + 1) / 2, SB = (2 * PAIRS * NQ + 3) & ~3;
    constexpr int NB = SC_BOX_BLOCK_FLOATS(NQ);
    SC_REQUIRE(c.tile + 15 <= kBulkBsr && c.edge + 1 <= kBulkBsr,
               "sc_batch_frame: tile %d + halo %d does not fit the bulk-copy buffers", c.tile,
               c.halo);
    const int rows = max(c.edge, c.tile + 2 * PAIRS - 1) + 1;
    const int half_rows = ((rows + 1) / 2 + 3) & ~3;
    const int64_t table_floats = (int64_t)n_slots * c.box_p * c.box_p * NB;
    const size_t fixed = (size_t)NW * ((2 * (half_rows * kBulkBsr + 16) + 31) & ~31) * sizeof(float) +
                         (size_t)NW * 64 * sizeof(int4);
    auto smem_for = [&](int st) {
        return fixed + (size_t)NW * st * SB * sizeof(float) + (size_t)NW * st * sizeof(uint64_t) +
               (size_t)NW * 2 * (c.edge + 2) * sizeof(int);
    };
    int stages = want_stages > 0 ? want_stages : 4;
    while (stages > 1 && smem_for(stages) > 160 * 1024) --stages;
    const size_t smem = smem_for(stages);
    SC_REQUIRE(smem <= 160 * 1024, "sc_batch_frame: %zu bytes of shared memory", smem);
    cudaError_t e = cudaFuncSetAttribute(batch_frame_kernel<NW, NQ>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return sc::cuda_status(e, "sc_batch_frame: smem attribute");
    int grid = sc::resident_grid((const void *)batch_frame_kernel<NW, NQ>, NW * 32, smem,
                                 (int64_t)b.n_work);
    if (b.blocks_per_sm > 0) {
        int dev = 0, sms = 152;
        if (cudaGetDevice(&dev) == cudaSuccess)
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        grid = min(grid, max(1, sms * b.blocks_per_sm));
    }
    batch_frame_kernel<NW, NQ><<<grid, NW * 32, smem, s>>>(recs, tile_start, items, sat, c,
                                                           n_tiles, stages, half_rows,
                                                           table_floats, ws, b, bc, status);
    int rc = sc::launch_status("sc_batch_frame");
    if (rc || b.n_chunks == 0) return rc;
    switch (bc.c.camera) {
#define SC_BATCH_CAM(K)                                                                         \
    case K:                                                                                     \
        batch_camera_kernel<K><<<sc::resident_grid((const void *)batch_camera_kernel<K>, 256, 0, \
                                                   (int64_t)b.n_chunks),                        \
                                 256, 0, s>>>(b, bc, c.nh, status);                             \
        break;
        SC_BATCH_CAM(SC_CAM_EMCCD)
        SC_BATCH_CAM(SC_CAM_CCD)
        SC_BATCH_CAM(SC_CAM_CMOS_TABLE)
        SC_BATCH_CAM(SC_CAM_SCMOS)
#undef SC_BATCH_CAM
    }
    return sc::launch_status("sc_batch_frame camera");
}

int splat_consts(const ScSplatParams *p, const sc::TileGeom &g, SplatConsts &c) {
    SC_REQUIRE(p->n_r >= 2 && p->sat_pitch >= p->n_r + 1, "sc_splat: n_r=%d pitch=%d", p->n_r,
               p->sat_pitch);
    SC_REQUIRE(p->px > 0 && p->res > 0, "sc_splat: px and res must be positive");
    c.tiles_per_image = g.tiles_per_image;
    c.tiles_y = g.tiles_y;
    c.tile = g.tile;
    c.halo = g.halo;
    c.edge = g.edge;
    c.nw = g.nw;
    c.nh = g.nh;
    c.n_r = p->n_r;
    c.n_signal = 2 * p->n_r - 1;
    c.pitch = p->sat_pitch;
    c.table_stride = (int64_t)(p->n_r + 1) * p->sat_pitch;
    c.px = p->px;
    c.res = p->res;
    const double b = p->px / p->res;
    c.b_hi = (float)b;
    c.b_lo = (float)(b - (double)c.b_hi);
    c.box = nullptr;
    c.box_nq = 0;
    c.box_p = 0;
    c.box_floats = 0;
    c.first_wait_tries = p->first_wait_polls < 0 ? 0u
                         : p->first_wait_polls == 0 ? kWaitTries
                                                    : (uint32_t)p->first_wait_polls;
    return SC_OK;
}

}  // namespace

extern "C" int sc_splat_fp64(const ScStepRec *d_recs, const double *d_norm, int n_rec,
                             const float *d_sat, const ScSplatParams *p, double *d_image,
                             int32_t *d_status, void *stream) {
    SC_REQUIRE(p != nullptr, "sc_splat_fp64: params are NULL");
    SC_REQUIRE(p->nw > 0 && p->nh > 0 && p->n_images >= 1, "sc_splat_fp64: image %dx%d x %d",
               p->nw, p->nh, p->n_images);
    SC_REQUIRE(n_rec >= 0, "sc_splat_fp64: n_rec=%d", n_rec);
    SC_REQUIRE(p->n_slots >= 1, "sc_splat_fp64: n_slots=%d", p->n_slots);
    if (n_rec == 0) return SC_OK;
    SC_REQUIRE(d_recs && d_norm && d_sat && d_image, "sc_splat_fp64: NULL pointer");
    SC_REQUIRE(p->rec_per_image >= 0 &&
                   (p->rec_per_image == 0 || (int64_t)p->rec_per_image * p->n_images >= n_rec),
               "sc_splat_fp64: rec_per_image too small for n_rec");
    sc::TileGeom g;
    g.tile = 1;
    g.halo = 0;
    g.edge = 1;
    g.tiles_per_image = 1;
    g.tiles_y = 1;
    g.nw = p->nw;
    g.nh = p->nh;
    SplatConsts c;
    int rc = splat_consts(p, g, c);
    if (rc) return rc;
    // bounds per axis: the pixels a footprint spans (ceil(sw / px) + 1) and one more
    const int max_bounds = (int)ceil(p->res * (double)(c.n_signal - 1) / p->px) + 3;
    const int threads = 256;
    const size_t smem = (size_t)(threads / 32) * 2 * max_bounds * sizeof(int);
    SC_REQUIRE(smem <= 48 * 1024, "sc_splat_fp64: footprints of %d bounds are too wide",
               max_bounds);
    int64_t blocks = ((int64_t)n_rec * 32 + threads - 1) / threads;
    if (blocks > 152 * 16) blocks = 152 * 16;
    splat_fp64_kernel<<<(int)blocks, threads, smem, sc::as_stream(stream)>>>(
        d_recs, d_norm, n_rec, reinterpret_cast<const float2 *>(d_sat), c, p->n_images,
        p->rec_per_image, p->n_slots, max_bounds, d_image, d_status);
    return sc::launch_status("sc_splat_fp64");
}

extern "C" size_t sc_splat_workspace_bytes(const ScSplatParams *p) {
    sc::TileGeom g;
    if (!p || sc::tile_geom(p, g) != SC_OK) return 0;
    return (size_t)g.n_tiles * g.edge * g.edge * sizeof(float);
}

extern "C" int sc_splat(const ScStepRec *d_recs, const int32_t *d_tile_start,
                        const int32_t *d_items, const float *d_sat, const float *d_box,
                        const ScSplatParams *p, void *d_ws, size_t ws_bytes, float *d_image,
                        int32_t *d_status, void *stream) {
    sc::TileGeom g;
    int rc = sc::tile_geom(p, g);
    if (rc) return rc;
    SplatConsts c;
    rc = splat_consts(p, g, c);
    if (rc) return rc;
    SC_REQUIRE(d_tile_start && d_ws, "sc_splat: NULL pointer");
    SC_REQUIRE(p->box_stages >= 0 && p->box_stages <= 8, "sc_splat: box_stages=%d not in 0..8",
               p->box_stages);
    SC_REQUIRE(p->box_kernel == 0 || p->box_kernel == 1, "sc_splat: box_kernel=%d",
               p->box_kernel);
    SC_REQUIRE_CAP(ws_bytes >= sc_splat_workspace_bytes(p), "sc_splat: workspace %zu < %zu bytes",
               ws_bytes, sc_splat_workspace_bytes(p));
    if (d_box) {
        SC_REQUIRE(p->box_p >= 1 && p->box_nq == (c.n_signal + p->box_p - 1) / p->box_p + 1,
                   "sc_splat: box_p=%d / box_nq=%d inconsistent", p->box_p, p->box_nq);
        c.box = d_box;
        c.box_nq = p->box_nq;
        c.box_p = p->box_p;
        c.box_floats = (int64_t)p->n_slots * p->box_p * p->box_p *
                       (((int64_t)p->box_nq * p->box_nq + 3) & ~3LL);
    }
    const float2 *sat = reinterpret_cast<const float2 *>(d_sat);
    cudaStream_t s = sc::as_stream(stream);
    float *ws = static_cast<float *>(d_ws);
    const bool box = d_box != nullptr;
    switch (g.warps) {
        case 1: rc = launch_splat<1>(d_recs, d_tile_start, d_items, sat, c, g.n_tiles, p->n_slots, p->box_stages, p->box_kernel, box, ws, d_status, s); break;
        case 2: rc = launch_splat<2>(d_recs, d_tile_start, d_items, sat, c, g.n_tiles, p->n_slots, p->box_stages, p->box_kernel, box, ws, d_status, s); break;
        case 4: rc = launch_splat<4>(d_recs, d_tile_start, d_items, sat, c, g.n_tiles, p->n_slots, p->box_stages, p->box_kernel, box, ws, d_status, s); break;
        default: rc = launch_splat<8>(d_recs, d_tile_start, d_items, sat, c, g.n_tiles, p->n_slots, p->box_stages, p->box_kernel, box, ws, d_status, s); break;
    }
    if (rc) return rc;
    if (!d_image) return SC_OK;  // the caller merges (sc_merge_camera)
    const int64_t total = (int64_t)g.nw * g.nh * g.n_images;
    int grid = (int)((total + 255) / 256);
    if (grid > 152 * 32) grid = 152 * 32;
    splat_merge_kernel<<<grid, 256, 0, s>>>(ws, c, g.n_images, d_image);
    return sc::launch_status("sc_splat merge");
}

extern "C" int sc_merge_camera(const ScSplatParams *sp, const void *d_ws, size_t ws_bytes,
                               const ScCameraParams *cp, const float *d_offset_f,
                               const float *d_inv_gain_f, const float *d_sigma,
                               const double *d_table_value, const double *d_table_cdf,
                               float *d_expect, float *d_adc32, int32_t *d_status, void *stream) {
    sc::TileGeom g;
    int rc = sc::tile_geom(sp, g);
    if (rc) return rc;
    SplatConsts c;
    rc = splat_consts(sp, g, c);
    if (rc) return rc;
    SC_REQUIRE(cp != nullptr && d_ws && d_adc32, "sc_merge_camera: NULL pointer");
    SC_REQUIRE(g.n_images == 1, "sc_merge_camera: one image per call (got %d)", g.n_images);
    SC_REQUIRE(!cp->exact, "sc_merge_camera: native draws only");
    SC_REQUIRE(cp->nw == g.nw && cp->nh == g.nh, "sc_merge_camera: camera %dx%d, splat %dx%d",
               cp->nw, cp->nh, g.nw, g.nh);
    SC_REQUIRE(cp->camera >= SC_CAM_EMCCD && cp->camera <= SC_CAM_SCMOS,
               "sc_merge_camera: camera %d", cp->camera);
    SC_REQUIRE(cp->d_poisson_table != nullptr,
               "sc_merge_camera: native draws need the Poisson tables (sc_poisson_table)");
    if (cp->camera == SC_CAM_CMOS_TABLE)
        SC_REQUIRE(cp->table_n > 0 && d_table_value && d_table_cdf,
                   "sc_merge_camera: CMOS table mode needs the noise table");
    SC_REQUIRE_CAP(ws_bytes >= sc_splat_workspace_bytes(sp),
                   "sc_merge_camera: workspace %zu < %zu bytes", ws_bytes,
                   sc_splat_workspace_bytes(sp));
    sc::cam::CamConsts cc;
    rc = sc::cam::cam_consts(cp, cc);
    if (rc) return rc;
    cudaStream_t s = sc::as_stream(stream);
    const float *ws = static_cast<const float *>(d_ws);
    const int block = 256;
    const int64_t want = (((int64_t)cc.n + 1) / 2 + block - 1) / block;
    // covering tiles per axis: at most ceil(edge / tile)
    const int mt = (c.edge + c.tile - 1) / c.tile;
    const int sel = mt == 2 ? 2 : mt == 3 ? 3 : 0;
    switch (cc.camera * 4 + sel) {
#define SC_MC_LAUNCH(K, M)                                                                        \
    case K * 4 + M:                                                                               \
        merge_camera_kernel<K, M><<<sc::resident_grid((const void *)merge_camera_kernel<K, M>,      \
                                                      block, 0, want),                            \
                                    block, 0, s>>>(ws, c, cc, cp->d_poisson_table, d_offset_f,    \
                                                   d_inv_gain_f, d_sigma, d_table_value,          \
                                                   d_table_cdf, d_expect, d_adc32, d_status);     \
        break;
        SC_MC_LAUNCH(SC_CAM_EMCCD, 0)
        SC_MC_LAUNCH(SC_CAM_EMCCD, 2)
        SC_MC_LAUNCH(SC_CAM_EMCCD, 3)
        SC_MC_LAUNCH(SC_CAM_CCD, 0)
        SC_MC_LAUNCH(SC_CAM_CCD, 2)
        SC_MC_LAUNCH(SC_CAM_CCD, 3)
        SC_MC_LAUNCH(SC_CAM_CMOS_TABLE, 0)
        SC_MC_LAUNCH(SC_CAM_CMOS_TABLE, 2)
        SC_MC_LAUNCH(SC_CAM_CMOS_TABLE, 3)
        SC_MC_LAUNCH(SC_CAM_SCMOS, 0)
        SC_MC_LAUNCH(SC_CAM_SCMOS, 2)
        SC_MC_LAUNCH(SC_CAM_SCMOS, 3)
#undef SC_MC_LAUNCH
    }
    return sc::launch_status("sc_merge_camera");
}

extern "C" int sc_batch_frame(const ScStepRec *d_recs, const int32_t *d_tile_start,
                              const int32_t *d_items, const float *d_sat, const float *d_box,
                              const ScSplatParams *sp, const ScBatchPlan *plan,
                              const ScCameraParams *cp, const float *d_offset_f,
                              const float *d_inv_gain_f, const float *d_sigma,
                              const double *d_table_value, const double *d_table_cdf,
                              void *d_ws, size_t ws_bytes, float *d_expect, float *d_adc32,
                              int32_t *d_status, void *stream) {
    sc::TileGeom g;
    int rc = sc::tile_geom(sp, g);
    if (rc) return rc;
    SC_REQUIRE(g.n_images == 1, "sc_batch_frame: one canvas image per call");
    SplatConsts c;
    rc = splat_consts(sp, g, c);
    if (rc) return rc;
    SC_REQUIRE(plan && cp, "sc_batch_frame: NULL plan or camera params");
    SC_REQUIRE(d_tile_start && d_items && d_sat && d_box && d_adc32 && d_expect && d_ws,
               "sc_batch_frame: NULL pointer");
    SC_REQUIRE(plan->d_work && plan->d_tile_field_off && plan->d_field && plan->d_counters &&
                   plan->n_work >= 0 && plan->n_fields >= 1 && plan->chunk_pixels >= 1 &&
                   (plan->n_chunks == 0 || plan->d_chunk),
               "sc_batch_frame: incomplete plan");
    SC_REQUIRE(!cp->exact && cp->d_poisson_table, "sc_batch_frame: native camera draws only");
    SC_REQUIRE(cp->nw == sp->nw && cp->nh == sp->nh, "sc_batch_frame: camera %dx%d, canvas %dx%d",
               cp->nw, cp->nh, sp->nw, sp->nh);
    if (cp->camera == SC_CAM_CMOS_TABLE)
        SC_REQUIRE(cp->table_n > 0 && d_table_value && d_table_cdf,
                   "sc_batch_frame: CMOS table mode needs the noise table");
    SC_REQUIRE(sp->box_p >= 1 && sp->box_nq >= 12 && sp->box_nq <= 16,
               "sc_batch_frame: box tables with 12..16 offsets per axis (got %d)", sp->box_nq);
    SC_REQUIRE_CAP(ws_bytes >= sc_splat_workspace_bytes(sp), "sc_batch_frame: workspace %zu < %zu",
                   ws_bytes, sc_splat_workspace_bytes(sp));
    c.box = d_box;
    c.box_nq = sp->box_nq;
    c.box_p = sp->box_p;
    c.box_floats = (int64_t)sp->n_slots * sp->box_p * sp->box_p *
                   (((int64_t)sp->box_nq * sp->box_nq + 3) & ~3LL);
    BatchPlanDev b;
    b.work = plan->d_work;
    b.tile_field_off = plan->d_tile_field_off;
    b.tile_field = plan->d_tile_field;
    b.field = plan->d_field;
    b.chunk = plan->d_chunk;
    b.counters = plan->d_counters;
    b.n_work = plan->n_work;
    b.n_fields = plan->n_fields;
    b.n_chunks = plan->n_chunks;
    b.chunk_pixels = plan->chunk_pixels;
    b.spin_limit = plan->spin_limit > 0 ? (uint32_t)plan->spin_limit : (1u << 22);
    b.target_extra = plan->target_extra;
    b.blocks_per_sm = plan->blocks_per_sm;
    BatchCam bc;
    rc = sc::cam::cam_consts(cp, bc.c);
    if (rc) return rc;
    bc.ptab = cp->d_poisson_table;
    bc.offset_f = d_offset_f;
    bc.inv_gain_f = d_inv_gain_f;
    bc.sigma = d_sigma;
    bc.table_value = d_table_value;
    bc.table_cdf = d_table_cdf;
    bc.expect = d_expect;
    bc.adc32 = d_adc32;
    cudaStream_t s = sc::as_stream(stream);
    rc = sc::cuda_status(cudaMemsetAsync(plan->d_counters, 0,
                                         sizeof(int32_t) * (2 + (size_t)plan->n_fields), s),
                         "sc_batch_frame: counters");
    if (rc) return rc;
    if (plan->n_work == 0) return SC_OK;
    const float2 *sat = reinterpret_cast<const float2 *>(d_sat);
    float *ws = static_cast<float *>(d_ws);
#define SC_BATCH_NQ(NW)                                                                         \
    switch (c.box_nq) {                                                                         \
        case 12: return launch_batch<NW, 12>(d_recs, d_tile_start, d_items, sat, c, g.n_tiles,  \
                                             sp->n_slots, sp->box_stages, ws, b, bc, d_status, s); \
        case 13: return launch_batch<NW, 13>(d_recs, d_tile_start, d_items, sat, c, g.n_tiles,  \
                                             sp->n_slots, sp->box_stages, ws, b, bc, d_status, s); \
        case 14: return launch_batch<NW, 14>(d_recs, d_tile_start, d_items, sat, c, g.n_tiles,  \
                                             sp->n_slots, sp->box_stages, ws, b, bc, d_status, s); \
        case 15: return launch_batch<NW, 15>(d_recs, d_tile_start, d_items, sat, c, g.n_tiles,  \
                                             sp->n_slots, sp->box_stages, ws, b, bc, d_status, s); \
        default: return launch_batch<NW, 16>(d_recs, d_tile_start, d_items, sat, c, g.n_tiles, \
                                             sp->n_slots, sp->box_stages, ws, b, bc, d_status, s); \
    }
    switch (g.warps) {
        case 2: SC_BATCH_NQ(2)
        case 4: SC_BATCH_NQ(4)
        default: SC_BATCH_NQ(8)
    }
#undef SC_BATCH_NQ
}
