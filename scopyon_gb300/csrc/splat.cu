// Tile splat of emitter footprints onto the pixel grid.
//
// Reference: PointSpreadingFunction.overlay_signal_ (src/scopyon/_epifm.py:224-282).
// For each particle and sub-step it adds, to every pixel (i, j) of the
// footprint, norm * res^2 * sum(P[a0:a1, b0:b1]) where P is the 1-nm
// cartesian PSF grid and the bounds are ceil((i*px - x0) / res).
//
// Records are filed under the tile of their first pixel (bin.cu).  One CTA per
// tile sums the whole footprints of its records into a (tile + halo)^2 buffer
// in shared memory, one FP32 copy per warp, then stores the sum over warps in
// FP64 to the workspace; a merge pass adds, per pixel, the up to
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
#include "sc_common.cuh"
#include "bin.cuh"
#include "fold.cuh"

#ifndef SC_SPLAT_ROWS
#define SC_SPLAT_ROWS 8  // footprint rows per lane loaded in one round trip (2 rows per step)
#endif

namespace {

struct SplatConsts {
    int tiles_per_image, tiles_y, tile, halo, edge, nw, nh, n_r, n_signal, pitch;
    int64_t table_stride;  // float2 entries per quadrant table
    double px, res;
    float b_hi, b_lo;  // px / res as a double-float
    const float *box;  // box tables (NULL when px / res is not an integer)
    int box_nq;        // row stride of a box table block
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


// The first 32 bytes of a ScStepRec: everything the box path reads.
struct RecHead {
    int off_lo, off_hi, ij0, ij1, w_bits, slot, box;
};

__device__ __forceinline__ RecHead load_head(const ScStepRec *rec) {
    const int4 *p = reinterpret_cast<const int4 *>(rec);
    const int4 a = __ldg(p), b = __ldg(p + 1);
    RecHead h;
    h.off_lo = a.x;
    h.off_hi = a.y;
    h.ij0 = a.z;
    h.ij1 = a.w;
    h.w_bits = b.x;
    h.slot = b.y;
    h.box = b.z;
    return h;
}

__device__ __forceinline__ RecHead shfl_head(const RecHead &h, int src) {
    RecHead o;
    o.off_lo = __shfl_sync(0xffffffffu, h.off_lo, src);
    o.off_hi = __shfl_sync(0xffffffffu, h.off_hi, src);
    o.ij0 = __shfl_sync(0xffffffffu, h.ij0, src);
    o.ij1 = __shfl_sync(0xffffffffu, h.ij1, src);
    o.w_bits = __shfl_sync(0xffffffffu, h.w_bits, src);
    o.slot = __shfl_sync(0xffffffffu, h.slot, src);
    o.box = __shfl_sync(0xffffffffu, h.box, src);
    return o;
}

// One summed-area-path record over its whole footprint.  Kept out of line so
// that the box path, which most records take, keeps a small register footprint.
__device__ __noinline__ void splat_sat_record(const ScStepRec *rp, int i_start, int n_i,
                                              int j_start, int n_j, int slot, float w, int base,
                                              const float2 *__restrict__ sat, const SplatConsts &c,
                                              int *bx, int *by, float *my_acc, int lane) {
    const ScStepRec &rec = *rp;
    const double x0 = rec.x0, y0 = rec.y0;
    const float axh = rec.ax_hi, axl = rec.ax_lo, ayh = rec.ay_hi, ayl = rec.ay_lo;
    for (int b = lane; b < n_i + n_j; b += 32) {
        if (b < n_i) bx[b] = axis_bound(b, n_i, i_start, axh, axl, x0, c);
        else by[b - n_i] = axis_bound(b - n_i, n_j, j_start, ayh, ayl, y0, c);
    }
    __syncwarp();
    const float2 *G = sat + (int64_t)slot * c.table_stride;
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

// Box-path values of one record for this lane: rows row0 + 2u of column
// block cb (16 columns), all issued before any is used.
struct BoxVals {
    float v[SC_SPLAT_ROWS];
};

__device__ __forceinline__ void load_box(const float *B, int nq, int ni, int nj, int cb, int col,
                                         int row0, int a0, BoxVals &bv) {
    const int b = cb + col;
#pragma unroll
    for (int u = 0; u < SC_SPLAT_ROWS; ++u) {
        const int a = a0 + row0 + 2 * u;
        bv.v[u] = (a < ni && b < nj) ? __ldg(B + a * nq + b) : 0.f;
    }
}

// Per-warp partial sums are plain FP32: a warp adds at most a few dozen
// footprints to one pixel (error <~ 1e-6 relative), and the sums across warps
// and across tiles are FP64.
template <int NW>
__global__ void __launch_bounds__(NW * 32)
splat_halo_kernel(const ScStepRec *__restrict__ recs, const int32_t *__restrict__ tile_start,
                  const int32_t *__restrict__ items, const float2 *__restrict__ sat,
                  SplatConsts c, double *__restrict__ ws, int32_t *status) {
    extern __shared__ float sm[];
    const int E = c.edge, EE = c.edge * c.edge;
    float *acc = sm;
    int *bnd = reinterpret_cast<int *>(acc + NW * EE);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tile = blockIdx.x;
    const int t = tile % c.tiles_per_image;
    const int x0 = (t / c.tiles_y) * c.tile, y0 = (t % c.tiles_y) * c.tile;
    for (int i = threadIdx.x; i < NW * EE; i += blockDim.x) sm[i] = 0.f;
    __syncthreads();
    float *my_acc = acc + warp * EE;
    int *bx = bnd + warp * 2 * (E + 2);
    int *by = bx + (E + 2);
    const int col = lane & 15, row0 = lane >> 4;
    const int it0 = tile_start[tile], it1 = tile_start[tile + 1];
    for (int base = it0 + warp * 32; base < it1; base += NW * 32) {
        // 32 records per batch: item index and header loaded lane-parallel
        int my_item = 0;
        RecHead my_head = {0, 0, 0, 0, 0, -1, 0};
        if (base + lane < it1) {
            my_item = __ldg(items + base + lane);
            my_head = load_head(recs + my_item);
        }
        const int cnt = min(32, it1 - base);
        // software pipeline over the batch: the next box record's first rows
        // are in flight while the current one is accumulated
        BoxVals next;
        int next_k = -1;
        for (int k = 0; k < cnt; ++k) {
            const RecHead h = shfl_head(my_head, k);
            const int i_start = (int)(int16_t)(h.ij0 & 0xffff), n_i = h.ij0 >> 16;
            const int j_start = (int)(int16_t)(h.ij1 & 0xffff), n_j = h.ij1 >> 16;
            const int ni = n_i - 1, nj = n_j - 1;
            const int ox = i_start - x0, oy = j_start - y0;
            const bool ok = ni >= 1 && nj >= 1 && h.slot >= 0;
            if (ok && (ox < 0 || oy < 0 || ox + ni > E || oy + nj > E)) {
                if (lane == 0) sc::flag_status(status, 2, i_start, j_start, tile);
                continue;
            }
            if (!ok) continue;
            const float w = __int_as_float(h.w_bits);
            const int buf0 = ox * E + oy;
            if (h.box && c.box != nullptr) {
                // pixel (i_start + a, j_start + b) is entry box_off + a * NQ + b
                const float *B = c.box + (((int64_t)h.off_hi << 32) | (uint32_t)h.off_lo);
                BoxVals cur;
                if (next_k == k) cur = next;
                else load_box(B, c.box_nq, ni, nj, 0, col, row0, 0, cur);
                // prefetch the following record's first block when it is a box record
                next_k = -1;
                if (k + 1 < cnt) {
                    const RecHead hn = shfl_head(my_head, k + 1);
                    if (hn.box && hn.slot >= 0) {
                        const int nin = (hn.ij0 >> 16) - 1, njn = (hn.ij1 >> 16) - 1;
                        const float *Bn = c.box + (((int64_t)hn.off_hi << 32) | (uint32_t)hn.off_lo);
                        load_box(Bn, c.box_nq, nin, njn, 0, col, row0, 0, next);
                        next_k = k + 1;
                    }
                }
                for (int cb = 0; cb < nj; cb += 16) {
                    for (int a0 = 0; a0 < ni; a0 += 2 * SC_SPLAT_ROWS) {
                        if (cb > 0 || a0 > 0) load_box(B, c.box_nq, ni, nj, cb, col, row0, a0, cur);
                        const int b = cb + col;
#pragma unroll
                        for (int u = 0; u < SC_SPLAT_ROWS; ++u) {
                            const int a = a0 + row0 + 2 * u;
                            if (a < ni && b < nj && cur.v[u] > 0.f)
                                my_acc[buf0 + a * E + b] += w * cur.v[u];
                        }
                    }
                }
                continue;
            }
            splat_sat_record(recs + __shfl_sync(0xffffffffu, my_item, k), i_start, n_i, j_start,
                             n_j, h.slot, w, buf0, sat, c, bx, by, my_acc, lane);
        }
    }
    __syncthreads();
    double *out = ws + (size_t)tile * EE;
    for (int p = threadIdx.x; p < EE; p += blockDim.x) {
        double sum = 0.0;
#pragma unroll
        for (int w = 0; w < NW; ++w) sum += (double)acc[w * EE + p];
        out[p] = sum;
    }
}

// Per pixel: the tile buffers that cover it, summed in a fixed order.
__global__ void splat_merge_kernel(const double *__restrict__ ws, SplatConsts c, int n_images,
                                   float *__restrict__ image) {
    const int n = c.nw * c.nh;
    const int E = c.edge, EE = c.edge * c.edge;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < (int64_t)n * n_images;
         g += (int64_t)gridDim.x * blockDim.x) {
        const int img = (int)(g / n);
        const int p = (int)(g - (int64_t)img * n);
        const int i = p / c.nh, j = p - (p / c.nh) * c.nh;
        const int tx = i / c.tile, ty = j / c.tile;
        const double *tiles = ws + (size_t)img * c.tiles_per_image * EE;
        double sum = 0.0;
        for (int a = 0; a <= tx; ++a) {
            const int li = i - (tx - a) * c.tile;
            if (li >= E) break;
            for (int b = 0; b <= ty; ++b) {
                const int lj = j - (ty - b) * c.tile;
                if (lj >= E) break;
                sum += tiles[(size_t)((tx - a) * c.tiles_y + (ty - b)) * EE + li * E + lj];
            }
        }
        image[g] = (float)sum;
    }
}

template <int NW>
int launch_halo(const ScStepRec *recs, const int32_t *tile_start, const int32_t *items,
                const float2 *sat, const SplatConsts &c, int n_tiles, double *ws, int32_t *status,
                cudaStream_t s) {
    const size_t smem = (size_t)NW * c.edge * c.edge * sizeof(float) +
                        (size_t)NW * 2 * (c.edge + 2) * sizeof(int);
    SC_REQUIRE(smem <= 227 * 1024, "sc_splat: tile %d + halo %d needs %zu bytes of shared memory "
               "with %d warps", c.tile, c.halo, smem, NW);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(splat_halo_kernel<NW>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return sc::cuda_status(e, "sc_splat: smem attribute");
    }
    splat_halo_kernel<NW><<<n_tiles, NW * 32, smem, s>>>(recs, tile_start, items, sat, c, ws,
                                                         status);
    return sc::launch_status("sc_splat");
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
    return SC_OK;
}

}  // namespace

extern "C" size_t sc_splat_workspace_bytes(const ScSplatParams *p) {
    sc::TileGeom g;
    if (!p || sc::tile_geom(p, g) != SC_OK) return 0;
    return (size_t)g.n_tiles * g.edge * g.edge * sizeof(double);
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
    SC_REQUIRE(d_tile_start && d_image && d_ws, "sc_splat: NULL pointer");
    SC_REQUIRE(ws_bytes >= sc_splat_workspace_bytes(p), "sc_splat: workspace %zu < %zu bytes",
               ws_bytes, sc_splat_workspace_bytes(p));
    if (d_box) {
        SC_REQUIRE(p->box_p >= 1 && p->box_nq == (c.n_signal + p->box_p - 1) / p->box_p + 1,
                   "sc_splat: box_p=%d / box_nq=%d inconsistent", p->box_p, p->box_nq);
        c.box = d_box;
        c.box_nq = p->box_nq;
    }
    const float2 *sat = reinterpret_cast<const float2 *>(d_sat);
    cudaStream_t s = sc::as_stream(stream);
    double *ws = static_cast<double *>(d_ws);
    switch (g.warps) {
        case 1: rc = launch_halo<1>(d_recs, d_tile_start, d_items, sat, c, g.n_tiles, ws, d_status, s); break;
        case 2: rc = launch_halo<2>(d_recs, d_tile_start, d_items, sat, c, g.n_tiles, ws, d_status, s); break;
        case 4: rc = launch_halo<4>(d_recs, d_tile_start, d_items, sat, c, g.n_tiles, ws, d_status, s); break;
        default: rc = launch_halo<8>(d_recs, d_tile_start, d_items, sat, c, g.n_tiles, ws, d_status, s); break;
    }
    if (rc) return rc;
    const int64_t total = (int64_t)g.nw * g.nh * g.n_images;
    int grid = (int)((total + 255) / 256);
    if (grid > 152 * 32) grid = 152 * 32;
    splat_merge_kernel<<<grid, 256, 0, s>>>(ws, c, g.n_images, d_image);
    return sc::launch_status("sc_splat merge");
}
