// Tile splat of emitter footprints onto the pixel grid.
//
// Reference: PointSpreadingFunction.overlay_signal_ (src/scopyon/_epifm.py:224-282).
// For each particle and sub-step it adds, to every pixel (i, j) of the
// footprint, norm * res^2 * sum(P[a0:a1, b0:b1]) where P is the 1-nm
// cartesian PSF grid and the bounds are ceil((i*px - x0) / res).
//
// Here one CTA owns one output tile and its list of records (bin.cu).  Each
// warp takes a record, recomputes the footprint bounds that fall in the tile
// (an FP32 double-float estimate, with the reference's FP64 expression
// evaluated exactly whenever the estimate is within 1e-6 of an integer), and
// evaluates each pixel's rectangle sum from the quadrant summed-area table of
// the record's depth key: P is mirror-symmetric, so a rectangle [a0,a1) x
// [b0,b1) folds onto at most 3 x 3 quadrant-table entries per axis pair.
// The table holds double-float pairs, so the differences keep ~2^-48
// relative precision without FP64 arithmetic.  Each warp accumulates into its
// own shared-memory copy of the tile with Kahan compensation; the copies are
// summed in a fixed order at the end, so there are no atomics at all.
#include "sc_common.cuh"
#include "bin.cuh"
#include "fold.cuh"

namespace {

struct SplatConsts {
    int tiles_per_image, tiles_y, nw, nh, n_r, n_signal;
    int64_t table_stride;  // float2 entries per quadrant table
    int pitch;
    double px, res;
    float b_hi, b_lo;  // px / res as a double-float
    const float *box;  // box tables (NULL when px / res is not an integer)
    int box_p, box_nq;
    int64_t box_stride;  // floats per box table
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

template <int T, int NW>
__global__ void __launch_bounds__(NW * 32)
splat_tile_kernel(const ScStepRec *__restrict__ recs, const int32_t *__restrict__ tile_start,
                  const int32_t *__restrict__ items, const float2 *__restrict__ sat,
                  SplatConsts c, float *__restrict__ image) {
    extern __shared__ float sm[];
    float *acc = sm;
    float *cmp = acc + NW * T * T;
    int *bnd = reinterpret_cast<int *>(cmp + NW * T * T);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tile = blockIdx.x;
    const int img = tile / c.tiles_per_image;
    const int t = tile - img * c.tiles_per_image;
    const int tx = t / c.tiles_y, ty = t - (t / c.tiles_y) * c.tiles_y;
    const int px0 = tx * T, py0 = ty * T;
    for (int i = threadIdx.x; i < 2 * NW * T * T; i += blockDim.x) sm[i] = 0.f;
    __syncthreads();
    float *my_acc = acc + warp * T * T;
    float *my_cmp = cmp + warp * T * T;
    int *bx = bnd + warp * 2 * (T + 1);
    int *by = bx + (T + 1);
    const int it1 = tile_start[tile + 1];
    for (int it = tile_start[tile] + warp; it < it1; it += NW) {
        const ScStepRec rec = recs[items[it]];
        const int pi_lo = max((int)rec.i_start, px0);
        const int pi_hi = min(min(rec.i_start + rec.n_i - 2, px0 + T - 1), c.nw - 1);
        const int pj_lo = max((int)rec.j_start, py0);
        const int pj_hi = min(min(rec.j_start + rec.n_j - 2, py0 + T - 1), c.nh - 1);
        if (pi_hi < pi_lo || pj_hi < pj_lo) continue;
        if (rec.box && c.box != nullptr) {
            // pixel (i, j) integrates grid rows [l0x + P (i - i_start), + P) and the
            // same for columns: one entry of the box table, contiguous along j
            const int P = c.box_p, NQ = c.box_nq;
            const int mx = rec.l0x + P, my = rec.l0y + P;
            const int qx0 = mx / P + (pi_lo - rec.i_start);
            const int qy0 = my / P + (pj_lo - rec.j_start);
            const float *B = c.box + (int64_t)rec.slot * c.box_stride +
                             (int64_t)((mx % P) * P + (my % P)) * NQ * NQ;
            const int npy = pj_hi - pj_lo + 1;
            const int npix = (pi_hi - pi_lo + 1) * npy;
            for (int q = lane; q < npix; q += 32) {
                const int a = q / npy, bj = q - (q / npy) * npy;
                const int qx = qx0 + a, qy = qy0 + bj;
                if (qx >= NQ || qy >= NQ) continue;
                const float val = __ldg(B + qx * NQ + qy);
                if (val > 0.f) {
                    const float f = rec.w * val;
                    const int idx = (pi_lo + a - px0) * T + (pj_lo + bj - py0);
                    const float y = f - my_cmp[idx];
                    const float tsum = my_acc[idx] + y;
                    my_cmp[idx] = (tsum - my_acc[idx]) - y;
                    my_acc[idx] = tsum;
                }
            }
            continue;
        }
        const int nbx = pi_hi - pi_lo + 2, nby = pj_hi - pj_lo + 2;
        for (int b = lane; b < nbx + nby; b += 32) {
            if (b < nbx)
                bx[b] = axis_bound(pi_lo - rec.i_start + b, rec.n_i, rec.i_start, rec.ax_hi,
                                   rec.ax_lo, rec.x0, c);
            else
                by[b - nbx] = axis_bound(pj_lo - rec.j_start + (b - nbx), rec.n_j, rec.j_start,
                                         rec.ay_hi, rec.ay_lo, rec.y0, c);
        }
        __syncwarp();
        const float2 *G = sat + (int64_t)rec.slot * c.table_stride;
        const int npy = nby - 1;
        const int npix = (nbx - 1) * npy;
        for (int q = lane; q < npix; q += 32) {
            const int a = q / npy, bj = q - (q / npy) * npy;
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
            if (val > 0.f) {
                const float f = rec.w * val;
                const int idx = (pi_lo + a - px0) * T + (pj_lo + bj - py0);
                const float y = f - my_cmp[idx];
                const float tsum = my_acc[idx] + y;
                my_cmp[idx] = (tsum - my_acc[idx]) - y;
                my_acc[idx] = tsum;
            }
        }
        __syncwarp();
    }
    __syncthreads();
    float *out = image + (size_t)img * c.nw * c.nh;
    for (int p = threadIdx.x; p < T * T; p += blockDim.x) {
        const int gi = px0 + p / T, gj = py0 + (p - (p / T) * T);
        if (gi >= c.nw || gj >= c.nh) continue;
        double sum = 0.0;
#pragma unroll
        for (int w = 0; w < NW; ++w) sum += (double)acc[w * T * T + p] - (double)cmp[w * T * T + p];
        out[(size_t)gi * c.nh + gj] = (float)sum;
    }
}

template <int T, int NW>
int launch_splat(const ScStepRec *recs, const int32_t *tile_start, const int32_t *items,
                 const float2 *sat, const SplatConsts &c, int n_tiles, float *image,
                 cudaStream_t s) {
    const size_t smem = (size_t)2 * NW * T * T * sizeof(float) + (size_t)NW * 2 * (T + 1) * sizeof(int);
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(splat_tile_kernel<T, NW>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return sc::cuda_status(e, "sc_splat: smem attribute");
        attr = true;
    }
    splat_tile_kernel<T, NW><<<n_tiles, NW * 32, smem, s>>>(recs, tile_start, items, sat, c, image);
    return sc::launch_status("sc_splat");
}

}  // namespace

extern "C" int sc_splat(const ScStepRec *d_recs, const int32_t *d_tile_start,
                        const int32_t *d_items, const float *d_sat, const float *d_box,
                        const ScSplatParams *p, float *d_image, int32_t *d_status,
                        void *stream) {
    (void)d_status;
    sc::TileGeom g;
    int rc = sc::tile_geom(p, g);
    if (rc) return rc;
    SC_REQUIRE(p->n_r >= 2 && p->sat_pitch >= p->n_r + 1, "sc_splat: n_r=%d pitch=%d", p->n_r,
               p->sat_pitch);
    SC_REQUIRE(d_tile_start && d_image, "sc_splat: NULL pointer");
    SC_REQUIRE(p->px > 0 && p->res > 0, "sc_splat: px and res must be positive");
    SplatConsts c;
    c.tiles_per_image = g.tiles_per_image;
    c.tiles_y = g.tiles_y;
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
    c.box = d_box;
    c.box_p = p->box_p;
    c.box_nq = p->box_nq;
    c.box_stride = (int64_t)p->box_p * p->box_p * p->box_nq * p->box_nq;
    if (d_box) {
        SC_REQUIRE(p->box_p >= 1 && p->box_nq == (c.n_signal + p->box_p - 1) / p->box_p + 1,
                   "sc_splat: box_p=%d / box_nq=%d inconsistent", p->box_p, p->box_nq);
    }
    const float2 *sat = reinterpret_cast<const float2 *>(d_sat);
    cudaStream_t s = sc::as_stream(stream);
    switch (g.tile) {
        case 16: return launch_splat<16, 8>(d_recs, d_tile_start, d_items, sat, c, g.n_tiles, d_image, s);
        case 32: return launch_splat<32, 8>(d_recs, d_tile_start, d_items, sat, c, g.n_tiles, d_image, s);
        case 64: return launch_splat<64, 4>(d_recs, d_tile_start, d_items, sat, c, g.n_tiles, d_image, s);
        default:
            sc::set_error("sc_splat: tile %d not compiled (use 16, 32 or 64)", g.tile);
            return SC_ERR_ARG;
    }
}
