// Deterministic counting sort of splat records by output tile.
//
// The reference adds each particle's footprint straight into the image
// (src/scopyon/_epifm.py:1262-1264, :277-282).  Here the image is cut into
// square tiles; every tile gets the list of records whose footprint touches
// it, so the splat can give each tile to one CTA and accumulate it in shared
// memory with no global atomics.  The list order depends only on the input
// (chunk, then 32-record group, then tile slot, then lane), never on
// scheduling, so repeated runs add contributions in the same order.
#include "sc_common.cuh"
#include "bin.cuh"

namespace {

__global__ void bin_count_kernel(const ScStepRec *recs, int n_rec, sc::TileGeom g, int chunk,
                                 int32_t *counts) {
    extern __shared__ int32_t hist[];
    for (int t = threadIdx.x; t < g.n_tiles; t += blockDim.x) hist[t] = 0;
    __syncthreads();
    const int r0 = blockIdx.x * chunk;
    const int r1 = min(n_rec, r0 + chunk);
    for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        sc::TileRange tr;
        if (!sc::record_tiles(recs[r], r, g, tr)) continue;
        for (int tx = tr.tx0; tx <= tr.tx1; ++tx)
            for (int ty = tr.ty0; ty <= tr.ty1; ++ty) atomicAdd(&hist[tr.base + tx * g.tiles_y + ty], 1);
    }
    __syncthreads();
    int32_t *out = counts + (size_t)blockIdx.x * g.n_tiles;
    for (int t = threadIdx.x; t < g.n_tiles; t += blockDim.x) out[t] = hist[t];
}

// counts[c][t] -> exclusive offset of chunk c inside tile t; totals per tile.
__global__ void bin_chunk_offsets_kernel(int32_t *counts, int n_chunks, int n_tiles,
                                         int32_t *tile_total) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_tiles) return;
    int32_t run = 0;
    for (int c = 0; c < n_chunks; ++c) {
        int32_t *p = counts + (size_t)c * n_tiles + t;
        const int32_t v = *p;
        *p = run;
        run += v;
    }
    tile_total[t] = run;
}

// Single-CTA exclusive scan of per-tile totals -> tile_start[0..n_tiles].
__global__ void bin_tile_scan_kernel(const int32_t *tile_total, int n_tiles, int64_t capacity,
                                     int32_t *tile_start, int32_t *status) {
    __shared__ int32_t warp_tot[32];
    __shared__ int32_t carry_s;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry_s = 0;
    __syncthreads();
    for (int base = 0; base < n_tiles; base += blockDim.x) {
        const int t = base + threadIdx.x;
        int32_t v = t < n_tiles ? tile_total[t] : 0;
        int32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int32_t n = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += n;
        }
        if (lane == 31) warp_tot[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int32_t w = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int32_t n = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += n;
            }
            warp_tot[lane] = w;
        }
        __syncthreads();
        const int32_t carry = carry_s;
        const int32_t incl = x + (warp > 0 ? warp_tot[warp - 1] : 0) + carry;
        // clamped so that a consumer never reads item slots past the buffer
        if (t < n_tiles) tile_start[t] = (int32_t)min((int64_t)(incl - v), capacity);
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry_s = incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        tile_start[n_tiles] = (int32_t)min((int64_t)carry_s, capacity);
        if ((int64_t)carry_s > capacity) sc::flag_status(status, 4, carry_s, 0, 0);
    }
}

__global__ void bin_scatter_kernel(const ScStepRec *recs, int n_rec, sc::TileGeom g, int chunk,
                                   const int32_t *chunk_off, const int32_t *tile_start,
                                   int32_t *items, int64_t capacity) {
    extern __shared__ int32_t cursor[];
    const int lane = threadIdx.x;
    const int32_t *off = chunk_off + (size_t)blockIdx.x * g.n_tiles;
    for (int t = lane; t < g.n_tiles; t += 32) cursor[t] = tile_start[t] + off[t];
    __syncwarp();
    const int r0 = blockIdx.x * chunk;
    const int r1 = min(n_rec, r0 + chunk);
    for (int base = r0; base < r1; base += 32) {
        const int r = base + lane;
        sc::TileRange tr;
        bool any = r < r1 && sc::record_tiles(recs[r], r, g, tr);
        int ntx = any ? tr.tx1 - tr.tx0 + 1 : 0;
        int nty = any ? tr.ty1 - tr.ty0 + 1 : 0;
        const int mine = ntx * nty;
        const int rounds = __reduce_max_sync(0xffffffffu, mine);
        for (int k = 0; k < rounds; ++k) {
            const int tile = k < mine ? tr.base + (tr.tx0 + k / nty) * g.tiles_y + (tr.ty0 + k % nty)
                                      : -1;
            const unsigned peers = __match_any_sync(0xffffffffu, tile);
            const int rank = __popc(peers & ((1u << lane) - 1u));
            int32_t pos = 0;
            if (tile >= 0) pos = cursor[tile] + rank;
            __syncwarp();
            if (tile >= 0 && rank == 0) cursor[tile] += __popc(peers);
            if (tile >= 0 && (int64_t)pos < capacity) items[pos] = r;
            __syncwarp();
        }
    }
}

}  // namespace

namespace sc {

int tile_geom(const ScSplatParams *p, TileGeom &g) {
    SC_REQUIRE(p != nullptr, "splat params are NULL");
    SC_REQUIRE(p->tile >= 8 && p->tile <= 64 && p->tile % 8 == 0,
               "tile=%d must be a multiple of 8 in [8, 64]", p->tile);
    SC_REQUIRE(p->nw > 0 && p->nh > 0, "image size %dx%d", p->nw, p->nh);
    SC_REQUIRE(p->tiles_x == (p->nw + p->tile - 1) / p->tile &&
                   p->tiles_y == (p->nh + p->tile - 1) / p->tile,
               "tiles_x/tiles_y inconsistent with image and tile size");
    SC_REQUIRE(p->n_images >= 1, "n_images=%d", p->n_images);
    g.tile = p->tile;
    g.tiles_x = p->tiles_x;
    g.tiles_y = p->tiles_y;
    g.tiles_per_image = p->tiles_x * p->tiles_y;
    g.n_tiles = g.tiles_per_image * p->n_images;
    g.nw = p->nw;
    g.nh = p->nh;
    g.rec_per_image = p->rec_per_image;
    SC_REQUIRE((size_t)g.n_tiles * 4 <= 200 * 1024, "too many tiles (%d) in one launch", g.n_tiles);
    return SC_OK;
}

int bin_chunk(int n_rec, int n_tiles) {
    int chunk = 2048;
    while ((int64_t)((n_rec + chunk - 1) / chunk) * n_tiles > (8 << 20)) chunk *= 2;
    return chunk;
}

}  // namespace sc

extern "C" size_t sc_bin_workspace_bytes(int n_rec, int n_tiles_total) {
    if (n_rec <= 0 || n_tiles_total <= 0) return 0;
    const int chunk = sc::bin_chunk(n_rec, n_tiles_total);
    const size_t n_chunks = (size_t)(n_rec + chunk - 1) / chunk;
    return (n_chunks * n_tiles_total + n_tiles_total) * sizeof(int32_t);
}

extern "C" int64_t sc_bin_capacity(int n_rec, double px, double res, int n_signal, int tile) {
    if (n_rec <= 0 || px <= 0 || tile <= 0) return 0;
    // footprint spans at most ceil(width / px) + 1 pixels per axis
    const double width = res * (double)(n_signal - 1);
    const int64_t span = (int64_t)ceil(width / px) + 2;
    const int64_t tiles = (span + tile - 1) / tile + 1;
    return (int64_t)n_rec * tiles * tiles;
}

extern "C" int sc_bin_steps(const ScStepRec *d_recs, int n_rec, const ScSplatParams *p,
                            void *d_ws, size_t ws_bytes, int32_t *d_tile_start, int32_t *d_items,
                            int64_t capacity, int32_t *d_status, void *stream) {
    sc::TileGeom g;
    int rc = sc::tile_geom(p, g);
    if (rc) return rc;
    SC_REQUIRE(n_rec >= 0, "n_rec=%d", n_rec);
    SC_REQUIRE(d_tile_start != nullptr, "sc_bin_steps: tile_start is NULL");
    cudaStream_t s = sc::as_stream(stream);
    if (n_rec == 0) {
        return sc::cuda_status(
            cudaMemsetAsync(d_tile_start, 0, sizeof(int32_t) * (g.n_tiles + 1), s), "sc_bin_steps");
    }
    SC_REQUIRE(d_recs && d_items && d_ws, "sc_bin_steps: NULL pointer");
    SC_REQUIRE(ws_bytes >= sc_bin_workspace_bytes(n_rec, g.n_tiles),
               "sc_bin_steps: workspace %zu < %zu bytes", ws_bytes,
               sc_bin_workspace_bytes(n_rec, g.n_tiles));
    SC_REQUIRE(g.rec_per_image == 0 || (int64_t)g.rec_per_image * (g.n_tiles / g.tiles_per_image) >= n_rec,
               "sc_bin_steps: rec_per_image too small for n_rec");
    const int chunk = sc::bin_chunk(n_rec, g.n_tiles);
    const int n_chunks = (n_rec + chunk - 1) / chunk;
    int32_t *counts = static_cast<int32_t *>(d_ws);
    int32_t *tile_total = counts + (size_t)n_chunks * g.n_tiles;
    const size_t smem = (size_t)g.n_tiles * sizeof(int32_t);
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(bin_count_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(bin_scatter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr_set = true;
    }
    bin_count_kernel<<<n_chunks, 256, smem, s>>>(d_recs, n_rec, g, chunk, counts);
    bin_chunk_offsets_kernel<<<(g.n_tiles + 255) / 256, 256, 0, s>>>(counts, n_chunks, g.n_tiles,
                                                                      tile_total);
    bin_tile_scan_kernel<<<1, 1024, 0, s>>>(tile_total, g.n_tiles, capacity, d_tile_start, d_status);
    bin_scatter_kernel<<<n_chunks, 32, smem, s>>>(d_recs, n_rec, g, chunk, counts, d_tile_start,
                                                  d_items, capacity);
    return sc::launch_status("sc_bin_steps");
}
