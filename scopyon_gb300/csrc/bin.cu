// Counting sort of splat records by tile.
//
// The reference adds each particle's footprint straight into the image
// (src/scopyon/_epifm.py:1262-1264, :277-282).  Here each record is filed
// under the tile that holds its first footprint pixel, so one CTA can sum all
// of a tile's footprints (which reach into a halo past the tile) in shared
// memory with no global atomics on pixels.  Box-path and summed-area-path
// records go to separate bins (bin t and n_tiles + t for tile t).  Records
// are counted per bin, scattered with one atomic cursor per bin, and each
// bin's list is then sorted by record index: the final order is the
// reference's own accumulation order (sub-step, then particle) and does not
// depend on scheduling.
#include <mutex>

#include "sc_common.cuh"
#include "bin.cuh"

namespace {

constexpr int kSortSmem = 4096;  // tile lists up to this length are sorted in shared memory

// Per-bin counts: a shared-memory histogram per CTA when the bins fit, else
// global atomics directly.
__global__ void bin_count_kernel(const ScStepRec *recs, int n_rec, sc::TileGeom g, int n_bins,
                                 int use_smem, int32_t *tile_count) {
    extern __shared__ int32_t hist[];
    if (use_smem) {
        for (int t = threadIdx.x; t < n_bins; t += blockDim.x) hist[t] = 0;
        __syncthreads();
    }
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_rec; r += gridDim.x * blockDim.x) {
        const int t = sc::record_tile(recs[r], r, g);
        if (t >= 0) atomicAdd(use_smem ? &hist[t] : &tile_count[t], 1);
    }
    if (use_smem) {
        __syncthreads();
        for (int t = threadIdx.x; t < n_bins; t += blockDim.x)
            if (hist[t]) atomicAdd(&tile_count[t], hist[t]);
    }
}

// Single-CTA exclusive scan of per-tile counts -> tile_start[0..n_tiles]; the
// scatter cursors start at the same offsets.
__global__ void bin_tile_scan_kernel(const int32_t *tile_count, int n_tiles, int32_t *tile_start,
                                     int32_t *cursor) {
    __shared__ int32_t warp_tot[32];
    __shared__ int32_t carry_s;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry_s = 0;
    __syncthreads();
    for (int base = 0; base < n_tiles; base += blockDim.x) {
        const int t = base + threadIdx.x;
        const int32_t v = t < n_tiles ? tile_count[t] : 0;
        int32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t n = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += n;
        }
        if (lane == 31) warp_tot[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int32_t w = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int32_t n = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += n;
            }
            warp_tot[lane] = w;
        }
        __syncthreads();
        const int32_t incl = x + (warp > 0 ? warp_tot[warp - 1] : 0) + carry_s;
        if (t < n_tiles) {
            tile_start[t] = incl - v;
            cursor[t] = incl - v;
        }
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry_s = incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) tile_start[n_tiles] = carry_s;
}

__global__ void bin_scatter_kernel(const ScStepRec *recs, int n_rec, sc::TileGeom g,
                                   int32_t *cursor, int32_t *items) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n_rec; r += gridDim.x * blockDim.x) {
        const int t = sc::record_tile(recs[r], r, g);
        if (t >= 0) items[atomicAdd(&cursor[t], 1)] = r;
    }
}

// Ascending compare-exchange of a[i] and a[l] (l > i); positions >= n hold
// +inf implicitly and are never touched.
__device__ __forceinline__ void cmp_swap(int32_t *a, int i, int l, int n) {
    if (l >= n) return;
    const int32_t x = a[i], y = a[l];
    if (x > y) {
        a[i] = y;
        a[l] = x;
    }
}

// Bitonic sorting network in its "flip" form (every comparator ascending), so
// that a list of any length n sorts in place with virtual +inf padding up to
// the next power of two.  Called by a whole CTA; a is shared or global memory
// owned by this CTA.
__device__ void bitonic_flip_sort(int32_t *a, int n) {
    int n2 = 1;
    while (n2 < n) n2 <<= 1;
    for (int k = 2; k <= n2; k <<= 1) {
        for (int i = threadIdx.x; i < n2; i += blockDim.x) {
            const int l = i ^ (k - 1);
            if (l > i) cmp_swap(a, i, l, n);
        }
        __syncthreads();
        for (int j = k >> 2; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < n2; i += blockDim.x) {
                const int l = i ^ j;
                if (l > i) cmp_swap(a, i, l, n);
            }
            __syncthreads();
        }
    }
}

// One CTA per tile: sort the tile's record indices ascending, in shared
// memory when the list fits, in place in global memory otherwise.
__global__ void bin_sort_kernel(const int32_t *tile_start, int32_t *items) {
    __shared__ int32_t buf[kSortSmem];
    const int t = blockIdx.x;
    const int b0 = tile_start[t], n = tile_start[t + 1] - b0;
    if (n <= 1) return;
    int32_t *list = items + b0;
    if (n <= kSortSmem) {
        for (int i = threadIdx.x; i < n; i += blockDim.x) buf[i] = list[i];
        __syncthreads();
        bitonic_flip_sort(buf, n);
        for (int i = threadIdx.x; i < n; i += blockDim.x) list[i] = buf[i];
        return;
    }
    bitonic_flip_sort(list, n);
}

}  // namespace

namespace sc {

int tile_geom(const ScSplatParams *p, TileGeom &g) {
    SC_REQUIRE(p != nullptr, "splat params are NULL");
    SC_REQUIRE(p->tile == 8 || p->tile == 16 || p->tile == 32, "tile=%d must be 8, 16 or 32",
               p->tile);
    SC_REQUIRE(p->warps == 1 || p->warps == 2 || p->warps == 4 || p->warps == 8,
               "warps=%d must be 1, 2, 4 or 8", p->warps);
    SC_REQUIRE(p->halo >= 1 && p->halo <= 512, "halo=%d out of range", p->halo);
    SC_REQUIRE(p->nw > 0 && p->nh > 0, "image size %dx%d", p->nw, p->nh);
    SC_REQUIRE(p->tiles_x == (p->nw + p->tile - 1) / p->tile &&
                   p->tiles_y == (p->nh + p->tile - 1) / p->tile,
               "tiles_x/tiles_y inconsistent with image and tile size");
    SC_REQUIRE(p->n_images >= 1, "n_images=%d", p->n_images);
    g.tile = p->tile;
    g.halo = p->halo;
    g.edge = p->tile + p->halo;
    g.warps = p->warps;
    g.tiles_x = p->tiles_x;
    g.tiles_y = p->tiles_y;
    g.tiles_per_image = p->tiles_x * p->tiles_y;
    g.n_tiles = g.tiles_per_image * p->n_images;
    g.nw = p->nw;
    g.nh = p->nh;
    g.rec_per_image = p->rec_per_image;
    g.n_images = p->n_images;
    SC_REQUIRE(g.n_tiles <= (1 << 24), "too many tiles (%d) in one launch", g.n_tiles);
    return SC_OK;
}

}  // namespace sc

extern "C" size_t sc_bin_workspace_bytes(int n_rec, int n_tiles_total) {
    if (n_rec <= 0 || n_tiles_total <= 0) return 0;
    return (size_t)4 * n_tiles_total * sizeof(int32_t);  // counts and cursors of 2 bins per tile
}

extern "C" int sc_bin_steps(const ScStepRec *d_recs, int n_rec, const ScSplatParams *p,
                            void *d_ws, size_t ws_bytes, int32_t *d_tile_start, int32_t *d_items,
                            int32_t *d_status, void *stream) {
    (void)d_status;
    sc::TileGeom g;
    int rc = sc::tile_geom(p, g);
    if (rc) return rc;
    SC_REQUIRE(n_rec >= 0, "n_rec=%d", n_rec);
    SC_REQUIRE(d_tile_start != nullptr, "sc_bin_steps: tile_start is NULL");
    cudaStream_t s = sc::as_stream(stream);
    if (n_rec == 0) {
        return sc::cuda_status(
            cudaMemsetAsync(d_tile_start, 0, sizeof(int32_t) * (2 * g.n_tiles + 1), s),
            "sc_bin_steps");
    }
    SC_REQUIRE(d_recs && d_items && d_ws, "sc_bin_steps: NULL pointer");
    SC_REQUIRE(ws_bytes >= sc_bin_workspace_bytes(n_rec, g.n_tiles),
               "sc_bin_steps: workspace %zu < %zu bytes", ws_bytes,
               sc_bin_workspace_bytes(n_rec, g.n_tiles));
    SC_REQUIRE(g.rec_per_image == 0 || (int64_t)g.rec_per_image * g.n_images >= n_rec,
               "sc_bin_steps: rec_per_image too small for n_rec");
    const int n_bins = 2 * g.n_tiles;
    int32_t *tile_count = static_cast<int32_t *>(d_ws);
    int32_t *cursor = tile_count + n_bins;
    rc = sc::cuda_status(cudaMemsetAsync(tile_count, 0, sizeof(int32_t) * n_bins, s),
                         "sc_bin_steps memset");
    if (rc) return rc;
    const size_t smem = (size_t)n_bins * sizeof(int32_t);
    const int use_smem = smem <= 96 * 1024;
    if (use_smem && smem > 48 * 1024)
        cudaFuncSetAttribute(bin_count_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int grid = (n_rec + 1023) / 1024;
    if (grid > 152 * 4) grid = 152 * 4;
    bin_count_kernel<<<grid, 256, use_smem ? smem : 0, s>>>(d_recs, n_rec, g, n_bins, use_smem,
                                                           tile_count);
    bin_tile_scan_kernel<<<1, 1024, 0, s>>>(tile_count, n_bins, d_tile_start, cursor);
    int sgrid = (n_rec + 255) / 256;
    if (sgrid > 152 * 16) sgrid = 152 * 16;
    bin_scatter_kernel<<<sgrid, 256, 0, s>>>(d_recs, n_rec, g, cursor, d_items);
    bin_sort_kernel<<<n_bins, 256, 0, s>>>(d_tile_start, d_items);
    return sc::launch_status("sc_bin_steps");
}

// ---------------------------------------------------------------------------
// sc_bin_steps_static: the same counting sort with its counts and cursors in
// a fixed device array instead of a caller workspace, for callers that have
// no device allocator to hand (a C or FFI host that is given only the record
// and output buffers) or that must not allocate per frame.
namespace {

static __device__ __align__(256) int32_t g_bin_scratch[4 * SC_BIN_STATIC_MAX_TILES];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void *g_scratch_ptr[kMaxDevices];

// Address of g_bin_scratch on the current device, looked up once per device.
int bin_scratch(void **out) {
    int dev = -1;
    int rc = sc::cuda_status(cudaGetDevice(&dev), "sc_bin_steps_static: cudaGetDevice");
    if (rc) return rc;
    SC_REQUIRE(dev >= 0 && dev < kMaxDevices, "sc_bin_steps_static: device %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (g_scratch_ptr[dev] == nullptr) {
        void *p = nullptr;
        rc = sc::cuda_status(cudaGetSymbolAddress(&p, g_bin_scratch),
                             "sc_bin_steps_static: cudaGetSymbolAddress");
        if (rc) return rc;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return SC_OK;
}

}  // namespace

extern "C" int sc_bin_steps_static(const ScStepRec *d_recs, int n_rec, const ScSplatParams *p,
                                   int32_t *d_tile_start, int32_t *d_items, int32_t *d_status,
                                   void *stream) {
    sc::TileGeom g;
    int rc = sc::tile_geom(p, g);
    if (rc) return rc;
    SC_REQUIRE(g.n_tiles <= SC_BIN_STATIC_MAX_TILES,
               "sc_bin_steps_static: %d tiles exceed the fixed scratch of %d tiles", g.n_tiles,
               SC_BIN_STATIC_MAX_TILES);
    void *ws = nullptr;
    rc = bin_scratch(&ws);
    if (rc) return rc;
    // sc_bin_steps clears the counts on the stream before counting; the
    // cursors are written by the scan.
    return sc_bin_steps(d_recs, n_rec, p, ws, sizeof(g_bin_scratch), d_tile_start, d_items,
                        d_status, stream);
}
