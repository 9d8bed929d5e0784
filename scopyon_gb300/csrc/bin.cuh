// Tile geometry shared by the binning and splat kernels.
#pragma once

#include "sc_common.cuh"

namespace sc {

struct TileGeom {
    int tile, halo, edge, warps, tiles_x, tiles_y, tiles_per_image, n_tiles, nw, nh,
        rec_per_image, n_images;
};

int tile_geom(const ScSplatParams *p, TileGeom &g);

// Pointers into a binning workspace: per-bin counts and cursors, then (when
// the workspace is large enough) each record's bin and rank in its bin.
struct BinLayout {
    int32_t *count, *cursor, *rec_bin, *rec_rank;
    int32_t *big;  // count of long bins, then their indices
    // radix sort scratch (record sets of kRadixMinRecords or more), else NULL
    int32_t *rx_vals, *rx_counts, *rx_total;
};

// From this many records on, bin lists are ordered by a radix sort.
constexpr int kRadixMinRecords = 1 << 20;
int bin_layout(const TileGeom &g, int n_rec, void *d_ws, size_t ws_bytes, BinLayout &b);

// Bin of a record: the tile holding its first footprint pixel, plus n_tiles
// for records that take the summed-area path; -1 when it has no pixels or
// its first pixel lies outside the image (the engine's producers clamp the
// first pixel to >= 0; a caller-built record with a negative start is
// dropped, and record_malformed() tells the counting pass to report it).
__device__ __forceinline__ int record_tile(const ScStepRec &rec, int r, const TileGeom &g) {
    if (rec.n_i < 2 || rec.n_j < 2 || rec.slot < 0) return -1;
    const int img = g.rec_per_image > 0 ? r / g.rec_per_image : 0;
    if (img >= g.n_images || rec.i_start < 0 || rec.j_start < 0 || rec.i_start >= g.nw ||
        rec.j_start >= g.nh)
        return -1;
    const int t = img * g.tiles_per_image + (rec.i_start / g.tile) * g.tiles_y + rec.j_start / g.tile;
    return rec.box ? t : t + g.n_tiles;
}

// A record with pixels to splat whose first pixel has a negative index: no
// producer of this library writes one, so it came from a caller and is
// reported (status bit 6) instead of being filed under a tile.
__device__ __forceinline__ bool record_malformed(const ScStepRec &rec) {
    return rec.n_i >= 2 && rec.n_j >= 2 && rec.slot >= 0 && (rec.i_start < 0 || rec.j_start < 0);
}

// Counts record r into its bin and keeps its bin and, when rec_rank is given,
// its rank (-1: no bin).  The radix path needs no ranks: its count is a
// reduction with no value returned.
__device__ __forceinline__ void bin_record(const TileGeom &g, const ScStepRec &rec, int r,
                                           int32_t *count, int32_t *rec_bin, int32_t *rec_rank) {
    const int t = record_tile(rec, r, g);
    rec_bin[r] = t;
    if (rec_rank)
        rec_rank[r] = t >= 0 ? atomicAdd(&count[t], 1) : -1;
    else if (t >= 0)
        atomicAdd(&count[t], 1);
}

// The rank array bin_record should fill: none on the radix path.
__host__ __device__ __forceinline__ int32_t *rank_array(const BinLayout &b) {
    return b.rx_vals ? nullptr : b.rec_rank;
}

}  // namespace sc
