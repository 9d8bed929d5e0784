// Tile geometry shared by the binning and splat kernels.
#pragma once

#include "sc_common.cuh"

namespace sc {

struct TileGeom {
    int tile, tiles_x, tiles_y, tiles_per_image, n_tiles, nw, nh, rec_per_image;
};

struct TileRange {
    int base, tx0, tx1, ty0, ty1;
};

int tile_geom(const ScSplatParams *p, TileGeom &g);
int bin_chunk(int n_rec, int n_tiles);

// Tiles touched by a record's pixel footprint; false when it has no pixels.
__device__ __forceinline__ bool record_tiles(const ScStepRec &rec, int r, const TileGeom &g,
                                             TileRange &tr) {
    if (rec.n_i < 2 || rec.n_j < 2) return false;
    const int img = g.rec_per_image > 0 ? r / g.rec_per_image : 0;
    tr.base = img * g.tiles_per_image;
    const int i1 = rec.i_start + rec.n_i - 2;
    const int j1 = rec.j_start + rec.n_j - 2;
    tr.tx0 = rec.i_start / g.tile;
    tr.tx1 = min(i1, g.nw - 1) / g.tile;
    tr.ty0 = rec.j_start / g.tile;
    tr.ty1 = min(j1, g.nh - 1) / g.tile;
    return tr.tx1 >= tr.tx0 && tr.ty1 >= tr.ty0;
}

}  // namespace sc
