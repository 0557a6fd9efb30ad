// Image geometry shared by the tile kernels (labelling, merge, stencils) so
// that one launch can cover one image or a whole batch of images.
//
// A batch keeps all its images in one pixel arena: image i occupies pixels
// [off, off + W * H) (row-major).  Every tile kernel runs over a 1-D grid of
// kTileH x kTileW tiles; a block finds its image by binary search over the
// images' first tile index.  A single image is a one-entry table carried by
// value in the kernel parameters.
#pragma once

#include <cuda.h>

#include "common.cuh"

namespace sg {

constexpr int kTileH = 32, kTileW = 64;

struct ImgGeom {
  int W, H;
  long long off;      // first pixel in the arena
  int tile_begin;     // first tile of this image in the launch's tile grid
  int tiles_x;        // tiles per tile row
  int tma_ok;         // int32 label rows / RGB8 rows addressable by TMA
};

struct Geoms {
  ImgGeom one;               // used when n == 1
  const ImgGeom* table;      // device table when n > 1
  const CUtensorMap* maps;   // optional per-image tensor maps (batch stencils)
  int n;
  int total_tiles;
  long long total_px;
};

inline int tiles_of(int W, int H) {
  return ((W + kTileW - 1) / kTileW) * ((H + kTileH - 1) / kTileH);
}

inline Geoms single_geom(int W, int H) {
  Geoms g{};
  g.one.W = W;
  g.one.H = H;
  g.one.off = 0;
  g.one.tile_begin = 0;
  g.one.tiles_x = (W + kTileW - 1) / kTileW;
  g.one.tma_ok = 1;
  g.table = nullptr;
  g.maps = nullptr;
  g.n = 1;
  g.total_tiles = tiles_of(W, H);
  g.total_px = (long long)W * H;
  return g;
}

struct TileRef {
  int img;
  int W, H;
  long long off;
  int tx0, ty0;   // tile origin (pixels)
  int tma_ok;
  int tiles_x;    // tiles per tile row of the image (neighbour tiles: +-1, +-tiles_x)
};

__device__ __forceinline__ TileRef tile_ref(const Geoms& gs, int tile) {
  int img = 0;
  if (gs.n > 1) {
    int lo = 0, hi = gs.n - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (gs.table[mid].tile_begin <= tile) lo = mid; else hi = mid - 1;
    }
    img = lo;
  }
  const ImgGeom& g = gs.n > 1 ? gs.table[img] : gs.one;
  const int t = tile - g.tile_begin;
  const int ty = t / g.tiles_x, tx = t - ty * g.tiles_x;
  TileRef r;
  r.img = img;
  r.W = g.W;
  r.H = g.H;
  r.off = g.off;
  r.tx0 = tx * kTileW;
  r.ty0 = ty * kTileH;
  r.tma_ok = g.tma_ok;
  r.tiles_x = g.tiles_x;
  return r;
}

// Sobel normals of the L* plane straight from RGB8 over a geometry table;
// with features4 set, the same pass writes the float4 byte / 255 features.
int normals_rgb8_geoms(const uint8_t* rgb, const Geoms& gs, float depth, float* normals,
                       float* features4, cudaStream_t st);

}  // namespace sg
