/*
 * Seeded synthetic inputs for the segmentation path.
 *
 * The reference ships no images, datasets or fixtures: its only driver loads a
 * user-supplied file (samples/src/main.cu:157-158).  Every workload here is a
 * seeded synthetic image with the shapes and value distributions of the
 * benchmark configurations: Voronoi cells of uniform colour (optionally drawn
 * from a small palette and lit by a horizontal gradient) plus clipped Gaussian
 * noise, and a maze + blob label image for the labelling stress case.
 *
 * Generators are plain C, deterministic for a given seed, and produce the same
 * bytes on x86-64 and AArch64 (integer geometry, IEEE double arithmetic with
 * contraction disabled by the build, libm only for the Box-Muller transform).
 *
 * PRNGs: SplitMix64 (Steele, Lea, Flood 2014) for seeding and PCG32 (O'Neill
 * 2014, XSH-RR variant) for streams; Gaussians by the Box-Muller transform.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/split_synth.h"

typedef struct {
  uint64_t state;
  uint64_t inc;
} pcg32_t;

static uint64_t splitmix64_next(uint64_t* s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static uint32_t pcg32_next(pcg32_t* r) {
  uint64_t old = r->state;
  r->state = old * 6364136223846793005ull + r->inc;
  uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
  uint32_t rot = (uint32_t)(old >> 59u);
  return (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
}

static pcg32_t pcg32_from(uint64_t seed) {
  uint64_t s = seed;
  pcg32_t r;
  r.state = 0;
  r.inc = (splitmix64_next(&s) << 1u) | 1u;
  pcg32_next(&r);
  r.state += splitmix64_next(&s);
  pcg32_next(&r);
  return r;
}

/* Uniform integer in [0, bound) by multiply-shift (bias < 2^-32 * bound). */
static uint32_t pcg32_bounded(pcg32_t* r, uint32_t bound) {
  return (uint32_t)(((uint64_t)pcg32_next(r) * (uint64_t)bound) >> 32);
}

/* Uniform double in (0, 1]. */
static double pcg32_unit_open0(pcg32_t* r) {
  return ((double)pcg32_next(r) + 1.0) * (1.0 / 4294967296.0);
}

static double gaussian(pcg32_t* r) {
  const double two_pi = 6.283185307179586476925286766559;
  double u1 = pcg32_unit_open0(r);
  double u2 = (double)pcg32_next(r) * (1.0 / 4294967296.0);
  return sqrt(-2.0 * log(u1)) * cos(two_pi * u2);
}

static uint8_t clip_round_u8(double v) {
  double f = floor(v + 0.5);
  if (f < 0.0) return 0;
  if (f > 255.0) return 255;
  return (uint8_t)f;
}

/* Stream for row y of an image: independent of every other row, so rows can
 * be generated in any order (and in parallel) with identical output. */
static pcg32_t row_stream(uint64_t seed, int y) {
  uint64_t s = seed ^ 0xD1B54A32D192ED03ull;
  uint64_t a = splitmix64_next(&s);
  return pcg32_from(a + (uint64_t)(uint32_t)y * 0x9E3779B97F4A7C15ull);
}

int split_synth_voronoi_rgb8(uint64_t seed, int width, int height, int ncells,
                             int npalette, int illum_gradient, double sigma,
                             uint8_t* out_rgb) {
  if (width <= 0 || height <= 0 || ncells <= 0 || !out_rgb || npalette < 0 ||
      npalette > 4096)
    return 1;
  pcg32_t rng = pcg32_from(seed);
  int32_t* cx = (int32_t*)malloc(sizeof(int32_t) * (size_t)ncells);
  int32_t* cy = (int32_t*)malloc(sizeof(int32_t) * (size_t)ncells);
  uint8_t* col = (uint8_t*)malloc(3u * (size_t)ncells);
  uint8_t* pal = (uint8_t*)malloc(3u * (size_t)(npalette > 0 ? npalette : 1));
  if (!cx || !cy || !col || !pal) {
    free(cx); free(cy); free(col); free(pal);
    return 2;
  }
  for (int i = 0; i < ncells; ++i) {
    cx[i] = (int32_t)pcg32_bounded(&rng, (uint32_t)width);
    cy[i] = (int32_t)pcg32_bounded(&rng, (uint32_t)height);
  }
  for (int i = 0; i < npalette; ++i) {
    uint32_t u = pcg32_next(&rng);
    pal[3 * i + 0] = (uint8_t)(u & 255u);
    pal[3 * i + 1] = (uint8_t)((u >> 8) & 255u);
    pal[3 * i + 2] = (uint8_t)((u >> 16) & 255u);
  }
  for (int i = 0; i < ncells; ++i) {
    if (npalette > 0) {
      uint32_t p = pcg32_bounded(&rng, (uint32_t)npalette);
      memcpy(col + 3 * i, pal + 3 * p, 3);
    } else {
      uint32_t u = pcg32_next(&rng);
      col[3 * i + 0] = (uint8_t)(u & 255u);
      col[3 * i + 1] = (uint8_t)((u >> 8) & 255u);
      col[3 * i + 2] = (uint8_t)((u >> 16) & 255u);
    }
  }
  const double inv_wm1 = width > 1 ? 1.0 / (double)(width - 1) : 0.0;
#pragma omp parallel for schedule(dynamic, 4)
  for (int y = 0; y < height; ++y) {
    pcg32_t rr = row_stream(seed, y);
    uint8_t* row = out_rgb + (size_t)y * (size_t)width * 3u;
    for (int x = 0; x < width; ++x) {
      int best = 0;
      int64_t bd = INT64_MAX;
      for (int i = 0; i < ncells; ++i) {
        int64_t dx = (int64_t)x - cx[i], dy = (int64_t)y - cy[i];
        int64_t d = dx * dx + dy * dy;
        if (d < bd) { bd = d; best = i; }
      }
      double gain = illum_gradient ? 0.6 + 0.4 * ((double)x * inv_wm1) : 1.0;
      for (int c = 0; c < 3; ++c) {
        double v = (double)col[3 * best + c] * gain;
        if (sigma > 0.0) v += sigma * gaussian(&rr);
        row[3 * x + c] = clip_round_u8(v);
      }
    }
  }
  free(cx); free(cy); free(col); free(pal);
  return 0;
}

int split_synth_pick_centroids(uint64_t seed, const uint8_t* rgb, int width,
                               int height, int nclusters, int dim,
                               float xy_scale, float* centroids) {
  if (!rgb || !centroids || width <= 0 || height <= 0 || nclusters <= 0 ||
      (dim != 3 && dim != 5))
    return 1;
  const int64_t n = (int64_t)width * height;
  if (n < nclusters) return 1;
  pcg32_t rng = pcg32_from(seed ^ 0xC2B2AE3D27D4EB4Full);
  int64_t* picked = (int64_t*)malloc(sizeof(int64_t) * (size_t)nclusters);
  if (!picked) return 2;
  for (int k = 0; k < nclusters; ++k) {
    int64_t idx;
    int dup;
    do {
      uint64_t r = ((uint64_t)pcg32_next(&rng) << 32) | pcg32_next(&rng);
      idx = (int64_t)(r % (uint64_t)n);
      dup = 0;
      for (int j = 0; j < k; ++j) dup |= (picked[j] == idx);
    } while (dup);
    picked[k] = idx;
    const uint8_t* p = rgb + 3 * idx;
    for (int c = 0; c < 3; ++c)
      centroids[c * nclusters + k] = split_synth_feature_u8(p[c]);
    if (dim == 5) {
      centroids[3 * nclusters + k] = xy_scale * (float)(idx % width);
      centroids[4 * nclusters + k] = xy_scale * (float)(idx / width);
    }
  }
  free(picked);
  return 0;
}

float split_synth_feature_u8(uint8_t v) { return (float)v / 255.0f; }

/*
 * Maze + blob label image for the labelling stress case.
 *
 * A perfect maze is carved by randomised depth-first search on a coarse grid
 * of 4x4-pixel cells: every cell owns a 2x2 corridor block and each tree edge
 * opens a 2-pixel-wide passage, so the corridor (label 0) is one serpentine
 * component covering half of the image whose 2-pixel walls keep 8-connected
 * labelling from leaking across diagonals.  The wall region is then cut by a
 * grid of random row/column strips (4..22 px) into blobs; each strip cell's
 * wall pixels take a random nonzero 32-bit label.  Pixels beyond the last full
 * coarse cell are wall.
 */
int split_synth_maze_labels(uint64_t seed, int width, int height,
                            int32_t* out) {
  if (!out || width <= 0 || height <= 0) return 1;
  const int cw = width / 4, ch = height / 4;
  pcg32_t rng = pcg32_from(seed ^ 0x165667B19E3779F9ull);
  uint8_t* wall = (uint8_t*)malloc((size_t)width * (size_t)height);
  if (!wall) return 2;
  memset(wall, 1, (size_t)width * (size_t)height);
  if (cw > 0 && ch > 0) {
    const int64_t nc = (int64_t)cw * ch;
    uint8_t* seen = (uint8_t*)calloc((size_t)nc, 1);
    int32_t* stack = (int32_t*)malloc(sizeof(int32_t) * (size_t)nc);
    if (!seen || !stack) {
      free(seen); free(stack); free(wall);
      return 2;
    }
    int64_t sp = 0;
    int32_t start = (int32_t)pcg32_bounded(&rng, (uint32_t)nc);
    stack[sp++] = start;
    seen[start] = 1;
#define OPEN2x2(px, py)                                            \
  do {                                                             \
    for (int dy_ = 0; dy_ < 2; ++dy_)                              \
      for (int dx_ = 0; dx_ < 2; ++dx_)                            \
        wall[(size_t)((py) + dy_) * width + (px) + dx_] = 0;       \
  } while (0)
    {
      int sx = start % cw, sy = start / cw;
      OPEN2x2(4 * sx, 4 * sy);
    }
    while (sp > 0) {
      int32_t c = stack[sp - 1];
      int x = c % cw, y = c / cw;
      int cand[4], nc4 = 0;
      if (x > 0 && !seen[c - 1]) cand[nc4++] = 0;
      if (x + 1 < cw && !seen[c + 1]) cand[nc4++] = 1;
      if (y > 0 && !seen[c - cw]) cand[nc4++] = 2;
      if (y + 1 < ch && !seen[c + cw]) cand[nc4++] = 3;
      if (nc4 == 0) {
        --sp;
        continue;
      }
      int dir = cand[pcg32_bounded(&rng, (uint32_t)nc4)];
      int nx = x + (dir == 1) - (dir == 0);
      int ny = y + (dir == 3) - (dir == 2);
      int32_t nxt = ny * cw + nx;
      seen[nxt] = 1;
      OPEN2x2(4 * nx, 4 * ny);
      /* passage between the two 2x2 blocks */
      int mx = (4 * x + 4 * nx) / 2, my = (4 * y + 4 * ny) / 2;
      OPEN2x2(mx, my);
      stack[sp++] = nxt;
    }
#undef OPEN2x2
    free(seen);
    free(stack);
  }
  /* random strip grid for the blobs */
  int32_t* colcut = (int32_t*)malloc(sizeof(int32_t) * (size_t)width);
  int32_t* rowcut = (int32_t*)malloc(sizeof(int32_t) * (size_t)height);
  if (!colcut || !rowcut) {
    free(colcut); free(rowcut); free(wall);
    return 2;
  }
  int ncol = 0;
  for (int x = 0; x < width;) {
    int w = 4 + (int)pcg32_bounded(&rng, 19);
    for (int i = 0; i < w && x < width; ++i, ++x) colcut[x] = ncol;
    ++ncol;
  }
  int nrow = 0;
  for (int y = 0; y < height;) {
    int h = 4 + (int)pcg32_bounded(&rng, 19);
    for (int i = 0; i < h && y < height; ++i, ++y) rowcut[y] = nrow;
    ++nrow;
  }
  const uint64_t lseed = splitmix64_next(&seed);
#pragma omp parallel for schedule(static)
  for (int y = 0; y < height; ++y) {
    for (int x = 0; x < width; ++x) {
      size_t i = (size_t)y * width + x;
      if (!wall[i]) {
        out[i] = 0;
      } else {
        uint64_t s = lseed + (uint64_t)rowcut[y] * 0x100000001B3ull +
                     (uint64_t)colcut[x] * 0x9E3779B97F4A7C15ull;
        uint32_t v = (uint32_t)splitmix64_next(&s);
        out[i] = (int32_t)(v | 1u);
      }
    }
  }
  free(colcut); free(rowcut); free(wall);
  return 0;
}
