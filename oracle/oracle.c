/*
 * ORACLE - test infrastructure only.
 *
 * CPU restatement of nitronoid/split's segmentation hot path, used by tests/,
 * by __graft_entry__.smoke() and by bench.py's cpu_baseline leg as the checker.
 * Nothing in the product library links, loads or calls this file.
 *
 * Each function names the reference file:line it restates (paths relative to
 * the reference project root).  Integer work (labelling, compression, merge,
 * erosion) is exact.  Floating-point work comes in two flavours:
 *   - *_f32 functions reproduce the device library's FP32 formula bit for bit
 *     (explicit fmaf chains), used for exact label comparisons;
 *   - *_f64 functions evaluate the same mathematics in double precision, used
 *     as the accuracy reference (centroids, normals, luminance).
 * Built with -ffp-contract=off so the compiler never fuses what is written as
 * separate operations.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_API __attribute__((visibility("default")))

/* ------------------------------------------------------------------------ */
/* k-means                                                                  */
/* ------------------------------------------------------------------------ */

/* Assignment step, FP32.  Restates split/src/split/device/kmeans/label.cu:23-32
 * (squared distance summed in dimension order) and :98-105 (argmin with
 * thrust::minimum over (distance, index) tuples: ties go to the lowest k).
 * The distance is accumulated as d = fmaf(t, t, d), t = x - c, exactly as the
 * device kernel does.  Points and centroids are planar (dim x n). */
ORC_API void orc_kmeans_assign_f32(const float* pts, int dim, int64_t n,
                                   const float* cent, int k,
                                   int32_t* labels) {
  /* pixels are independent: threads change nothing in the result */
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    float best = INFINITY;
    int bk = 0;
    for (int c = 0; c < k; ++c) {
      float d = 0.0f;
      for (int j = 0; j < dim; ++j) {
        float t = pts[(int64_t)j * n + i] - cent[j * k + c];
        d = fmaf(t, t, d);
      }
      if (d < best) {
        best = d;
        bk = c;
      }
    }
    labels[i] = bk;
  }
}

/* Assignment step in FP64: best label plus best and second-best distances,
 * for the near-tie rule (labels may differ where (d2 - d1) <= rel * d2). */
ORC_API void orc_kmeans_assign_f64(const float* pts, int dim, int64_t n,
                                   const float* cent, int k, int32_t* labels,
                                   double* d1, double* d2) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    double b1 = INFINITY, b2 = INFINITY;
    int bk = 0;
    for (int c = 0; c < k; ++c) {
      double d = 0.0;
      for (int j = 0; j < dim; ++j) {
        double t = (double)pts[(int64_t)j * n + i] - (double)cent[j * k + c];
        d += t * t;
      }
      if (d < b1) {
        b2 = b1;
        b1 = d;
        bk = c;
      } else if (d < b2) {
        b2 = d;
      }
    }
    labels[i] = bk;
    if (d1) d1[i] = b1;
    if (d2) d2[i] = b2;
  }
}

/* Update step in FP64.  Restates split/src/split/device/kmeans/centroids.cu:
 * 22-101 (per-cluster mean of the member points).  Deliberate divergence: a
 * cluster with no members keeps its previous centroid (the reference's
 * compacted reduce_by_key shifts later centroids down a slot instead,
 * centroids.cu:78-100).  counts[k] receives the member count. */
ORC_API void orc_kmeans_update_f64(const int32_t* labels, const float* pts,
                                   int dim, int64_t n, const float* cent_in,
                                   int k, double* cent_out, int64_t* counts) {
  double* sum = (double*)calloc((size_t)dim * k, sizeof(double));
  int64_t* cnt = (int64_t*)calloc((size_t)k, sizeof(int64_t));
  for (int64_t i = 0; i < n; ++i) {
    int l = labels[i];
    if (l < 0 || l >= k) continue;
    cnt[l]++;
    for (int j = 0; j < dim; ++j) sum[j * k + l] += (double)pts[(int64_t)j * n + i];
  }
  for (int c = 0; c < k; ++c) {
    for (int j = 0; j < dim; ++j)
      cent_out[j * k + c] =
          cnt[c] ? sum[j * k + c] / (double)cnt[c] : (double)cent_in[j * k + c];
    if (counts) counts[c] = cnt[c];
  }
  free(sum);
  free(cnt);
}

/* ------------------------------------------------------------------------ */
/* connected components                                                     */
/* ------------------------------------------------------------------------ */

static int32_t uf_find(int32_t* p, int32_t x) {
  int32_t r = x;
  while (p[r] != r) r = p[r];
  while (p[x] != r) {
    int32_t nx = p[x];
    p[x] = r;
    x = nx;
  }
  return r;
}

static void uf_union_min(int32_t* p, int32_t a, int32_t b) {
  a = uf_find(p, a);
  b = uf_find(p, b);
  if (a == b) return;
  if (a < b) p[b] = a; else p[a] = b;
}

/* Connected-component labelling.  Restates the fixed point of
 * split/src/split/device/ccl/connected_components.cu:80-181 (iterated max
 * propagation over row runs and column runs of equal cluster label, i.e.
 * 4-connectivity, converging to the maximum linear index of the component).
 * connectivity is 4 or 8 (8 adds the diagonals, an extension); convention 0
 * labels every pixel with the minimum linear index of its component, 1 with
 * the maximum (the reference's fixed point).  Sequential union-find. */
ORC_API int orc_ccl(const int32_t* in, int width, int height, int connectivity,
                    int convention, int32_t* out) {
  if (width <= 0 || height <= 0 || (connectivity != 4 && connectivity != 8))
    return 1;
  const int64_t n = (int64_t)width * height;
  if (n > 0x7fffffff) return 1;
  int32_t* p = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  if (!p) return 2;
  for (int64_t i = 0; i < n; ++i) p[i] = (int32_t)i;
  for (int y = 0; y < height; ++y) {
    for (int x = 0; x < width; ++x) {
      int32_t i = y * width + x;
      int32_t v = in[i];
      if (x > 0 && in[i - 1] == v) uf_union_min(p, i, i - 1);
      if (y > 0) {
        if (in[i - width] == v) uf_union_min(p, i, i - width);
        if (connectivity == 8) {
          if (x > 0 && in[i - width - 1] == v) uf_union_min(p, i, i - width - 1);
          if (x + 1 < width && in[i - width + 1] == v)
            uf_union_min(p, i, i - width + 1);
        }
      }
    }
  }
  if (convention == 0) {
    for (int64_t i = 0; i < n; ++i) out[i] = uf_find(p, (int32_t)i);
  } else {
    /* maximum member index per root */
    int32_t* mx = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    if (!mx) {
      free(p);
      return 2;
    }
    for (int64_t i = 0; i < n; ++i) {
      int32_t r = uf_find(p, (int32_t)i);
      mx[r] = (int32_t)i; /* increasing i: last write is the maximum */
    }
    for (int64_t i = 0; i < n; ++i) out[i] = mx[uf_find(p, (int32_t)i)];
    free(mx);
  }
  free(p);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* label compression                                                        */
/* ------------------------------------------------------------------------ */

static int cmp_i32(const void* a, const void* b) {
  int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
  return (x > y) - (x < y);
}

/* Restates split/src/split/device/ccl/compress_labels.cu:10-35: every label is
 * replaced by its rank among the sorted unique labels; returns the count. */
ORC_API int64_t orc_compress_labels(int32_t* labels, int64_t n) {
  if (n <= 0) return 0;
  int32_t* s = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  if (!s) return -1;
  memcpy(s, labels, sizeof(int32_t) * (size_t)n);
  qsort(s, (size_t)n, sizeof(int32_t), cmp_i32);
  int64_t u = 1;
  for (int64_t i = 1; i < n; ++i)
    if (s[i] != s[u - 1]) s[u++] = s[i];
  for (int64_t i = 0; i < n; ++i) {
    int64_t lo = 0, hi = u;
    while (lo < hi) {
      int64_t mid = (lo + hi) / 2;
      if (s[mid] < labels[i]) lo = mid + 1; else hi = mid;
    }
    labels[i] = (int32_t)lo;
  }
  free(s);
  return u;
}

/* ------------------------------------------------------------------------ */
/* small-segment merge                                                      */
/* ------------------------------------------------------------------------ */

static int cmp_u64(const void* a, const void* b) {
  uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
  return (x > y) - (x < y);
}

/*
 * Small-segment merge.  Labels are segment ids in [0, n).
 *
 * Adjacency: for every pixel p and each of its 8 in-image neighbours q with a
 * different label, the directed edge (L[p], L[q]) is counted - the edge set of
 * split/src/split/device/ccl/segment_adjacency.cu:112-142 and :139-144.
 *
 * policy 0 (most shared boundary): a segment s with size < P picks the
 * neighbour t with the most edges (s, t); ties go to the lowest t.
 *
 * policy 1 (reference chroma rule, merge_small_segments.cu:92-196): s picks
 * the neighbour minimising (d2, t) lexicographically, where d2 = x*x + x*x in
 * float with x = mean0[s] - mean0[t]; mean0 is the float segment mean of
 * chroma channel 0, read twice because the reference's cycle iterator wraps
 * the second channel back onto the first (merge_small_segments.cu:135-147,
 * cycle_iterator.cuh:14-21).  The mean is (float)sum / (float)size with the sum
 * formed exactly (double).  If the input labels are already non-decreasing in
 * pixel order the reference applies no merge (map_until_converged.cuh:25-30
 * compares against the sorted label copy); this is reproduced.
 *
 * Segments with size >= P map to themselves (merge_small_segments.cu:176-187);
 * a mutual pair keeps the larger id (fix_map_cycles.cuh:28-43); every pixel
 * then takes the end of its segment's map chain (map_until_converged.cuh:
 * 14-31).  One pass only.  Returns 0, or 3 if a chain does not terminate.
 */
ORC_API int orc_merge_small(const int32_t* in, int width, int height, int P,
                            int policy, const float* chroma, int32_t* out) {
  const int64_t n = (int64_t)width * height;
  if (width <= 0 || height <= 0 || n > 0x7fffffff) return 1;
  for (int64_t i = 0; i < n; ++i)
    if (in[i] < 0 || in[i] >= n) return 1;
  if (policy == 1) {
    int sorted = 1;
    for (int64_t i = 1; i < n && sorted; ++i) sorted = in[i - 1] <= in[i];
    if (sorted) {
      memcpy(out, in, sizeof(int32_t) * (size_t)n);
      return 0;
    }
  }
  int64_t* size = (int64_t*)calloc((size_t)n, sizeof(int64_t));
  int32_t* map = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  float* mean0 = NULL;
  for (int64_t i = 0; i < n; ++i) size[in[i]]++;
  for (int64_t i = 0; i < n; ++i) map[i] = (int32_t)i;
  if (policy == 1) {
    double* sum = (double*)calloc((size_t)n, sizeof(double));
    mean0 = (float*)calloc((size_t)n, sizeof(float));
    for (int64_t i = 0; i < n; ++i) sum[in[i]] += (double)chroma[i];
    for (int64_t s = 0; s < n; ++s)
      if (size[s]) mean0[s] = (float)sum[s] / (float)size[s];
    free(sum);
  }
  /* edges of small segments */
  int64_t nsmallpx = 0;
  for (int64_t i = 0; i < n; ++i) nsmallpx += size[in[i]] < P;
  uint64_t* e = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)(8 * nsmallpx + 1));
  int64_t ne = 0;
  static const int dx[8] = {-1, 0, 1, -1, 1, -1, 0, 1};
  static const int dy[8] = {-1, -1, -1, 0, 0, 1, 1, 1};
  for (int y = 0; y < height; ++y)
    for (int x = 0; x < width; ++x) {
      int32_t s = in[(int64_t)y * width + x];
      if (size[s] >= P) continue;
      for (int d = 0; d < 8; ++d) {
        int nx = x + dx[d], ny = y + dy[d];
        if (nx < 0 || ny < 0 || nx >= width || ny >= height) continue;
        int32_t t = in[(int64_t)ny * width + nx];
        if (t != s) e[ne++] = ((uint64_t)(uint32_t)s << 32) | (uint32_t)t;
      }
    }
  qsort(e, (size_t)ne, sizeof(uint64_t), cmp_u64);
  for (int64_t a = 0; a < ne;) {
    int32_t s = (int32_t)(e[a] >> 32);
    int32_t best_t = -1;
    int64_t best_c = -1;
    float best_d = INFINITY;
    int64_t b = a;
    while (b < ne && (int32_t)(e[b] >> 32) == s) {
      int32_t t = (int32_t)(uint32_t)e[b];
      int64_t c = b;
      while (c < ne && e[c] == e[b]) ++c;
      int64_t cnt = c - b;
      if (policy == 0) {
        if (cnt > best_c) { best_c = cnt; best_t = t; } /* t ascending: ties keep lowest */
      } else {
        float xx = mean0[s] - mean0[t];
        float d2 = xx * xx + xx * xx;
        if (d2 < best_d) { best_d = d2; best_t = t; }
      }
      b = c;
    }
    map[s] = best_t;
    a = b;
  }
  /* mutual pairs: the smaller id joins the larger */
  int32_t* fixed = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  for (int64_t s = 0; s < n; ++s) {
    int32_t t = map[s];
    fixed[s] = (map[t] == s && s > t) ? (int32_t)s : t;
  }
  /* every segment follows its chain to the end (map_until_converged.cuh:
   * 14-31); ends already found are remembered (done[] marks them), so each
   * chain link is walked once */
  int rc = 0;
  unsigned char* done = (unsigned char*)calloc((size_t)n, 1);
  int32_t* path = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  for (int64_t s = 0; s < n && !rc; ++s) {
    if (done[s]) continue;
    int64_t len = 0;
    int32_t r = (int32_t)s;
    while (!done[r] && fixed[r] != r) {
      path[len++] = r;
      r = fixed[r];
      if (len > n) { rc = 3; break; }
    }
    if (rc) break;
    const int32_t end = done[r] ? map[r] : r;
    if (!done[r]) { map[r] = r; done[r] = 1; }
    for (int64_t i = 0; i < len; ++i) { map[path[i]] = end; done[path[i]] = 1; }
  }
  free(done);
  free(path);
  for (int64_t i = 0; i < n; ++i) out[i] = map[in[i]];
  free(fixed);
  free(e);
  free(size);
  free(map);
  free(mean0);
  return rc;
}

/* ------------------------------------------------------------------------ */
/* erosion                                                                  */
/* ------------------------------------------------------------------------ */

/* Square (2r+1)^2 erosion of every label's mask with the image border as
 * background; eroded pixels become -1.  Restates split/src/split/device/morph/
 * erode.cu:57-159 (a vertical then a horizontal run shrink by r on each side;
 * a pixel survives iff its window lies inside the image and holds one label).
 * r >= 1. */
ORC_API int orc_erode(const int32_t* in, int width, int height, int r,
                      int32_t* out) {
  if (width <= 0 || height <= 0 || r < 1) return 1;
  for (int y = 0; y < height; ++y)
    for (int x = 0; x < width; ++x) {
      int32_t v = in[(int64_t)y * width + x];
      int keep = (x >= r && y >= r && x + r < width && y + r < height);
      for (int yy = y - r; keep && yy <= y + r; ++yy)
        for (int xx = x - r; keep && xx <= x + r; ++xx)
          keep = in[(int64_t)yy * width + xx] == v;
      out[(int64_t)y * width + x] = keep ? v : -1;
    }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Sobel normals                                                            */
/* ------------------------------------------------------------------------ */

/* Restates split/src/split/device/sfs/sobel_normals.cu:16-119 and
 * detail/normalize_vectors.cu:15-41 in double precision:
 *   S(x, y)  = h(x-1, y) + 2 h(x, y) + h(x+1, y), zero beyond the row ends
 *   Gy(x, y) = S(x, min(y+1, H-1)) - S(x, max(y-1, 0))
 *   T(x, y)  = h(x, y-1) + 2 h(x, y) + h(x, y+1), zero beyond the column ends
 *   Gx(x, y) = T(min(x+1, W-1), y) - T(max(x-1, 0), y)
 *   n = (Gx, Gy, 1 / max(0.001, depth)) / |.|, with z <- |z|.
 * Output planar 3 x n (x, y, z rows). */
static double hv(const float* h, int w, int x, int y) {
  return (double)h[(int64_t)y * w + x];
}

ORC_API int orc_sobel_normals_f64(const float* h, int width, int height,
                                  float depth, double* out) {
  if (width <= 0 || height <= 0) return 1;
  const int64_t n = (int64_t)width * height;
  const double z = 1.0 / (double)fmaxf(0.001f, depth);
  for (int y = 0; y < height; ++y)
    for (int x = 0; x < width; ++x) {
      int yb = y + 1 < height ? y + 1 : height - 1;
      int yt = y > 0 ? y - 1 : 0;
      double sb = 2.0 * hv(h, width, x, yb), st = 2.0 * hv(h, width, x, yt);
      if (x > 0) { sb += hv(h, width, x - 1, yb); st += hv(h, width, x - 1, yt); }
      if (x + 1 < width) { sb += hv(h, width, x + 1, yb); st += hv(h, width, x + 1, yt); }
      double gy = sb - st;
      int xr = x + 1 < width ? x + 1 : width - 1;
      int xl = x > 0 ? x - 1 : 0;
      double tr = 2.0 * hv(h, width, xr, y), tl = 2.0 * hv(h, width, xl, y);
      if (y > 0) { tr += hv(h, width, xr, y - 1); tl += hv(h, width, xl, y - 1); }
      if (y + 1 < height) { tr += hv(h, width, xr, y + 1); tl += hv(h, width, xl, y + 1); }
      double gx = tr - tl;
      double m = sqrt(gx * gx + gy * gy + z * z);
      int64_t i = (int64_t)y * width + x;
      out[i] = gx / m;
      out[n + i] = gy / m;
      out[2 * n + i] = fabs(z) / m;
    }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* feature preparation                                                      */
/* ------------------------------------------------------------------------ */

/* Luminance (L-star / 100) of RGB8 pixels in double precision.  Restates the sample's
 * feature preparation: clamp channels to >= 1/255 (samples/src/main.cu:
 * 170-173), sRGB -> XYZ (split/include/split/device/color/detail/
 * conversion.inl:8-25), XYZ -> L* (conversion.inl:46-64), L* row kept as the
 * luminance plane (main.cu:221-223). */
ORC_API void orc_luminance_f64(const uint8_t* rgb, int64_t n, double* lum) {
  for (int64_t i = 0; i < n; ++i) {
    double lin[3];
    for (int c = 0; c < 3; ++c) {
      double v = (double)rgb[3 * i + c] / 255.0;
      if (v < 1.0 / 255.0) v = 1.0 / 255.0;
      lin[c] = (v > 0.04045 ? pow((v + 0.055) / 1.055, 2.4) : v / 12.92) * 100.0;
    }
    double Y = lin[0] * 0.2126729 + lin[1] * 0.7151522 + lin[2] * 0.0721750;
    double y = Y * 0.01;
    double fy = y > 0.008856 ? cbrt(y) : 7.787 * y + 16.0 / 116.0;
    lum[i] = (116.0 * fy - 16.0) / 100.0;
  }
}

/* ------------------------------------------------------------------------ */
/* smooth-boundary merge                                                     */
/* ------------------------------------------------------------------------ */
/* Restates the documented behaviour of split/src/split/device/ccl/
 * merge_smooth_boundaries.cu:134-243 (the file itself does not compile: its
 * reduce_by_key is given thrust::less as the reduction):
 *   directed 8-neighbour edges between different labels, image border
 *   excluded (segment_adjacency.cu:112-142, :170-254); per pair (s, t) the
 *   edge count and the mean of |x_p - x_q| over feature rows 0..2 (FP32
 *   norm, VecNorm :25-35); pairs with mean >= D = threshold * max_i |x_i|
 *   (:193-195) or with at most 15 edges (:197-205) dropped; each segment maps
 *   to its candidate with the smallest (mean, id) (:207-226); mutual pairs
 *   keep the larger id (fix_map_cycles.cuh:14-44); labels follow their chains
 *   (map_until_converged.cuh:14-31).
 * The pair sums are formed like the CUDA path's: every edge norm rounded to
 * a multiple of 2^-32 and summed as an integer, the mean in double, rounded
 * to float.  Sequential, sort-based.  Labels must lie in [0, w * h). */
typedef struct {
  int32_t s, t;
  long long q;
} SmEdge;

static int sm_cmp(const void* a, const void* b) {
  const SmEdge* x = (const SmEdge*)a;
  const SmEdge* y = (const SmEdge*)b;
  if (x->s != y->s) return x->s < y->s ? -1 : 1;
  if (x->t != y->t) return x->t < y->t ? -1 : 1;
  return 0;
}

static float sm_norm(const float* pts, int64_t n, int64_t p, int64_t q) {
  float s = 0.0f;
  for (int d = 0; d < 3; ++d) {
    const float v = pts[d * n + p] - pts[d * n + q];
    s = s + v * v;
  }
  return sqrtf(s);
}

ORC_API int orc_merge_smooth(int32_t* labels, int width, int height, const float* pts,
                             float threshold) {
  const int64_t n = (int64_t)width * height;
  SmEdge* e = (SmEdge*)malloc(sizeof(SmEdge) * (size_t)(8 * n + 1));
  int32_t* map = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  float* bestd = (float*)malloc(sizeof(float) * (size_t)n);
  int32_t* bestt = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  if (!e || !map || !bestd || !bestt) {
    free(e); free(map); free(bestd); free(bestt);
    return 2;
  }
  for (int64_t i = 0; i < n; ++i)
    if (labels[i] < 0 || labels[i] >= n) {
      free(e); free(map); free(bestd); free(bestt);
      return 1;
    }
  /* threshold */
  float maxsq = 0.0f;
  for (int64_t i = 0; i < n; ++i) {
    float s = 0.0f;
    for (int d = 0; d < 3; ++d) s = s + pts[d * n + i] * pts[d * n + i];
    if (s > maxsq) maxsq = s;
  }
  const float D = threshold * sqrtf(maxsq);
  /* edges */
  int64_t ne = 0;
  for (int y = 0; y < height; ++y)
    for (int x = 0; x < width; ++x) {
      const int64_t p = (int64_t)y * width + x;
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          if (!dx && !dy) continue;
          const int nx = x + dx, ny = y + dy;
          if (nx < 0 || ny < 0 || nx >= width || ny >= height) continue;
          const int64_t q = (int64_t)ny * width + nx;
          if (labels[q] == labels[p]) continue;
          e[ne].s = labels[p];
          e[ne].t = labels[q];
          e[ne].q = llrintf(sm_norm(pts, n, p, q) * 4294967296.0f);
          ++ne;
        }
    }
  qsort(e, (size_t)ne, sizeof(SmEdge), sm_cmp);
  for (int64_t i = 0; i < n; ++i) {
    map[i] = (int32_t)i;
    bestt[i] = -1;
  }
  for (int64_t a = 0; a < ne;) {
    int64_t b = a;
    long long sum = 0;
    while (b < ne && e[b].s == e[a].s && e[b].t == e[a].t) sum += e[b++].q;
    const int64_t cnt = b - a;
    const float mean = (float)(((double)sum * (1.0 / 4294967296.0)) / (double)cnt);
    const int s = e[a].s, t = e[a].t;
    if (mean < D && cnt > 15) {
      if (bestt[s] < 0 || mean < bestd[s] || (mean == bestd[s] && t < bestt[s])) {
        bestd[s] = mean;
        bestt[s] = t;
      }
    }
    a = b;
  }
  for (int64_t s = 0; s < n; ++s)
    if (bestt[s] >= 0) map[s] = bestt[s];
  /* mutual pairs: the larger id keeps itself */
  for (int64_t s = 0; s < n; ++s) {
    const int32_t t = map[s];
    if (t != s && map[t] == s && s > t) map[s] = (int32_t)s;
  }
  /* chains */
  for (int64_t i = 0; i < n; ++i) {
    int32_t r = labels[i];
    for (int64_t steps = 0; map[r] != r && steps <= n; ++steps) r = map[r];
    labels[i] = r;
  }
  free(e); free(map); free(bestd); free(bestt);
  return 0;
}
