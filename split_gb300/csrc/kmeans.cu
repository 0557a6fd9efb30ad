// k-means for the segmentation path: assignment over packed or planar pixel
// features with the centroids in shared memory, and a deterministic FP32
// centroid update, fused in one persistent cooperative kernel per call.
//
// Restates split/src/split/device/kmeans/{cluster,label,centroids,
// propagation}.cu (see the per-function notes) without the N x K distance
// matrix, the radix sort per iteration or the host round trip per iteration.
//
// Work decomposition (fixed per image, so a result never depends on what else
// shares the launch): an image is cut into units of kUnit pixels; units are
// grouped kGroup at a time.  Blocks take units from a device work counter.
// Per unit, every warp accumulates (x - c_label) over its 32-pixel batches in
// a warp-private shared-memory slot (warp butterfly sums per distinct label),
// the block sums the 8 warp slots in warp order and writes the unit partial.
// The last block to finish a unit of a group sums the group's unit partials in
// unit order; the last block to finish a group of an image sums the group
// partials in group order and forms c_new = c + S / n.  All sums therefore
// have one fixed shape: the update is bit-reproducible.
#include <limits.h>
#include <math.h>

#include "common.cuh"

namespace sg {
namespace km {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kUnit = 8192;            // pixels per unit
constexpr int kWarpSpan = kUnit / kWarps;  // 1024 pixels per warp per unit
constexpr int kGroup = 32;             // units per group
constexpr int kMaxK = 64;
constexpr int kMaxDim = 5;
// partial record: kMaxK * kMaxDim float sums then kMaxK int counts
constexpr int kRec = kMaxK * kMaxDim + kMaxK;

enum Mode { kCluster = 0, kUpdateOnly = 1, kAssignOnly = 2 };

struct Image {
  const void* points;
  int unit_range;           // colour features known to lie in [0, 1]
  int64_t npoints;
  int width;
  float xy_scale;
  float* centroids;         // user array, dim x K planar (in/out)
  int32_t* labels;          // output labels (cluster / assign modes)
  const int32_t* labels_in; // update-only mode
  int K;
  int max_iter;
  float threshold;
  int32_t* d_iterations;
  int unit_begin;
  int nunits;
  int group_begin;
  int ngroups;
};

struct ImageState {
  float delta;
  float old_delta;
  int iters;
  int done;
};

struct Params {
  Image img0;            // used when nimages == 1
  const Image* images;   // device array when nimages > 1
  int nimages;
  int total_units;
  int max_iter;
  float* unit_part;      // [total_units][kRec]
  float* group_part;     // [total_groups][kRec]
  float* cur;            // [2][nimages][kMaxK * 8]
  unsigned* group_cnt;   // [total_groups]
  unsigned* image_cnt;   // [nimages]
  ImageState* state;     // [nimages]
  WsHeader* hdr;
};

constexpr int cstride(int dim) { return dim == 3 ? 4 : 8; }

__device__ __forceinline__ const Image& image_of(const Params& p, int i) {
  return p.nimages == 1 ? p.img0 : p.images[i];
}

__device__ __forceinline__ int find_image(const Params& p, int unit) {
  if (p.nimages == 1) return 0;
  int lo = 0, hi = p.nimages - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (p.images[mid].unit_begin <= unit) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Pixel feature loader.  dim == 5 appends xy_scale * (column, row).
template <int LAYOUT, int DIM>
struct Loader {
  const void* pts;
  int64_t n;
  float xy;
  const float* lut;
  __device__ __forceinline__ void load(int64_t i, int row, int col,
                                       float (&f)[DIM]) const {
    if (LAYOUT == SPLIT_LAYOUT_PLANAR) {
      const float* p = static_cast<const float*>(pts);
#pragma unroll
      for (int d = 0; d < DIM; ++d) f[d] = __ldg(p + d * n + i);
      return;
    } else if (LAYOUT == SPLIT_LAYOUT_FLOAT4) {
      float4 v = __ldg(static_cast<const float4*>(pts) + i);
      f[0] = v.x;
      f[1] = v.y;
      f[2] = v.z;
    } else {
      const uint8_t* p = static_cast<const uint8_t*>(pts) + 3 * i;
      f[0] = lut[__ldg(p + 0)];
      f[1] = lut[__ldg(p + 1)];
      f[2] = lut[__ldg(p + 2)];
    }
    if (DIM == 5) {
      f[3] = __fmul_rn(xy, (float)col);
      f[4] = __fmul_rn(xy, (float)row);
    }
  }
};

// Order-preserving float -> int key (for warp min/max reductions).
__device__ __forceinline__ int fkey(float x) {
  const int i = __float_as_int(x);
  return i ^ ((i >> 31) & 0x7fffffff);
}
__device__ __forceinline__ float fkey_inv(int k) {
  return __int_as_float(k ^ ((k >> 31) & 0x7fffffff));
}

// Candidate clusters of a 32-pixel batch whose features lie in the box
// [lo, hi]: lane l bounds clusters l and l + 32.  For every cluster,
// LB = squared distance from the centroid to the box (a lower bound of each
// pixel's distance) and UB = squared distance to the farthest box corner (an
// upper bound).  A cluster whose LB exceeds the smallest UB by more than the
// 1e-4 relative margin is strictly farther than the winner from every pixel
// of the batch even after FP32 rounding (a few ulp), so skipping it leaves
// every argmin - ties included - unchanged.
template <int DIM>
__device__ __forceinline__ unsigned long long candidates(const float (&lo)[DIM],
                                                         const float (&hi)[DIM],
                                                         const float* __restrict__ cs, int K) {
  constexpr int CS = cstride(DIM);
  const int lane = threadIdx.x & 31;
  float lb[2], ubm = INFINITY;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int k = lane + 32 * h;
    lb[h] = INFINITY;
    if (k < K) {
      float l = 0.0f, u = 0.0f;
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        const float c = cs[k * CS + d];
        const float g = fmaxf(fmaxf(lo[d] - c, c - hi[d]), 0.0f);
        const float e = fmaxf(c - lo[d], hi[d] - c);
        l = __fmaf_rn(g, g, l);
        u = __fmaf_rn(e, e, u);
      }
      lb[h] = l;
      ubm = fminf(ubm, u);
    }
  }
  // UB >= 0: its bit pattern orders like the value
  const float ub = __int_as_float(__reduce_min_sync(0xffffffffu, __float_as_int(ubm)));
  const float thr = ub * 1.0001f;
  const unsigned m0 = __ballot_sync(0xffffffffu, lb[0] <= thr);
  const unsigned m1 = __ballot_sync(0xffffffffu, lb[1] <= thr);
  return ((unsigned long long)m1 << 32) | m0;
}

// Nearest centroid among `mask`: d = fma chain of (x - c)^2 in dimension
// order, strict < in ascending k, so ties go to the lowest k (label.cu:23-32,
// :98-105).
template <int DIM>
__device__ __forceinline__ int nearest(const float (&f)[DIM], const float* __restrict__ cs,
                                       unsigned long long mask) {
  constexpr int CS = cstride(DIM);
  float best = INFINITY;
  int bk = 0;
  while (mask) {
    const int k = __ffsll((long long)mask) - 1;
    mask &= mask - 1;
    const float4 c0 = *reinterpret_cast<const float4*>(cs + k * CS);
    float t = __fsub_rn(f[0], c0.x);
    float d = __fmul_rn(t, t);
    t = __fsub_rn(f[1], c0.y);
    d = __fmaf_rn(t, t, d);
    t = __fsub_rn(f[2], c0.z);
    d = __fmaf_rn(t, t, d);
    if (DIM == 5) {
      // dims 0..3 sit in c0 (x = column feature in c0.w), dim 4 right after
      t = __fsub_rn(f[3], c0.w);
      d = __fmaf_rn(t, t, d);
      t = __fsub_rn(f[4], cs[k * CS + 4]);
      d = __fmaf_rn(t, t, d);
    }
    if (d < best) {
      best = d;
      bk = k;
    }
  }
  return bk;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = __fadd_rn(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

constexpr int kChunk = 8;     // records summed per thread in one pass
constexpr int kChunks = 8;    // chunks per pass (64 records per pass)
constexpr int kVals = kMaxK * kMaxDim + kMaxK;

// Warp slots are double-buffered by unit parity: warp 0 reduces a finished
// unit's slots while the other warps already accumulate the next unit.
struct Smem {
  alignas(16) float cent[kMaxK * 8];
  float scratch[kChunks][kVals];
  float acc[2][kWarps][kMaxK * kMaxDim];
  int cnt[2][kWarps][kMaxK];
  float lut[256];
  int next[2];   // prefetched work-counter values
  int pend[2];   // unit whose group became complete, per buffer parity
  int flag;
};

// Advance a (row, col) pair by s pixels along the row-major order.
__device__ __forceinline__ void advance(int& row, int& col, int s, int w) {
  col += s;
  if (col >= w) {
    int q = col / w;
    row += q;
    col -= q * w;
  }
}

// ---- packed FP32x2 helpers (per-lane IEEE round-to-nearest, so results are
// bit-identical to the scalar __fsub_rn / __fmul_rn / __fmaf_rn forms)
__device__ __forceinline__ float2 fsub2(float2 a, float2 b) {
  float2 r;
  asm("{.reg .b64 a_, b_, r_;\n\t"
      "mov.b64 a_, {%2, %3};\n\tmov.b64 b_, {%4, %5};\n\t"
      "sub.rn.f32x2 r_, a_, b_;\n\tmov.b64 {%0, %1}, r_;}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
__device__ __forceinline__ float2 fmul2(float2 a, float2 b) {
  float2 r;
  asm("{.reg .b64 a_, b_, r_;\n\t"
      "mov.b64 a_, {%2, %3};\n\tmov.b64 b_, {%4, %5};\n\t"
      "mul.rn.f32x2 r_, a_, b_;\n\tmov.b64 {%0, %1}, r_;}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) {
  float2 r;
  asm("{.reg .b64 a_, b_, c_, r_;\n\t"
      "mov.b64 a_, {%2, %3};\n\tmov.b64 b_, {%4, %5};\n\tmov.b64 c_, {%6, %7};\n\t"
      "fma.rn.f32x2 r_, a_, b_, c_;\n\tmov.b64 {%0, %1}, r_;}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return r;
}

constexpr int kPx = 4;                 // consecutive pixels per lane
constexpr int kBatch = 32 * kPx;       // pixels per warp batch
static_assert(kWarpSpan % kBatch == 0, "whole batches per warp span");

// The lane's kPx consecutive pixels starting at px0 (row, col of px0).
template <int LAYOUT, int DIM>
__device__ __forceinline__ void load_px(const Image& im, const float* lut, int64_t px0, int row,
                                        int col, float (&f)[kPx][DIM], bool (&ok)[kPx]) {
  const int64_t n = im.npoints;
#pragma unroll
  for (int j = 0; j < kPx; ++j) ok[j] = px0 + j < n;
  if (LAYOUT == SPLIT_LAYOUT_FLOAT4) {
    const float4* p = static_cast<const float4*>(im.points) + px0;
#pragma unroll
    for (int j = 0; j < kPx; ++j) {
      const float4 v = ok[j] ? __ldg(p + j) : make_float4(0.f, 0.f, 0.f, 0.f);
      f[j][0] = v.x;
      f[j][1] = v.y;
      f[j][2] = v.z;
    }
  } else if (LAYOUT == SPLIT_LAYOUT_RGB8) {
    const uint8_t* p = static_cast<const uint8_t*>(im.points) + 3 * px0;
#pragma unroll
    for (int j = 0; j < kPx; ++j)
#pragma unroll
      for (int c = 0; c < 3; ++c) f[j][c] = ok[j] ? lut[__ldg(p + 3 * j + c)] : 0.0f;
  } else {
    const float* p = static_cast<const float*>(im.points);
#pragma unroll
    for (int d = 0; d < DIM; ++d)
#pragma unroll
      for (int j = 0; j < kPx; ++j) f[j][d] = ok[j] ? __ldg(p + (int64_t)d * n + px0 + j) : 0.0f;
  }
  if (DIM == 5 && LAYOUT != SPLIT_LAYOUT_PLANAR) {
    if (col + kPx <= im.width) {
      const float fy = __fmul_rn(im.xy_scale, (float)row);
#pragma unroll
      for (int j = 0; j < kPx; ++j) {
        f[j][3] = __fmul_rn(im.xy_scale, (float)(col + j));
        f[j][4] = fy;
      }
    } else {
      int r = row, c = col;
#pragma unroll
      for (int j = 0; j < kPx; ++j) {
        f[j][3] = __fmul_rn(im.xy_scale, (float)c);
        f[j][4] = __fmul_rn(im.xy_scale, (float)r);
        if (++c == im.width) {
          c = 0;
          ++r;
        }
      }
    }
  }
}

// Nearest centroid among `mask` for the lane's pixels; the distance is the
// fma chain of (x - c)^2 in dimension order, strict < in ascending k (ties to
// the lowest k; label.cu:23-32, :98-105), evaluated on pixel pairs with the
// packed f32x2 pipe.
template <int DIM>
__device__ __forceinline__ void nearest_px(const float (&f)[kPx][DIM],
                                           const float* __restrict__ cs,
                                           unsigned long long mask, int (&lab)[kPx]) {
  constexpr int CS = cstride(DIM);
  float best[kPx];
#pragma unroll
  for (int j = 0; j < kPx; ++j) {
    best[j] = INFINITY;
    lab[j] = 0;
  }
  while (mask) {
    const int k = __ffsll((long long)mask) - 1;
    mask &= mask - 1;
    const float4 c0 = *reinterpret_cast<const float4*>(cs + k * CS);
    const float cc[5] = {c0.x, c0.y, c0.z, c0.w, DIM == 5 ? cs[k * CS + 4] : 0.0f};
#pragma unroll
    for (int q = 0; q < kPx / 2; ++q) {
      const int a = 2 * q, b = 2 * q + 1;
      float2 t = fsub2(make_float2(f[a][0], f[b][0]), make_float2(cc[0], cc[0]));
      float2 d = fmul2(t, t);
#pragma unroll
      for (int dd = 1; dd < DIM; ++dd) {
        t = fsub2(make_float2(f[a][dd], f[b][dd]), make_float2(cc[dd], cc[dd]));
        d = ffma2(t, t, d);
      }
      if (d.x < best[a]) {
        best[a] = d.x;
        lab[a] = k;
      }
      if (d.y < best[b]) {
        best[b] = d.y;
        lab[b] = k;
      }
    }
  }
}

// Warp-collective: add the per-lane sums `acc` (label l, warp-uniform) to the
// warp's shared slot.
template <int DIM>
__device__ __forceinline__ void flush_acc(Smem& sm, int buf, int warp, int l,
                                          const float (&acc)[DIM], int n) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    const float s = warp_sum(acc[d]);
    if (lane == 0)
      sm.acc[buf][warp][l * kMaxDim + d] = __fadd_rn(sm.acc[buf][warp][l * kMaxDim + d], s);
  }
  const int c = __reduce_add_sync(0xffffffffu, n);
  if (lane == 0) sm.cnt[buf][warp][l] += c;
}

// Process one unit: assign (unless update-only) and accumulate per-warp sums
// of (x - c_label).  Each lane holds kPx consecutive pixels of a 128-pixel
// warp batch.  While consecutive batches carry one label, every lane keeps a
// register running sum; a batch with several labels is reduced label by label
// in ascending order.  All orders depend only on the data.
template <int LAYOUT, int DIM, int MODE>
__device__ void process_unit(const Image& im, int unit, Smem& sm, int buf, bool write_labels) {
  const unsigned full = 0xffffffffu;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int CS = cstride(DIM);
  if (MODE != kAssignOnly) {
    // this warp's slot of buffer `buf` (read by warp 0 two units ago)
    for (int i = lane; i < im.K * kMaxDim; i += 32) sm.acc[buf][warp][i] = 0.0f;
    for (int i = lane; i < im.K; i += 32) sm.cnt[buf][warp][i] = 0;
    __syncwarp();
  }
  int64_t px0 = (int64_t)unit * kUnit + (int64_t)warp * kWarpSpan + (int64_t)lane * kPx;
  int row = 0, col = 0;
  if (DIM == 5 && LAYOUT != SPLIT_LAYOUT_PLANAR) {
    row = (int)(px0 / im.width);
    col = (int)(px0 - (int64_t)row * im.width);
  }
  const bool vec_labels = (reinterpret_cast<uintptr_t>(MODE == kUpdateOnly ? im.labels_in : im.labels) & 15) == 0;
  int acc_l = -1, acc_n = 0;
  float acc[DIM];
#pragma unroll
  for (int d = 0; d < DIM; ++d) acc[d] = 0.0f;

  for (int b = 0; b < kWarpSpan / kBatch; ++b, px0 += kBatch) {
    if (b > 0 && DIM == 5 && LAYOUT != SPLIT_LAYOUT_PLANAR) advance(row, col, kBatch, im.width);
    if (__all_sync(full, px0 >= im.npoints)) break;
    float f[kPx][DIM];
    bool ok[kPx];
    load_px<LAYOUT, DIM>(im, sm.lut, px0, row, col, f, ok);
    const bool all_ok = ok[kPx - 1];
    int lab[kPx];
    if (MODE == kUpdateOnly) {
      if (all_ok && vec_labels) {
        const int4 v = __ldg(reinterpret_cast<const int4*>(im.labels_in + px0));
        lab[0] = v.x; lab[1] = v.y; lab[2] = v.z; lab[3] = v.w;
      } else {
#pragma unroll
        for (int j = 0; j < kPx; ++j) lab[j] = ok[j] ? __ldg(im.labels_in + px0 + j) : -1;
      }
#pragma unroll
      for (int j = 0; j < kPx; ++j)
        if (!ok[j] || lab[j] < 0 || lab[j] >= im.K) lab[j] = -1;
    } else {
      // Bounding box of the batch, then the candidate clusters.  fminf /
      // fmaxf skip NaN: a NaN pixel gets label 0 whatever the mask (every
      // distance compares false), and the box still bounds all other pixels.
      float lo[DIM], hi[DIM];
      constexpr bool kXY = DIM == 5 && LAYOUT != SPLIT_LAYOUT_PLANAR;
      constexpr int kBoxDims = kXY ? 3 : DIM;
      const bool warp_all_ok = __all_sync(full, all_ok);
      const bool unit = LAYOUT == SPLIT_LAYOUT_RGB8 || (LAYOUT == SPLIT_LAYOUT_FLOAT4 && im.unit_range);
#pragma unroll
      for (int d = 0; d < kBoxDims; ++d) {
        if (unit && d < 3) {
          lo[d] = 0.0f;
          hi[d] = 1.0f;
          continue;
        }
        float a, z;
        if (warp_all_ok) {
          a = fminf(fminf(f[0][d], f[1][d]), fminf(f[2][d], f[3][d]));
          z = fmaxf(fmaxf(f[0][d], f[1][d]), fmaxf(f[2][d], f[3][d]));
        } else {
          a = INFINITY;
          z = -INFINITY;
#pragma unroll
          for (int j = 0; j < kPx; ++j) {
            if (ok[j]) {
              a = fminf(a, f[j][d]);
              z = fmaxf(z, f[j][d]);
            }
          }
        }
        lo[d] = fkey_inv(__reduce_min_sync(full, fkey(a)));
        hi[d] = fkey_inv(__reduce_max_sync(full, fkey(z)));
      }
      if (kXY) {
        // the batch's pixels are consecutive: lane 0 holds the first, lane 31
        // the last; a batch that wraps a row spans whole columns
        const int r0 = __shfl_sync(full, row, 0), c0 = __shfl_sync(full, col, 0);
        const int64_t last = min(px0 - (int64_t)lane * kPx + kBatch, im.npoints) - 1;
        const int64_t first = px0 - (int64_t)lane * kPx;
        const int c1 = c0 + (int)(last - first);
        if (c1 < im.width) {
          lo[3] = __fmul_rn(im.xy_scale, (float)c0);
          hi[3] = __fmul_rn(im.xy_scale, (float)c1);
          lo[4] = hi[4] = __fmul_rn(im.xy_scale, (float)r0);
        } else {
          const int r1 = (int)(last / im.width);
          lo[3] = 0.0f;
          hi[3] = __fmul_rn(im.xy_scale, (float)(im.width - 1));
          lo[4] = __fmul_rn(im.xy_scale, (float)r0);
          hi[4] = __fmul_rn(im.xy_scale, (float)r1);
        }
      }
      const unsigned long long mask = candidates<DIM>(lo, hi, sm.cent, im.K);
      nearest_px<DIM>(f, sm.cent, mask, lab);
      if (write_labels) {
        if (all_ok && vec_labels) {
          *reinterpret_cast<int4*>(im.labels + px0) = make_int4(lab[0], lab[1], lab[2], lab[3]);
        } else {
#pragma unroll
          for (int j = 0; j < kPx; ++j)
            if (ok[j]) im.labels[px0 + j] = lab[j];
        }
      }
#pragma unroll
      for (int j = 0; j < kPx; ++j)
        if (!ok[j]) lab[j] = -1;
    }
    if (MODE == kAssignOnly) continue;

    // ---- accumulate x - c_label
    int mn = INT_MAX, mx = -1;
#pragma unroll
    for (int j = 0; j < kPx; ++j) {
      if (lab[j] >= 0) {
        mn = min(mn, lab[j]);
        mx = max(mx, lab[j]);
      }
    }
    mn = __reduce_min_sync(full, mn);
    mx = __reduce_max_sync(full, mx);
    if (mx < 0) continue;
    if (mn == mx) {
      if (mn != acc_l) {
        if (acc_l >= 0) flush_acc<DIM>(sm, buf, warp, acc_l, acc, acc_n);
        acc_l = mn;
        acc_n = 0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) acc[d] = 0.0f;
      }
      float c[DIM];
#pragma unroll
      for (int d = 0; d < DIM; ++d) c[d] = sm.cent[mn * CS + d];
#pragma unroll
      for (int j = 0; j < kPx; ++j) {
        if (lab[j] >= 0) {
#pragma unroll
          for (int d = 0; d < DIM; ++d) acc[d] = __fadd_rn(acc[d], __fsub_rn(f[j][d], c[d]));
          ++acc_n;
        }
      }
    } else {
      if (acc_l >= 0) flush_acc<DIM>(sm, buf, warp, acc_l, acc, acc_n);
      acc_l = -1;
      for (int l = mn; l != INT_MAX;) {
        float s[DIM];
        int c = 0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) s[d] = 0.0f;
        int nxt = INT_MAX;
#pragma unroll
        for (int j = 0; j < kPx; ++j) {
          if (lab[j] == l) {
#pragma unroll
            for (int d = 0; d < DIM; ++d) s[d] = __fadd_rn(s[d], __fsub_rn(f[j][d], sm.cent[l * CS + d]));
            ++c;
          } else if (lab[j] > l) {
            nxt = min(nxt, lab[j]);
          }
        }
        flush_acc<DIM>(sm, buf, warp, l, s, c);
        l = __reduce_min_sync(full, nxt);
      }
    }
  }
  if (MODE != kAssignOnly && acc_l >= 0) flush_acc<DIM>(sm, buf, warp, acc_l, acc, acc_n);
}

// Warp 0: sum the 8 warp slots of buffer `buf` in warp order into a unit
// record.
__device__ __forceinline__ void warp_to_record(const Smem& sm, int buf, float* rec, int K,
                                               int dim) {
  const int lane = threadIdx.x & 31;
  for (int idx = lane; idx < K * kMaxDim; idx += 32) {
    if ((idx % kMaxDim) >= dim) continue;
    float s = 0.0f;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) s = __fadd_rn(s, sm.acc[buf][w][idx]);
    __stcg(rec + idx, s);
  }
  for (int k = lane; k < K; k += 32) {
    int c = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) c += sm.cnt[buf][w][k];
    __stcg(reinterpret_cast<int*>(rec + kMaxK * kMaxDim) + k, c);
  }
}

// Sum `count` records (stride kRec) into `out` with one fixed shape: records
// are summed 8 at a time in order (all 8 loads in flight), the chunk sums of a
// pass are then summed in chunk order, and the passes in pass order.  Value v
// enumerates the K*dim float sums followed by the K counts.
__device__ void sum_records(Smem& sm, const float* src, int count, float* out,
                            int K, int dim) {
  const int nv = K * dim + K;
  for (int pass0 = 0; pass0 < count; pass0 += kChunk * kChunks) {
    const int in_pass = min(count - pass0, kChunk * kChunks);
    const int nch = (in_pass + kChunk - 1) / kChunk;
    __syncthreads();
    for (int w = threadIdx.x; w < nv * nch; w += blockDim.x) {
      const int v = w % nv, c = w / nv;
      const int r0 = pass0 + c * kChunk;
      const int rn = min(kChunk, count - r0);
      const bool is_cnt = v >= K * dim;
      const int off = is_cnt ? kMaxK * kMaxDim + (v - K * dim)
                             : (v / dim) * kMaxDim + (v % dim);
      const float* s = src + (size_t)r0 * kRec + off;
      float x[kChunk];
#pragma unroll
      for (int r = 0; r < kChunk; ++r) x[r] = r < rn ? __ldcg(s + (size_t)r * kRec) : 0.0f;
      if (is_cnt) {
        int a = 0;
#pragma unroll
        for (int r = 0; r < kChunk; ++r) a += __float_as_int(x[r]);
        sm.scratch[c][v] = __int_as_float(a);
      } else {
        float a = x[0];
#pragma unroll
        for (int r = 1; r < kChunk; ++r) a = __fadd_rn(a, x[r]);
        sm.scratch[c][v] = a;
      }
    }
    __syncthreads();
    for (int v = threadIdx.x; v < nv; v += blockDim.x) {
      const bool is_cnt = v >= K * dim;
      const int off = is_cnt ? kMaxK * kMaxDim + (v - K * dim)
                             : (v / dim) * kMaxDim + (v % dim);
      if (is_cnt) {
        int a = pass0 ? __float_as_int(__ldcg(out + off)) : 0;
        for (int c = 0; c < nch; ++c) a += __float_as_int(sm.scratch[c][v]);
        __stcg(reinterpret_cast<int*>(out + off), a);
      } else {
        float a = sm.scratch[0][v];
        for (int c = 1; c < nch; ++c) a = __fadd_rn(a, sm.scratch[c][v]);
        if (pass0) a = __fadd_rn(__ldcg(out + off), a);
        __stcg(out + off, a);
      }
    }
  }
  __syncthreads();
}

template <int DIM>
__device__ __forceinline__ void load_centroids(const float* src, int K,
                                               float* cent) {
  constexpr int CS = cstride(DIM);
  for (int idx = threadIdx.x; idx < K * CS; idx += blockDim.x) {
    const int k = idx / CS, d = idx % CS;
    cent[idx] = d < DIM ? __ldcg(src + k * 8 + d) : 0.0f;
  }
}

// Image-level finish: new centroids c + S / n (empty cluster: unchanged),
// convergence test of cluster.cu:71-88, outputs on the last iteration.
template <int DIM, int MODE>
__device__ void finish_image(const Params& p, int img, const Image& im, int it,
                             const float* total) {
  __shared__ float sdelta;
  const float* c_old = p.cur + ((size_t)(it & 1) * p.nimages + img) * (kMaxK * 8);
  float* c_new = p.cur + ((size_t)((it + 1) & 1) * p.nimages + img) * (kMaxK * 8);
  const int* cnt = reinterpret_cast<const int*>(total + kMaxK * kMaxDim);
  __shared__ float sdiff[kMaxK * kMaxDim];
  for (int idx = threadIdx.x; idx < im.K * DIM; idx += blockDim.x) {
    const int k = idx / DIM, d = idx % DIM;
    const float c = __ldcg(c_old + k * 8 + d);
    const int n = __ldcg(cnt + k);
    float cn = c;
    if (n > 0) cn = __fadd_rn(c, __fdiv_rn(__ldcg(total + k * kMaxDim + d), (float)n));
    __stcg(c_new + k * 8 + d, cn);
    const float df = __fsub_rn(cn, c);
    sdiff[idx] = __fmul_rn(df, df);
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    // squared centroid shift, summed in a fixed order
    float acc = 0.0f;
    for (int idx = threadIdx.x; idx < im.K * DIM; idx += 32) acc = __fadd_rn(acc, sdiff[idx]);
    acc = warp_sum(acc);
    if (threadIdx.x == 0) sdelta = acc;
  }
  __syncthreads();
  __shared__ int sdone;
  if (threadIdx.x == 0) {
    // state is shared across blocks: volatile accesses bypass the
    // incoherent L1
    volatile ImageState* vs = p.state + img;
    const int iters = vs->iters + 1;
    const float old_delta = vs->delta;
    const float delta = sqrtf(sdelta);
    bool more = iters < im.max_iter && fabsf(delta - old_delta) > im.threshold;
    if (MODE == kUpdateOnly) more = false;
    vs->old_delta = old_delta;
    vs->delta = delta;
    vs->iters = iters;
    vs->done = more ? 0 : 1;
    sdone = more ? 0 : 1;
    if (im.d_iterations && !more) *im.d_iterations = iters;
  }
  __syncthreads();
  // final centroids back to the caller's planar array
  if (sdone) {
    for (int idx = threadIdx.x; idx < im.K * DIM; idx += blockDim.x) {
      const int k = idx / DIM, d = idx % DIM;
      im.centroids[d * im.K + k] = __ldcg(c_new + k * 8 + d);
    }
  }
}

// Sums the group of unit u (whose last unit just completed); the last group
// of the image then forms the image total and the new centroids.
template <int DIM, int MODE>
__device__ void group_task(const Params& p, Smem& sm, int u, int it) {
  const int img = find_image(p, u);
  const Image& im = image_of(p, img);
  const int lu = u - im.unit_begin;
  const int g = lu / kGroup;
  const int gbeg = g * kGroup;
  const int gcount = min(kGroup, im.nunits - gbeg);
  __threadfence();
  float* grec = p.group_part + (size_t)(im.group_begin + g) * kRec;
  sum_records(sm, p.unit_part + (size_t)(im.unit_begin + gbeg) * kRec, gcount, grec, im.K, DIM);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned prev = atomicAdd(&p.image_cnt[img], 1u);
    sm.flag = (prev == (unsigned)im.ngroups - 1);
    if (sm.flag) p.image_cnt[img] = 0;
  }
  __syncthreads();
  if (!sm.flag) return;
  __threadfence();
  // image total into the record slot of the image's first unit (its partial
  // was consumed by the first group's sum)
  float* tot = p.unit_part + (size_t)im.unit_begin * kRec;
  sum_records(sm, p.group_part + (size_t)im.group_begin * kRec, im.ngroups, tot, im.K, DIM);
  __threadfence();
  __syncthreads();
  finish_image<DIM, MODE>(p, img, im, it, tot);
  __syncthreads();
}

template <int LAYOUT, int DIM, int MODE>
__global__ void __launch_bounds__(kThreads, 4) kmeans_kernel(Params p) {
  __shared__ Smem sm;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (LAYOUT == SPLIT_LAYOUT_RGB8)
    for (int i = threadIdx.x; i < 256; i += blockDim.x) sm.lut[i] = (float)i / 255.0f;

  for (int it = 0; it < p.max_iter; ++it) {
    unsigned* counter = &p.hdr->work_counter[it & 1];
    if (threadIdx.x == 0) {
      if (blockIdx.x == 0) p.hdr->work_counter[(it + 1) & 1] = 0;
      sm.next[0] = (int)atomicAdd(counter, 1u);
      sm.pend[0] = sm.pend[1] = -1;
    }
    __syncthreads();
    int cached = -1, npar = 0, buf = 0;
    int raw = sm.next[0];
    while (raw < p.total_units) {
      // odd iterations walk the units backwards: they start on the units the
      // previous iteration touched last, which are still resident in L2
      const int u = (it & 1) ? p.total_units - 1 - raw : raw;
      const int img = find_image(p, u);
      const Image& im = image_of(p, img);
      if (threadIdx.x == 0) sm.next[npar ^ 1] = (int)atomicAdd(counter, 1u);
      if (MODE != kAssignOnly && *(volatile int*)&p.state[img].done) {
        __syncthreads();
        raw = sm.next[npar ^ 1];
        npar ^= 1;
        continue;
      }
      if (img != cached) {
        // every warp is past the previous unit (its end-of-unit barrier)
        if (MODE == kAssignOnly)
          load_centroids<DIM>(p.cur + (size_t)img * (kMaxK * 8), im.K, sm.cent);
        else
          load_centroids<DIM>(p.cur + ((size_t)(it & 1) * p.nimages + img) * (kMaxK * 8),
                              im.K, sm.cent);
        cached = img;
        __syncthreads();
      }
      const int lu = u - im.unit_begin;
      const bool wl = (MODE == kAssignOnly) ||
                      (MODE == kCluster && (im.threshold >= 0.0f || it == im.max_iter - 1));
      process_unit<LAYOUT, DIM, MODE>(im, lu, sm, buf, wl);
      __syncthreads();  // the unit's slots are complete; next[] and pend[] visible
      raw = sm.next[npar ^ 1];
      npar ^= 1;
      if (MODE == kAssignOnly) continue;
      const int task = sm.pend[buf ^ 1];
      if (task >= 0) {
        group_task<DIM, MODE>(p, sm, task, it);
        if (threadIdx.x == 0) sm.pend[buf ^ 1] = -1;
      }
      if (warp == 0) {
        warp_to_record(sm, buf, p.unit_part + (size_t)u * kRec, im.K, DIM);
        __threadfence();
        __syncwarp();
        if (lane == 0) {
          const int g = lu / kGroup;
          const int gcount = min(kGroup, im.nunits - g * kGroup);
          const unsigned prev = atomicAdd(&p.group_cnt[im.group_begin + g], 1u);
          if (prev == (unsigned)gcount - 1) {
            p.group_cnt[im.group_begin + g] = 0;
            sm.pend[buf] = u;
          }
        }
      }
      buf ^= 1;
    }
    if (MODE == kAssignOnly) break;
    __syncthreads();
    const int task = sm.pend[buf ^ 1];
    if (task >= 0) group_task<DIM, MODE>(p, sm, task, it);
    if (!grid_barrier(p.hdr)) return;
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

struct Layout {
  float* unit_part;
  float* group_part;
  float* cur;
  unsigned* group_cnt;
  unsigned* image_cnt;
  ImageState* state;
  Image* images;
  WsHeader* hdr;
  size_t bytes;
};

inline int units_of(int64_t n) { return (int)((n + kUnit - 1) / kUnit); }
inline int groups_of(int units) { return (units + kGroup - 1) / kGroup; }

static Layout carve(void* ws, int total_units, int total_groups, int nimages) {
  Carver c(ws);
  Layout l;
  l.hdr = c.take<WsHeader>(1);
  l.unit_part = c.take<float>((size_t)total_units * kRec);
  l.group_part = c.take<float>((size_t)total_groups * kRec);
  l.cur = c.take<float>((size_t)2 * nimages * kMaxK * 8);
  l.group_cnt = c.take<unsigned>((size_t)total_groups);
  l.image_cnt = c.take<unsigned>((size_t)nimages);
  l.state = c.take<ImageState>((size_t)nimages);
  l.images = nimages > 1 ? c.take<Image>((size_t)nimages) : nullptr;
  l.bytes = c.size();
  return l;
}

// Per-image iteration state (cluster.cu:65-68: delta = 0, old_delta =
// delta + threshold + 1, so the first convergence test always passes).
__global__ void init_kernel(Params p) {
  for (int img = blockIdx.x * blockDim.x + threadIdx.x; img < p.nimages;
       img += gridDim.x * blockDim.x) {
    const Image& im = image_of(p, img);
    ImageState st;
    st.delta = 0.0f;
    st.old_delta = st.delta + im.threshold + 1.0f;
    st.iters = 0;
    st.done = im.max_iter <= 0;
    p.state[img] = st;
    if (im.d_iterations && st.done) *im.d_iterations = 0;
  }
}

template <int DIM>
__global__ void load_user_centroids(Params p) {
  for (int img = blockIdx.x; img < p.nimages; img += gridDim.x) {
    const Image& im = image_of(p, img);
    float* c0 = p.cur + (size_t)img * (kMaxK * 8);
    for (int idx = threadIdx.x; idx < im.K * DIM; idx += blockDim.x) {
      const int k = idx / DIM, d = idx % DIM;
      c0[k * 8 + d] = im.centroids[d * im.K + k];
    }
  }
}

template <int LAYOUT, int DIM, int MODE>
static int launch(Params& p, cudaStream_t st) {
  DeviceInfo di;
  SG_TRY(device_info(&di));
  auto kern = kmeans_kernel<LAYOUT, DIM, MODE>;
  int per_sm = 0;
  SG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, 0));
  if (per_sm < 1) return SPLIT_ERR_UNSUPPORTED;
  int grid = di.sm_count * per_sm;
  if (grid > p.total_units) grid = p.total_units > 0 ? p.total_units : 1;
  if (MODE == kAssignOnly) {
    kern<<<grid, kThreads, 0, st>>>(p);
    return launch_status();
  }
  void* args[] = {&p};
  SG_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)kern, dim3(grid), dim3(kThreads),
                                          args, 0, st));
  return launch_status();
}

template <int MODE>
static int dispatch(int layout, int dim, Params& p, cudaStream_t st) {
#define SG_KM_CASE(L, D) \
  if (layout == L && dim == D) return launch<L, D, MODE>(p, st);
  SG_KM_CASE(SPLIT_LAYOUT_PLANAR, 3)
  SG_KM_CASE(SPLIT_LAYOUT_PLANAR, 5)
  SG_KM_CASE(SPLIT_LAYOUT_FLOAT4, 3)
  SG_KM_CASE(SPLIT_LAYOUT_FLOAT4, 5)
  SG_KM_CASE(SPLIT_LAYOUT_RGB8, 3)
  SG_KM_CASE(SPLIT_LAYOUT_RGB8, 5)
#undef SG_KM_CASE
  return SPLIT_ERR_INVALID;
}

static bool valid_features(const void* points, int layout, int dim, int64_t n,
                           int width, int K) {
  layout &= ~SPLIT_FEATURES_UNIT_RANGE;
  if (!points || n <= 0 || n > 0x7fffffffLL || K < 1 || K > kMaxK) return false;
  if (dim != 3 && dim != 5) return false;
  if (layout < SPLIT_LAYOUT_PLANAR || layout > SPLIT_LAYOUT_RGB8) return false;
  if (width < 1) return false;
  if (layout == SPLIT_LAYOUT_FLOAT4 && (reinterpret_cast<uintptr_t>(points) & 15)) return false;
  return true;
}

static int run(int mode, const void* points, int layout, int dim, int64_t n,
               int width, float xy_scale, float* centroids,
               const float* centroids_in, int K, int32_t* labels,
               const int32_t* labels_in, void* ws, size_t ws_bytes, int max_iter,
               float threshold, int32_t* d_iter, cudaStream_t st) {
  if (!valid_features(points, layout, dim, n, width, K)) return SPLIT_ERR_INVALID;
  const int unit_range = (layout & SPLIT_FEATURES_UNIT_RANGE) ? 1 : 0;
  layout &= ~SPLIT_FEATURES_UNIT_RANGE;
  const int units = units_of(n), groups = groups_of(units);
  Layout l = carve(nullptr, units, groups, 1);
  if (!ws || ws_bytes < l.bytes || (reinterpret_cast<uintptr_t>(ws) & 255))
    return SPLIT_ERR_WORKSPACE;
  l = carve(ws, units, groups, 1);
  Params p{};
  Image& im = p.img0;
  im.points = points;
  im.unit_range = unit_range;
  im.npoints = n;
  im.width = width;
  im.xy_scale = xy_scale;
  im.centroids = centroids;
  im.labels = labels;
  im.labels_in = labels_in;
  im.K = K;
  im.max_iter = max_iter;
  im.threshold = threshold;
  im.d_iterations = d_iter;
  im.unit_begin = 0;
  im.nunits = units;
  im.group_begin = 0;
  im.ngroups = groups;
  p.nimages = 1;
  p.images = nullptr;
  p.total_units = units;
  p.max_iter = max_iter;
  p.unit_part = l.unit_part;
  p.group_part = l.group_part;
  p.cur = l.cur;
  p.group_cnt = l.group_cnt;
  p.image_cnt = l.image_cnt;
  p.state = l.state;
  p.hdr = l.hdr;
  // header words used by the barrier and the work counters start at zero
  SG_CUDA_TRY(cudaMemsetAsync(reinterpret_cast<char*>(l.hdr) + sizeof(int), 0,
                              sizeof(unsigned) * 4, st));
  (void)centroids_in;
  init_kernel<<<1, 256, 0, st>>>(p);
  SG_TRY(launch_status());
  if (dim == 3) load_user_centroids<3><<<1, 256, 0, st>>>(p);
  else load_user_centroids<5><<<1, 256, 0, st>>>(p);
  SG_TRY(launch_status());
  if (max_iter <= 0) return SPLIT_OK;
  if (mode == kCluster) return dispatch<kCluster>(layout, dim, p, st);
  if (mode == kUpdateOnly) return dispatch<kUpdateOnly>(layout, dim, p, st);
  return dispatch<kAssignOnly>(layout, dim, p, st);
}

}  // namespace km
}  // namespace sg

using namespace sg;

extern "C" size_t split_kmeans_cluster_workspace_size(int64_t npoints, int nclusters, int dim) {
  (void)nclusters;
  (void)dim;
  if (npoints <= 0) return 0;
  const int u = km::units_of(npoints);
  return km::carve(nullptr, u, km::groups_of(u), 1).bytes;
}

extern "C" int split_kmeans_cluster(const void* points, int layout, int dim, int64_t npoints,
                                    int width, float xy_scale, float* centroids, int nclusters,
                                    int32_t* labels, void* workspace, size_t workspace_bytes,
                                    int max_iter, float threshold, int32_t* d_iterations,
                                    void* stream) {
  if (!centroids || !labels) return SPLIT_ERR_INVALID;
  return km::run(km::kCluster, points, layout, dim, npoints, width, xy_scale, centroids,
                 centroids, nclusters, labels, nullptr, workspace, workspace_bytes, max_iter,
                 threshold, d_iterations, as_stream(stream));
}

extern "C" size_t split_kmeans_assign_workspace_size(int64_t npoints, int nclusters) {
  return split_kmeans_cluster_workspace_size(npoints, nclusters, 5);
}

extern "C" int split_kmeans_assign(const void* points, int layout, int dim, int64_t npoints,
                                   int width, float xy_scale, const float* centroids,
                                   int nclusters, int32_t* labels, void* workspace,
                                   size_t workspace_bytes, void* stream) {
  if (!centroids || !labels) return SPLIT_ERR_INVALID;
  return km::run(km::kAssignOnly, points, layout, dim, npoints, width, xy_scale,
                 const_cast<float*>(centroids), centroids, nclusters, labels, nullptr,
                 workspace, workspace_bytes, 1, -1.0f, nullptr, as_stream(stream));
}

extern "C" size_t split_kmeans_update_workspace_size(int64_t npoints, int nclusters, int dim) {
  return split_kmeans_cluster_workspace_size(npoints, nclusters, dim);
}

extern "C" int split_kmeans_update(const int32_t* labels, const void* points, int layout,
                                   int dim, int64_t npoints, int width, float xy_scale,
                                   float* centroids, int nclusters, void* workspace,
                                   size_t workspace_bytes, void* stream) {
  if (!centroids || !labels) return SPLIT_ERR_INVALID;
  return km::run(km::kUpdateOnly, points, layout, dim, npoints, width, xy_scale, centroids,
                 centroids, nclusters, nullptr, labels, workspace, workspace_bytes, 1, -1.0f,
                 nullptr, as_stream(stream));
}

namespace {
__global__ void propagate_kernel(const int32_t* __restrict__ labels, int64_t n,
                                 const float* __restrict__ cent, int K, int dim,
                                 float* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int l = __ldg(labels + i);
    const bool ok = l >= 0 && l < K;
    for (int d = 0; d < dim; ++d) out[d * n + i] = ok ? __ldg(cent + d * K + l) : 0.0f;
  }
}
}  // namespace

extern "C" int split_kmeans_propagate(const int32_t* labels, int64_t npoints,
                                      const float* centroids, int nclusters, int dim,
                                      float* out, void* stream) {
  if (!labels || !centroids || !out || npoints <= 0 || nclusters < 1 || dim < 1)
    return SPLIT_ERR_INVALID;
  DeviceInfo di;
  SG_TRY(device_info(&di));
  int64_t blocks = (npoints + 255) / 256;
  const int64_t cap = (int64_t)di.sm_count * 8;
  if (blocks > cap) blocks = cap;
  propagate_kernel<<<(int)blocks, 256, 0, as_stream(stream)>>>(labels, npoints, centroids,
                                                                nclusters, dim, out);
  return launch_status();
}
