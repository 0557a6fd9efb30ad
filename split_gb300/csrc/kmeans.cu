// k-means for the segmentation path: assignment over packed or planar pixel
// features with the centroids in shared memory, and a deterministic FP32
// centroid update, fused in one persistent cooperative kernel per call.
//
// Restates split/src/split/device/kmeans/{cluster,label,centroids,
// propagation}.cu (see the per-function notes) without the N x K distance
// matrix, the radix sort per iteration or the host round trip per iteration.
//
// Work decomposition (fixed per image, so a result never depends on what else
// shares the launch): an image is cut into units (tiles of 16, 32, 64 or 128
// rows by 64 columns), a unit into warp spans (each warp's rows of it).
// Every warp accumulates (x - c_label) over its span's pixel batches in FP32
// registers and a warp-private shared-memory slot (warp butterfly sums per
// distinct label); at the end of the span the slots are rounded to multiples
// of 2^-24 and added, as integers, into the block's shared sums
// (warp_to_fix).  A span whose candidate mask names one cluster adds the
// exact integer sum of its pixels' features instead (add_span_sums).  The
// block adds its integer sums into per-image accumulators as 96-bit fixed
// point (64-bit atomics on a low and a high word).  Integer addition does not
// depend on order, so the image total is the same whatever blocks took which
// spans and whatever else shares the launch.
//
// Iterations: the first (and every iteration of a batch, of a workspace
// without room for kept sums) goes by units taken from a device work counter.
// The first iteration keeps every fast span's exact feature sum; later
// iterations of a single image go by spans (span_iteration), where a span
// with one candidate needs none of its pixels.  The grid barrier that ends
// the iteration publishes the sums; then c_new = c + S / n is formed in FP32
// from the exact sum (form_centroids): for a single image by every block from
// the same inputs (bit-identical), block 0 publishing it; in a batch by one
// owner block per image, published before a second grid barrier.  The sums
// are kept in three slots by iteration, so the owner can clear the slot of
// the iteration after next while the current slot fills and the last one is
// read.
#include <limits.h>
#include <math.h>
#include <string.h>

#include <atomic>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "f32x2.cuh"
#include "fixsum.cuh"

namespace sg {
namespace km {

// Resident blocks per SM the register budget is set for.  Single images: 2
// (up to 128 registers a thread) keeps the span passes free of spills; at 3
// (80 registers) they spill, and small images, whose iterations are
// latency-bound, lose more than the extra occupancy gives.  Batches (many
// small images through the unit loop): 3, where the extra resident blocks
// hide more latency than the spills cost.
#ifndef SG_KM_MINBLOCKS
#define SG_KM_MINBLOCKS 2
#endif
constexpr int kBatchMinBlocks = 3;
constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
// A unit is a tile of unit_rows x kTile pixels (unit_rows = 16 to 128, per
// image from the tuning table); warp w owns rows [w * r, (w + 1) * r) of it,
// r = unit_rows / 8.
constexpr int kTile = 64;
constexpr int kMaxK = 64;
constexpr int kMaxDim = 5;
constexpr int kSpanSums = 8;   // words of a span's entry in Image::span_sum (kMaxDim used)
constexpr int kHeavyCap = 256; // deferred spans a block lists per iteration
// Span sums are added into the image accumulators as multiples of 2^-24; a
// span's FP32 sum must stay below 2^38 in magnitude (a span holds at most
// 1024 pixels, so |x - c| below 2.6e8 everywhere).  Beyond it the call
// reports SPLIT_ERR_OVERFLOW.
constexpr float kFixScale = 16777216.0f;   // 2^24
constexpr float kFixLimit = 274877906944.0f;   // 2^38

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
  int height;               // rows (ceil(npoints / width))
  int ntx;                  // tiles per row of tiles
  int unit_rows;            // rows of a unit (kTile or 2 * kTile, from the tuning table)
  int ref_shift;            // SPLIT_KMEANS_REFERENCE_SHIFT (D = 3, K >= 3)
  // Exact feature sums of the fast spans (kSpanSums words each), written in
  // the first iteration of a call (null: none kept).  A fast span's slot is
  // (first row / span rows) * span_cols + tile column.
  long long* span_sum;
  int span_cols;            // width / kTile: tile columns of full width
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
  // sums of iteration i live in slot i % 3 (see form_centroids)
  unsigned long long* acc_lo;  // [3][nimages][kMaxK * kMaxDim] low 32-bit words of the sums
  unsigned long long* acc_hi;  // [3][nimages][kMaxK * kMaxDim] high words (signed)
  unsigned* acc_cnt;           // [3][nimages][kMaxK] member counts
  float* cur;                  // [2][nimages][kMaxK * 8]: centroids of iteration i in i & 1
  ImageState* state;     // [2][nimages]: state after iteration i - 1 in slot i & 1
  WsHeader* hdr;
  int blocks_per_sm;     // 0: as many as fit (host side only)
  // grid barriers: polls before a wait gives up, and a block that leaves
  // without arriving (-1: none); see split_kmeans_set_wait_test
  unsigned wait_limit;
  int wait_skip;
};

constexpr int cstride(int dim) { return dim == 3 ? 4 : 8; }

__device__ __forceinline__ const Image& image_of(const Params& p, int i) {
  return p.images ? p.images[i] : p.img0;
}

__device__ __forceinline__ size_t acc_slot(const Params& p, int slot, int img) {
  return (size_t)slot * p.nimages + img;
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
    // a slot past K compares false even against an infinite thr (a box
    // with an infinite feature)
    lb[h] = __int_as_float(0x7fffffff);
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

struct Smem {
  alignas(16) float cent[kMaxK * 8];
  float acc[kWarps][kMaxK * kMaxDim];
  int cnt[kWarps][kMaxK];
  // the sums of the spans processed since the last flush, in fixed point
  // (each span's converted on its own, then added as integers)
  long long fix[kMaxK * kMaxDim];
  int fixn[kMaxK];
  // spans deferred to the second pass of an iteration (see kmeans_kernel)
  int heavy[kHeavyCap];
  int nheavy;
  int next_heavy;
  float lut[256];
  int next[2];
  int more;
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

// acc[d] += x[d] - c[d] for every dimension, in IEEE single precision: the
// pairs (0, 1) and (3, 4) on the packed pipe (per-lane results, the same bits
// as the scalar operations).
template <int DIM>
__device__ __forceinline__ void add_centered(const float (&x)[DIM], const float* c,
                                             float (&acc)[DIM]) {
  const float2 a01 = fadd2(make_float2(acc[0], acc[1]),
                           fsub2(make_float2(x[0], x[1]), make_float2(c[0], c[1])));
  acc[0] = a01.x;
  acc[1] = a01.y;
  acc[2] = __fadd_rn(acc[2], __fsub_rn(x[2], c[2]));
  if (DIM == 5) {
    constexpr int X = DIM == 5 ? 3 : 0, Y = DIM == 5 ? 4 : 0;
    const float2 a34 = fadd2(make_float2(acc[X], acc[Y]),
                             fsub2(make_float2(x[X], x[Y]), make_float2(c[X], c[Y])));
    acc[X] = a34.x;
    acc[Y] = a34.y;
  }
}

constexpr int kPx = 4;                 // consecutive pixels per lane
constexpr int kLanesPerRow = kTile / kPx;  // 16 lanes cover a tile row
constexpr int kBatchRows = 32 / kLanesPerRow;
static_assert((kTile / kWarps) % kBatchRows == 0, "whole batches per warp span");

// The lane's kPx consecutive pixels of image row `row` starting at column
// `col`; ok[j] marks pixels inside the image.
template <int LAYOUT, int DIM>
__device__ __forceinline__ void load_px(const Image& im, const float* lut, int row, int col,
                                        float (&f)[kPx][DIM], bool (&ok)[kPx]) {
  const int64_t n = im.npoints;
  const int64_t px0 = (int64_t)row * im.width + col;
#pragma unroll
  for (int j = 0; j < kPx; ++j) ok[j] = row < im.height && col + j < im.width && px0 + j < n;
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
    const float fy = __fmul_rn(im.xy_scale, (float)row);
#pragma unroll
    for (int j = 0; j < kPx; ++j) {
      f[j][3] = __fmul_rn(im.xy_scale, (float)(col + j));
      f[j][4] = fy;
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
  // ascending k over the two 32-bit halves of the mask
  unsigned m = (unsigned)mask, hi = (unsigned)(mask >> 32);
  int base = 0;
  for (;;) {
    if (!m) {
      if (!hi) break;
      m = hi;
      hi = 0;
      base = 32;
    }
    const int k = base + __ffs(m) - 1;
    m &= m - 1;
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
__device__ __forceinline__ void flush_acc(Smem& sm, int warp, int l, const float (&acc)[DIM],
                                          int n) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    const float s = warp_sum(acc[d]);
    if (lane == 0) sm.acc[warp][l * kMaxDim + d] = __fadd_rn(sm.acc[warp][l * kMaxDim + d], s);
  }
  const int c = __reduce_add_sync(0xffffffffu, n);
  if (lane == 0) sm.cnt[warp][l] += c;
}

// The end of a span: the warp's FP32 sums (its slots, one per label it met)
// rounded to fixed point and added into the block's integer sums, the slots
// cleared.  Each span's sums are converted on their own, so the totals do not
// depend on which block or pass took the span, nor in what order.
template <int DIM>
__device__ __forceinline__ void warp_to_fix(Smem& sm, int warp, int K, int* status) {
  __syncwarp();   // lane 0's slot updates are visible to the warp
  for (int k = threadIdx.x & 31; k < K; k += 32) {
    const int c = sm.cnt[warp][k];
    if (c == 0) continue;
    sm.cnt[warp][k] = 0;
    atomicAdd(&sm.fixn[k], c);
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const float v = sm.acc[warp][k * kMaxDim + d];
      if (v == 0.0f) continue;
      sm.acc[warp][k * kMaxDim + d] = 0.0f;
      if (!(fabsf(v) < kFixLimit)) set_status(status, SPLIT_ERR_OVERFLOW);
      atomicAdd(reinterpret_cast<unsigned long long*>(&sm.fix[k * kMaxDim + d]),
                (unsigned long long)__float2ll_rn(__fmul_rn(v, kFixScale)));
    }
  }
  __syncwarp();
}

// Accumulate one batch whose kPx labels are all valid: the same sums, in the
// same order, as the general path below.
template <int DIM>
__device__ __forceinline__ void accumulate_valid(Smem& sm, int warp, const float (&f)[kPx][DIM],
                                                 const int (&lab)[kPx], int& acc_l, int& acc_n,
                                                 float (&acc)[DIM]) {
  const unsigned full = 0xffffffffu;
  constexpr int CS = cstride(DIM);
  int mn = min(min(lab[0], lab[1]), min(lab[2], lab[3]));
  int mx = max(max(lab[0], lab[1]), max(lab[2], lab[3]));
  mn = __reduce_min_sync(full, mn);
  mx = __reduce_max_sync(full, mx);
  if (mn == mx) {
    if (mn != acc_l) {
      if (acc_l >= 0) flush_acc<DIM>(sm, warp, acc_l, acc, acc_n);
      acc_l = mn;
      acc_n = 0;
#pragma unroll
      for (int d = 0; d < DIM; ++d) acc[d] = 0.0f;
    }
    float c[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) c[d] = sm.cent[mn * CS + d];
#pragma unroll
    for (int j = 0; j < kPx; ++j) add_centered<DIM>(f[j], c, acc);
    acc_n += kPx;
    return;
  }
  if (acc_l >= 0) flush_acc<DIM>(sm, warp, acc_l, acc, acc_n);
  acc_l = -1;
  for (int l = mn; l != INT_MAX;) {
    float sum[DIM];
    int c = 0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) sum[d] = 0.0f;
    int nxt = INT_MAX;
#pragma unroll
    for (int j = 0; j < kPx; ++j) {
      if (lab[j] == l) {
        add_centered<DIM>(f[j], sm.cent + l * CS, sum);
        ++c;
      } else if (lab[j] > l) {
        nxt = min(nxt, lab[j]);
      }
    }
    flush_acc<DIM>(sm, warp, l, sum, c);
    l = __reduce_min_sync(full, nxt);
  }
}

// ---- asynchronous copies into shared memory (no registers hold the data)
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
// Staging of the float4 fast path: per warp two batches of kPx x 32 float4,
// pixel j of lane l at [j][l] (conflict-free copies and reads).
constexpr int kStageFloat4 = kWarps * 2 * 4 * 32;   // float4 elements per block
constexpr size_t kStageBytes = (size_t)kStageFloat4 * 16;

// Labels of the lane's pixels when the candidates are exactly ka < kb: the
// same distances, in the same order and with the same comparisons, as
// nearest_px over a two-bit mask.
template <int DIM>
__device__ __forceinline__ void nearest_pair(const float (&f)[kPx][DIM],
                                             const float* __restrict__ cs, int ka, int kb,
                                             int (&lab)[kPx]) {
  constexpr int CS = cstride(DIM);
  float best[kPx];
#pragma unroll
  for (int j = 0; j < kPx; ++j) {
    best[j] = INFINITY;
    lab[j] = 0;
  }
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int k = h ? kb : ka;
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

// Labels of a whole fast span set to k (lane rows and columns as in a batch).
__device__ __forceinline__ void write_span_labels(const Image& im, int row_first, int col,
                                                  int nbatches, int k, bool vec_labels) {
  const int64_t step = (int64_t)kBatchRows * im.width;
  int64_t px0 = (int64_t)row_first * im.width + col;
  for (int b = 0; b < nbatches; ++b, px0 += step) {
    if (vec_labels) {
      *reinterpret_cast<int4*>(im.labels + px0) = make_int4(k, k, k, k);
    } else {
#pragma unroll
      for (int j = 0; j < kPx; ++j) im.labels[px0 + j] = k;
    }
  }
}

// Adds a single-candidate span's pixels to cluster k's sums of the unit, as
// the exact fixed-point sum of (x - c_k): S (the span's exact feature words,
// lane d holding dimension d) minus n * c_k * 2^24 (exact in FP64, rounded
// once).  The same integers whether S was just summed from the pixels or
// kept from the first iteration, so a call's result does not depend on
// which; integer adds, so not on their order either.
template <int DIM>
__device__ __forceinline__ void add_span_sums(Smem& sm, int k, long long s_lane, int n) {
  constexpr int CS = cstride(DIM);
  const int lane = threadIdx.x & 31;
  if (lane < DIM) {
    const double nc = __dmul_rn((double)n, __dmul_rn((double)sm.cent[k * CS + lane], 16777216.0));
    atomicAdd(reinterpret_cast<unsigned long long*>(&sm.fix[k * kMaxDim + lane]),
              (unsigned long long)(s_lane - __double2ll_rn(nc)));
  } else if (lane == DIM) {
    atomicAdd(&sm.fixn[k], n);
  }
}

// Exact feature words of a span (2^-24 units): colour from the lanes' pixel
// sums `qc`, the xy features from the geometry (each lane's kPx columns in
// every batch row it covers); summed over the warp, lane d returns
// dimension d.
template <int DIM>
__device__ __forceinline__ long long span_words(const long long (&qc)[3], const float (&fx)[kPx],
                                                float xy_scale, int row_first, int nbatches) {
  const int lane = threadIdx.x & 31;
  long long w[DIM];
  w[0] = qc[0];
  w[1] = qc[1];
  w[2] = qc[2];
  if (DIM == 5) {
    long long qx = 0, qy = 0;
#pragma unroll
    for (int j = 0; j < kPx; ++j) qx += __float2ll_rn(__fmul_rn(fx[j], kFixScale));
    for (int b = 0; b < nbatches; ++b)
      qy += __float2ll_rn(
          __fmul_rn(__fmul_rn(xy_scale, (float)(row_first + b * kBatchRows)), kFixScale));
    w[DIM == 5 ? 3 : 0] = qx * nbatches;
    w[DIM == 5 ? 4 : 0] = qy * kPx;
  }
  long long mine = 0;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      w[d] += (long long)__shfl_xor_sync(0xffffffffu, (unsigned long long)w[d], o);
    if (lane == d) mine = w[d];
  }
  return mine;
}

// How a span's candidate mask is used: one cluster (every pixel's label
// outright), two clusters with finite centroids (two running sums per lane),
// or any other mask (per-batch reduction by label).
enum SpanKind { kSpanSingle = 0, kSpanPair = 1, kSpanAny = 2 };

// The batches of a fast span (see fast_span).  For kSpanPair every pixel's
// label is ka or kb (finite features and centroids), so `acc` runs for ka
// and a second per-lane sum for kb, reduced once at the end of the span
// however often the two labels mix within its batches.
//
// A single-candidate span of a clustering adds its pixels' exact feature
// words instead of running FP32 sums, and keeps them in `entry` (if any);
// any other span given an `entry` (the first iteration's) also sums and keeps
// its words, besides its FP32 sums.
template <int LAYOUT, int DIM, int MODE, int KIND>
__device__ __forceinline__ void span_batches(const Image& im, Smem& sm, int warp, int row_first,
                                             int col, int nbatches, unsigned long long mask,
                                             int ka, int kb, bool write_labels, bool vec_labels,
                                             int& acc_l, int& acc_n, float (&acc)[DIM],
                                             long long* entry) {
  constexpr int CS = cstride(DIM);
  constexpr bool kFixSingle = KIND == kSpanSingle && MODE == kCluster;
  // the first iteration also keeps the words of spans with several candidates
  const bool keep = MODE == kCluster && KIND != kSpanSingle && entry != nullptr;
  long long qc[3] = {0, 0, 0};
  const int64_t step = (int64_t)kBatchRows * im.width;
  int64_t px0 = (int64_t)row_first * im.width + col;
  float acc2[DIM];
  int acc2_n = 0;
  if (KIND == kSpanPair) {
#pragma unroll
    for (int d = 0; d < DIM; ++d) acc2[d] = 0.0f;
  }
  float fx[kPx];
#pragma unroll
  for (int j = 0; j < kPx; ++j) fx[j] = __fmul_rn(im.xy_scale, (float)(col + j));
  // float4: the next batch is copied into shared memory while this one runs.
  // Lane l copies batch pixels l + 32 j (each copy a contiguous 512 bytes of
  // one row) and reads its own pixels 4 l + j; slots are swizzled so that
  // both are free of bank conflicts.
  extern __shared__ float4 km_stage[];
  const int ln = threadIdx.x & 31;
  float4* stage = km_stage + warp * (2 * kPx * 32);
  const int64_t gw = (int64_t)im.width;
  // batch pixel q = 64 r + c of the batch's first row (row_first - lrow)
  const float4* gb0 = static_cast<const float4*>(im.points) + (px0 - (int64_t)(ln / kLanesPerRow) * gw
                                                               - (ln % kLanesPerRow) * kPx);
  // slot(q) = (q & ~7) | ((q + (q >> 3)) & 7), in closed form for the lane's
  // copies (q = ln + 32 j) and reads (q = 4 ln + j)
  const int cs0 = (ln & ~7) + ((ln + (ln >> 3)) & 7), cs1 = cs0 ^ 4;
  const int rs0 = 8 * (ln >> 1), rt = (4 * ln + (ln >> 1)) & 7;
  const float4* grow1 = gb0 + gw;
  if (LAYOUT == SPLIT_LAYOUT_FLOAT4) {
    cp_async16(stage + cs0, gb0 + ln);
    cp_async16(stage + 32 + cs1, gb0 + ln + 32);
    cp_async16(stage + 64 + cs0, grow1 + ln);
    cp_async16(stage + 96 + cs1, grow1 + ln + 32);
    cp_async_commit();
  }
  for (int b = 0; b < nbatches; ++b, px0 += step) {
    float f[kPx][DIM];
    if (LAYOUT == SPLIT_LAYOUT_FLOAT4) {
      // every lane has read the buffer about to be refilled (batch b - 1)
      __syncwarp();
      if (b + 1 < nbatches) {
        const float4* g = gb0 + (int64_t)(b + 1) * step + ln;
        float4* dst = stage + ((b + 1) & 1) * (kPx * 32);
        cp_async16(dst + cs0, g);
        cp_async16(dst + 32 + cs1, g + 32);
        cp_async16(dst + 64 + cs0, g + gw);
        cp_async16(dst + 96 + cs1, g + gw + 32);
        cp_async_commit();
        cp_async_wait<1>();
      } else {
        cp_async_wait<0>();
      }
      // the copies of the other lanes must have landed too
      __syncwarp();
      const float4* src = stage + (b & 1) * (kPx * 32);
#pragma unroll
      for (int j = 0; j < kPx; ++j) {
        const float4 v = src[rs0 + ((rt + j) & 7)];
        f[j][0] = v.x;
        f[j][1] = v.y;
        f[j][2] = v.z;
      }
    } else {
      const uint32_t* p =
          reinterpret_cast<const uint32_t*>(static_cast<const uint8_t*>(im.points) + 3 * px0);
      const uint32_t w[3] = {__ldg(p), __ldg(p + 1), __ldg(p + 2)};
#pragma unroll
      for (int j = 0; j < kPx; ++j)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const int byte = 3 * j + c;
          f[j][c] = sm.lut[(w[byte >> 2] >> (8 * (byte & 3))) & 0xffu];
        }
    }
    if (DIM == 5) {
      const float fy = __fmul_rn(im.xy_scale, (float)(row_first + b * kBatchRows));
#pragma unroll
      for (int j = 0; j < kPx; ++j) {
        f[j][3] = fx[j];
        f[j][4] = fy;
      }
    }
    if (kFixSingle || keep) {
#pragma unroll
      for (int j = 0; j < kPx; ++j)
#pragma unroll
        for (int c = 0; c < 3; ++c) qc[c] += __float2int_rn(__fmul_rn(f[j][c], kFixScale));
    }
    int lab[kPx];
    if (KIND == kSpanSingle) {
      // one candidate for the whole span: every pixel's argmin, no distances
#pragma unroll
      for (int j = 0; j < kPx; ++j) lab[j] = ka;
    } else if (KIND == kSpanPair) {
      nearest_pair<DIM>(f, sm.cent, ka, kb, lab);
    } else {
      nearest_px<DIM>(f, sm.cent, mask, lab);
    }
    if (write_labels) {
      if (vec_labels) {
        *reinterpret_cast<int4*>(im.labels + px0) = make_int4(lab[0], lab[1], lab[2], lab[3]);
      } else {
#pragma unroll
        for (int j = 0; j < kPx; ++j) im.labels[px0 + j] = lab[j];
      }
    }
    if (MODE != kAssignOnly) {
      if (KIND == kSpanSingle) {
        // a clustering's single spans are summed exactly (after the loop)
        if (!kFixSingle) {
          const float* c = sm.cent + ka * CS;
#pragma unroll
          for (int j = 0; j < kPx; ++j) add_centered<DIM>(f[j], c, acc);
          acc_n += kPx;
        }
      } else if (KIND == kSpanPair) {
        const float* ca = sm.cent + ka * CS;
        const float* cb = sm.cent + kb * CS;
#pragma unroll
        for (int j = 0; j < kPx; ++j) {
          if (lab[j] == ka) {
            add_centered<DIM>(f[j], ca, acc);
            ++acc_n;
          } else {
            add_centered<DIM>(f[j], cb, acc2);
            ++acc2_n;
          }
        }
      } else {
        accumulate_valid<DIM>(sm, warp, f, lab, acc_l, acc_n, acc);
      }
    }
  }
  // the second candidate's sums (the first's stay running)
  if (MODE != kAssignOnly && KIND == kSpanPair) flush_acc<DIM>(sm, warp, kb, acc2, acc2_n);
  if (kFixSingle || keep) {
    const long long w = span_words<DIM>(qc, fx, im.xy_scale, row_first, nbatches);
    if (entry && (threadIdx.x & 31) < DIM) __stcg(entry + (threadIdx.x & 31), w);
    if (kFixSingle) add_span_sums<DIM>(sm, ka, w, 32 * kPx * nbatches);
  }
}


// A warp span that lies wholly inside the image, with packed features (float4,
// or RGB8 read as three 32-bit words per 4 pixels) and a candidate mask known
// for the whole span: no per-pixel bounds checks, one pointer step per batch,
// the column feature hoisted.  Results equal the general path's labels; the
// sums are the same pixels' in a fixed, data-dependent order.
//
// In a clustering, `entry` is the span's slot of kept feature words (or
// null).  Iteration 0 writes it for every span; in later iterations a span
// with one candidate reads it back instead of its pixels: its labels are
// that candidate's (written when asked) and its sums are exact integers, so
// nothing else needs the pixels.
template <int LAYOUT, int DIM, int MODE>
__device__ __forceinline__ void fast_span(const Image& im, Smem& sm, int warp, int row_first,
                                          int col, int nbatches, unsigned long long mask,
                                          bool write_labels, bool vec_labels, int& acc_l,
                                          int& acc_n, float (&acc)[DIM], long long* entry,
                                          int it) {
  constexpr int CS = cstride(DIM);
  // A mask with one cluster names every pixel's nearest centroid outright:
  // the span's box excludes all others for every pixel it holds (and the
  // features of this path lie in the unit cube, so none is NaN).
  int kind = kSpanAny, ka = -1, kb = -1;
  if (mask != 0ull && (mask & (mask - 1ull)) == 0ull) {
    kind = kSpanSingle;
    ka = __ffsll((long long)mask) - 1;
  } else if (MODE != kAssignOnly && __popcll((long long)mask) == 2) {
    const int a = __ffsll((long long)mask) - 1, b = 63 - __clzll((long long)mask);
    bool fin = true;
#pragma unroll
    for (int d = 0; d < DIM; ++d)
      fin = fin && isfinite(sm.cent[a * CS + d]) && isfinite(sm.cent[b * CS + d]);
    if (fin) {
      kind = kSpanPair;
      ka = a;
      kb = b;
    }
  }
  if (MODE == kCluster && kind == kSpanSingle && entry && it > 0) {
    const int lane = threadIdx.x & 31;
    add_span_sums<DIM>(sm, ka, lane < DIM ? __ldcg(entry + lane) : 0ll, 32 * kPx * nbatches);
    if (write_labels) write_span_labels(im, row_first, col, nbatches, ka, vec_labels);
    return;
  }
  // with one running label for the whole span the sums switch to it once
  // (a clustering sums its single spans exactly instead)
  if (MODE != kAssignOnly && ka >= 0 && ka != acc_l && !(MODE == kCluster && kind == kSpanSingle)) {
    if (acc_l >= 0) flush_acc<DIM>(sm, warp, acc_l, acc, acc_n);
    acc_l = ka;
    acc_n = 0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) acc[d] = 0.0f;
  }
  if (kind == kSpanSingle)
    span_batches<LAYOUT, DIM, MODE, kSpanSingle>(im, sm, warp, row_first, col, nbatches, mask, ka,
                                                 kb, write_labels, vec_labels, acc_l, acc_n, acc,
                                                 entry);
  else if (kind == kSpanPair)
    span_batches<LAYOUT, DIM, MODE, kSpanPair>(im, sm, warp, row_first, col, nbatches, mask, ka,
                                               kb, write_labels, vec_labels, acc_l, acc_n, acc,
                                               it == 0 ? entry : nullptr);
  else
    span_batches<LAYOUT, DIM, MODE, kSpanAny>(im, sm, warp, row_first, col, nbatches, mask, ka,
                                              kb, write_labels, vec_labels, acc_l, acc_n, acc,
                                              it == 0 ? entry : nullptr);
}

// Whether a warp span takes the fast path: xy features with colour known to
// lie in [0, 1], the whole span inside the image, and (RGB8) 4-pixel-aligned
// rows.  It depends only on the geometry and the layout, so a span is fast in
// every iteration or in none.
template <int LAYOUT, int DIM, int MODE>
__device__ __forceinline__ bool fast_geometry(const Image& im, int row0, int col0, int wrows,
                                              bool vec_labels) {
  constexpr bool kXY = DIM == 5 && LAYOUT != SPLIT_LAYOUT_PLANAR;
  const bool unit_box = kXY && (LAYOUT == SPLIT_LAYOUT_RGB8 || im.unit_range);
  return MODE != kUpdateOnly && unit_box && row0 + wrows <= im.height &&
         col0 + kTile <= im.width &&
         (LAYOUT == SPLIT_LAYOUT_FLOAT4 ||
          (LAYOUT == SPLIT_LAYOUT_RGB8 && vec_labels &&
           (reinterpret_cast<uintptr_t>(im.points) & 3) == 0));
}

// The candidate mask of a span with xy features and colour in [0, 1]: the
// box is exact without the pixels.
template <int DIM>
__device__ __forceinline__ unsigned long long unit_box_mask(const Image& im, const Smem& sm,
                                                            int row0, int col0, int rows_in,
                                                            int cols_in) {
  float lo[DIM], hi[DIM];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    lo[d] = 0.0f;
    hi[d] = 1.0f;
  }
  lo[DIM == 5 ? 3 : 0] = __fmul_rn(im.xy_scale, (float)col0);
  hi[DIM == 5 ? 3 : 0] = __fmul_rn(im.xy_scale, (float)(col0 + cols_in - 1));
  lo[DIM == 5 ? 4 : 0] = __fmul_rn(im.xy_scale, (float)row0);
  hi[DIM == 5 ? 4 : 0] = __fmul_rn(im.xy_scale, (float)(row0 + rows_in - 1));
  return candidates<DIM>(lo, hi, sm.cent, im.K);
}

// One warp span: rows srow * wrows .. + wrows of tile column tx (wrows =
// unit_rows / kWarps; a unit, a 64-column tile of unit_rows rows, is the
// spans of its kWarps warps): assign (unless update-only) and accumulate the
// calling warp's sums of (x - c_label).  A batch is 2 rows x 64 columns, each
// lane holding kPx consecutive pixels of a row.
//
// Candidate clusters: with xy features and colour features known to lie in
// [0, 1] the box of the warp's span is exact without touching the pixels, so
// one candidate mask serves all its batches.  Otherwise the colour box of
// every batch is measured (warp min / max) and joined with the batch's xy
// extent.
//
// While consecutive batches carry one label, every lane keeps a register
// running sum; a batch with several labels is reduced label by label in
// ascending order.  All orders depend only on the data.  The span's sums end
// in the block's integer sums (warp_to_fix).
template <int LAYOUT, int DIM, int MODE>
__device__ void process_span(const Image& im, int srow, int tx, Smem& sm, bool write_labels,
                             int it, int* status) {
  const unsigned full = 0xffffffffu;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int CS = cstride(DIM);
  constexpr bool kXY = DIM == 5 && LAYOUT != SPLIT_LAYOUT_PLANAR;
  const int wrows = im.unit_rows / kWarps;
  const int row0 = srow * wrows;
  const int col0 = tx * kTile;
  if (row0 >= im.height) return;
  const int lrow = lane / kLanesPerRow, lcol = (lane % kLanesPerRow) * kPx;
  const int rows_in = min(wrows, im.height - row0);
  const int cols_in = min(kTile, im.width - col0);
  const bool unit_box = kXY && (LAYOUT == SPLIT_LAYOUT_RGB8 || im.unit_range);
  const bool vec_labels =
      (reinterpret_cast<uintptr_t>(MODE == kUpdateOnly ? im.labels_in : im.labels) & 15) == 0 &&
      (im.width % kPx) == 0;
  // float4 features: any width (labels stored one by one where a row's
  // start is not 16-byte aligned); RGB8 read as 32-bit words needs
  // 4-pixel-aligned rows
  const bool fast = fast_geometry<LAYOUT, DIM, MODE>(im, row0, col0, wrows, vec_labels);
  // slot (srow, tx) of a fast span's kept sums
  long long* entry = (fast && MODE == kCluster && im.span_sum)
                         ? im.span_sum + ((size_t)srow * im.span_cols + tx) * kSpanSums
                         : nullptr;

  unsigned long long span_mask = 0;
  if (MODE != kUpdateOnly && unit_box)
    span_mask = unit_box_mask<DIM>(im, sm, row0, col0, rows_in, cols_in);

  int acc_l = -1, acc_n = 0;
  float acc[DIM];
#pragma unroll
  for (int d = 0; d < DIM; ++d) acc[d] = 0.0f;

  if (fast)
    fast_span<LAYOUT, DIM, MODE>(im, sm, warp, row0 + lrow, col0 + lcol, wrows / kBatchRows,
                                 span_mask, write_labels, vec_labels, acc_l, acc_n, acc, entry,
                                 it);
  for (int b = 0; !fast && b < wrows / kBatchRows; ++b) {
    if (b * kBatchRows >= rows_in) break;
    const int row = row0 + b * kBatchRows + lrow;
    const int col = col0 + lcol;
    float f[kPx][DIM];
    bool ok[kPx];
    load_px<LAYOUT, DIM>(im, sm.lut, row, col, f, ok);
    const bool all_ok = ok[kPx - 1];
    const int64_t px0 = (int64_t)row * im.width + col;
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
      unsigned long long mask = span_mask;
      if (!unit_box) {
        // Box of the batch.  fminf / fmaxf skip NaN: a NaN pixel gets label
        // 0 whatever the mask (every distance compares false), and the box
        // still bounds all other pixels.
        float lo[DIM], hi[DIM];
        constexpr int kBoxDims = kXY ? 3 : DIM;
#pragma unroll
        for (int d = 0; d < kBoxDims; ++d) {
          float a = INFINITY, z = -INFINITY;
#pragma unroll
          for (int j = 0; j < kPx; ++j) {
            if (ok[j]) {
              a = fminf(a, f[j][d]);
              z = fmaxf(z, f[j][d]);
            }
          }
          lo[d] = fkey_inv(__reduce_min_sync(full, fkey(a)));
          hi[d] = fkey_inv(__reduce_max_sync(full, fkey(z)));
        }
        if (kXY) {
          const int r0 = row0 + b * kBatchRows;
          lo[3] = __fmul_rn(im.xy_scale, (float)col0);
          hi[3] = __fmul_rn(im.xy_scale, (float)(col0 + cols_in - 1));
          lo[4] = __fmul_rn(im.xy_scale, (float)r0);
          hi[4] = __fmul_rn(im.xy_scale, (float)min(r0 + kBatchRows - 1, im.height - 1));
        }
        mask = candidates<DIM>(lo, hi, sm.cent, im.K);
      }
      if (unit_box && mask != 0ull && (mask & (mask - 1ull)) == 0ull) {
        // one candidate for the span names every pixel's label (features in
        // the unit cube: none is NaN), as on the fast path
        const int k1 = __ffsll((long long)mask) - 1;
#pragma unroll
        for (int j = 0; j < kPx; ++j) lab[j] = k1;
      } else {
        nearest_px<DIM>(f, sm.cent, mask, lab);
      }
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
        if (acc_l >= 0) flush_acc<DIM>(sm, warp, acc_l, acc, acc_n);
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
          add_centered<DIM>(f[j], c, acc);
          ++acc_n;
        }
      }
    } else {
      if (acc_l >= 0) flush_acc<DIM>(sm, warp, acc_l, acc, acc_n);
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
            add_centered<DIM>(f[j], sm.cent + l * CS, s);
            ++c;
          } else if (lab[j] > l) {
            nxt = min(nxt, lab[j]);
          }
        }
        flush_acc<DIM>(sm, warp, l, s, c);
        l = __reduce_min_sync(full, nxt);
      }
    }
  }
  if (MODE != kAssignOnly) {
    if (acc_l >= 0) flush_acc<DIM>(sm, warp, acc_l, acc, acc_n);
    warp_to_fix<DIM>(sm, warp, im.K, status);
  }
}

// Adds the block's integer sums into the image accumulators (96-bit fixed
// point: low 32 bits and the signed rest in two 64-bit words) and clears
// them.
__device__ void block_to_accum(Smem& sm, const Params& p, int img, int K, int dim, int slot) {
  __syncthreads();
  unsigned long long* lo = p.acc_lo + acc_slot(p, slot, img) * (kMaxK * kMaxDim);
  unsigned long long* hi = p.acc_hi + acc_slot(p, slot, img) * (kMaxK * kMaxDim);
  for (int idx = threadIdx.x; idx < K * kMaxDim; idx += blockDim.x) {
    const long long q = sm.fix[idx];
    if (q == 0) continue;
    sm.fix[idx] = 0;
    if ((idx % kMaxDim) < dim) {
      atomicAdd(lo + idx, (unsigned long long)q & 0xffffffffull);
      atomicAdd(hi + idx, (unsigned long long)(q >> 32));
    }
  }
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    const int c = sm.fixn[k];
    sm.fixn[k] = 0;
    if (c) atomicAdd(p.acc_cnt + acc_slot(p, slot, img) * kMaxK + k, (unsigned)c);
  }
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

// The squared "centroid shift" as the reference's cluster() measures it
// (cluster.cu:40-50, :73-87): it keeps the previous centroids at float
// offset 2N of its workspace, but within the same iteration label_points
// writes its N x K distance matrix from offset 0 (label.cu:80-88, entry
// i * K + c = distance of point i to centroid c, Norm2 at label.cu:23-32) and
// calculate_centroids writes its K reciprocal cluster sizes at offset 2N
// (centroids.cu:40-63).  So the words it compares the new centroids with
// (planar, entry j = d * K + k) are
//   j < K:  1 / n_j (the reciprocal size of cluster j, FP32 division);
//   j >= K: the distance of point (2N + j) / K to centroid (2N + j) % K of
//           the iteration's input, sum of squares in dimension order;
// and the shift is the FP32 sum of (c_new[j] - word[j])^2 in j order.  Only
// the reference's 3-D case is defined, and only for K >= 3 (smaller K would
// read words no call of the iteration wrote).
template <int LAYOUT, int DIM>
__device__ float reference_shift(const Image& im, const float* cent, const float* c_old,
                                 const unsigned* cnt, const float* lut) {
  constexpr int CS = cstride(DIM);
  Loader<LAYOUT, DIM> ld{im.points, im.npoints, im.xy_scale, lut};
  const int64_t base = 2 * im.npoints;
  float acc = 0.0f;
  for (int j = 0; j < im.K * 3; ++j) {
    const int d = j / im.K, k = j % im.K;
    float word;
    if (j < im.K) {
      word = __fdiv_rn(1.0f, (float)__ldcg(cnt + j));
    } else {
      const int64_t e = base + j;
      const int64_t px = e / im.K;
      const int c = (int)(e % im.K);
      float f[DIM];
      ld.load(px, 0, 0, f);
      const float a0 = __fsub_rn(f[0], __ldcg(c_old + c * 8 + 0));
      const float a1 = __fsub_rn(f[1], __ldcg(c_old + c * 8 + 1));
      const float a2 = __fsub_rn(f[2], __ldcg(c_old + c * 8 + 2));
      word = __fadd_rn(__fadd_rn(__fmul_rn(a0, a0), __fmul_rn(a1, a1)), __fmul_rn(a2, a2));
    }
    const float t = __fsub_rn(cent[k * CS + d], word);
    acc = __fadd_rn(acc, __fmul_rn(t, t));
  }
  return acc;
}

// Centroids of iteration i >= 1 of an image, c(i) = c(i-1) + S(i-1) / n
// (empty cluster: unchanged; cluster.cu:71-88), formed after the grid barrier
// that ended iteration i - 1, and the convergence test of that iteration.
//
// Its inputs are not written during iteration i (c(i-1) in cur[(i-1) & 1],
// the sums in slot (i-1) % 3, the state after iteration i-2 in state[(i-1) &
// 1]), so every block that calls it gets bit-identical centroids and the same
// decision: for a single image every block calls it, block 0 as the owner; in
// a batch only the owner (img = blockIdx.x mod gridDim.x) does.  The owner
// publishes: c(i) to
// cur[i & 1], the state after iteration i-1 to state[i & 1], zeros for slot
// (i+1) % 3 (read for the last time in iteration i-1, written again in
// iteration i+1), and on convergence the caller's centroids and iteration
// count.  Returns whether the image runs iteration i (uniform in the block);
// its centroids are left in `cent` (stride cstride(DIM)).
template <int LAYOUT, int DIM, int MODE>
__device__ bool form_centroids(const Params& p, int img, const Image& im, int i, float* cent,
                               bool owner, const float* lut) {
  constexpr int CS = cstride(DIM);
  __shared__ float sdiff[kMaxK * kMaxDim];
  __shared__ int smore, sstopped;
  const ImageState* prev = p.state + acc_slot(p, (i - 1) & 1, img);
  ImageState* next = p.state + acc_slot(p, i & 1, img);
  // one reader, so the whole block takes the same branch
  if (threadIdx.x == 0) sstopped = __ldcg(&prev->done);
  __syncthreads();
  if (sstopped) {
    // stopped earlier: carry the state forward
    if (owner && threadIdx.x == 0) {
      next->delta = __ldcg(&prev->delta);
      next->old_delta = __ldcg(&prev->old_delta);
      next->iters = __ldcg(&prev->iters);
      next->done = 1;
    }
    __syncthreads();
    return false;
  }
  const size_t sb = acc_slot(p, (i - 1) % 3, img);
  const unsigned long long* lo = p.acc_lo + sb * (kMaxK * kMaxDim);
  const unsigned long long* hi = p.acc_hi + sb * (kMaxK * kMaxDim);
  const unsigned* cnt = p.acc_cnt + sb * kMaxK;
  const float* c_old = p.cur + acc_slot(p, (i - 1) & 1, img) * (kMaxK * 8);
  float* c_new = p.cur + acc_slot(p, i & 1, img) * (kMaxK * 8);
  for (int idx = threadIdx.x; idx < im.K * DIM; idx += blockDim.x) {
    const int k = idx / DIM, d = idx % DIM, a = k * kMaxDim + d;
    const float c = __ldcg(c_old + k * 8 + d);
    const unsigned n = __ldcg(cnt + k);
    float cn = c;
    if (n > 0) {
      // S = (hi * 2^32 + lo) * 2^-24: one FP64 rounding of the exact sum,
      // one to FP32 (the scaling by 2^-24 is exact); then c + S / n in FP32
      // (every block forms all K x D values, so the FP64 pipe is kept to the
      // conversion: a division there costs the iteration about a microsecond)
      const double S64 = __fma_rn((double)(long long)__ldcg(hi + a), 4294967296.0,
                                  (double)__ldcg(lo + a));
      const float S = __fmul_rn(__double2float_rn(S64), 1.0f / 16777216.0f);
      cn = __fadd_rn(c, __fdiv_rn(S, (float)n));
    }
    cent[k * CS + d] = cn;
    if (owner) __stcg(c_new + k * 8 + d, cn);
    const float df = __fsub_rn(cn, c);
    sdiff[idx] = __fmul_rn(df, df);
  }
  if (owner) {
    const size_t zb = acc_slot(p, (i + 1) % 3, img);
    for (int idx = threadIdx.x; idx < im.K * kMaxDim; idx += blockDim.x) {
      __stcg(p.acc_lo + zb * (kMaxK * kMaxDim) + idx, 0ull);
      __stcg(p.acc_hi + zb * (kMaxK * kMaxDim) + idx, 0ull);
    }
    for (int k = threadIdx.x; k < im.K; k += blockDim.x) __stcg(p.acc_cnt + zb * kMaxK + k, 0u);
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    // squared centroid shift, summed in a fixed order
    float acc = 0.0f;
    for (int idx = threadIdx.x; idx < im.K * DIM; idx += 32) acc = __fadd_rn(acc, sdiff[idx]);
    acc = warp_sum(acc);
    if (DIM == 3 && im.ref_shift && threadIdx.x == 0)
      acc = reference_shift<LAYOUT, DIM>(im, cent, c_old, cnt, lut);
    if (threadIdx.x == 0) {
      const float delta = sqrtf(acc);
      const float old_delta = __ldcg(&prev->delta);
      bool more = i < im.max_iter && fabsf(delta - old_delta) > im.threshold;
      if (MODE == kUpdateOnly) more = false;
      smore = more ? 1 : 0;
      if (owner) {
        next->delta = delta;
        next->old_delta = old_delta;
        next->iters = i;
        next->done = more ? 0 : 1;
        if (im.d_iterations && !more) *im.d_iterations = i;
      }
    }
  }
  __syncthreads();
  const bool more = smore != 0;
  if (owner && !more) {
    // final centroids back to the caller's planar array
    for (int idx = threadIdx.x; idx < im.K * DIM; idx += blockDim.x) {
      const int k = idx / DIM, d = idx % DIM;
      im.centroids[d * im.K + k] = cent[k * CS + d];
    }
  }
  __syncthreads();
  return more;
}

// An iteration after the first of a single image whose fast spans' sums are
// kept, by spans instead of units.  Most spans then need none of their pixels
// (one candidate: labels and sums known), so the block takes its share of
// spans, s = blockIdx.x + j * gridDim.x with warp w taking j = w, w + kWarps,
// ... (odd iterations in reverse order, starting on what the last one left
// in L2), finishes those at once and lists the others; its warps then take
// the listed spans one at a time (with at most one span per warp, a warp
// does its span at once).  No block barrier per span, and the block's
// integer sums go to the image accumulators once.  Each span's contribution
// is the same as in the unit loop, so the result is too.
template <int LAYOUT, int DIM, int MODE>
__device__ void span_iteration(const Params& p, Smem& sm, int it) {
  constexpr unsigned full = 0xffffffffu;
  const Image& im = p.img0;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wrows = im.unit_rows / kWarps;
  const int nspans = ((im.height + wrows - 1) / wrows) * im.ntx;
  const bool wl = im.threshold >= 0.0f || it == im.max_iter - 1;
  int* status = &p.hdr->status;
  if (threadIdx.x == 0) {
    sm.nheavy = 0;
    sm.next_heavy = 0;
  }
  __syncthreads();
  const int rows = wrows / kBatchRows;
  const int lrow = lane / kLanesPerRow, lcol = (lane % kLanesPerRow) * kPx;
  const bool vec_labels = (reinterpret_cast<uintptr_t>(im.labels) & 15) == 0 && (im.width % kPx) == 0;
  // Groups of up to kGroup of the warp's spans: classify each (candidates
  // from the geometry alone), then one round of loads brings every light
  // span's kept words (lane g * DIM + d: span g, dimension d).
  constexpr int kGroup = 32 / DIM < 6 ? 32 / DIM : 6;
  // with at most one span per warp (small images) nothing is gained by
  // deferring: a warp does its span at once
  const bool defer = nspans > (int)gridDim.x * kWarps;
  for (int j0 = warp;; j0 += kGroup * kWarps) {
    int s_lane = -1, k_lane = -1;   // lane g: light span g and its cluster
    int g = 0;
    for (; g < kGroup; ++g) {
      const int64_t s64 = (int64_t)blockIdx.x + (int64_t)(j0 + g * kWarps) * gridDim.x;
      if (s64 >= nspans) break;
      const int s = (it & 1) ? nspans - 1 - (int)s64 : (int)s64;
      const int sr = s / im.ntx, tx = s - sr * im.ntx;
      int k = -1;
      if (fast_geometry<LAYOUT, DIM, MODE>(im, sr * wrows, tx * kTile, wrows, vec_labels)) {
        const unsigned long long m =
            unit_box_mask<DIM>(im, sm, sr * wrows, tx * kTile, wrows, kTile);
        if (m != 0ull && (m & (m - 1ull)) == 0ull) k = __ffsll((long long)m) - 1;
      }
      if (k >= 0) {
        if (lane == g) {
          s_lane = s;
          k_lane = k;
        }
        if (wl) write_span_labels(im, sr * wrows + lrow, tx * kTile + lcol, rows, k, vec_labels);
        continue;
      }
      if (defer) {
        int slot = 0;
        if (lane == 0) slot = atomicAdd(&sm.nheavy, 1);
        slot = __shfl_sync(full, slot, 0);
        if (slot < kHeavyCap) {
          if (lane == 0) sm.heavy[slot] = s;
          continue;
        }
      }
      // not deferred, or the list is full: this one now
      process_span<LAYOUT, DIM, MODE>(im, sr, tx, sm, wl, it, status);
    }
    const int gs = lane / DIM, d = lane - gs * DIM;
    const int s = __shfl_sync(full, s_lane, gs < kGroup ? gs : 0);
    const int k = __shfl_sync(full, k_lane, gs < kGroup ? gs : 0);
    if (gs < kGroup && s >= 0) {
      const int sr = s / im.ntx;
      const long long w =
          __ldcg(im.span_sum + ((size_t)sr * im.span_cols + (s - sr * im.ntx)) * kSpanSums + d);
      const double nc = __dmul_rn((double)(wrows * kTile),
                                  __dmul_rn((double)sm.cent[k * cstride(DIM) + d], 16777216.0));
      atomicAdd(reinterpret_cast<unsigned long long*>(&sm.fix[k * kMaxDim + d]),
                (unsigned long long)(w - __double2ll_rn(nc)));
    }
    if (lane < kGroup && s_lane >= 0) atomicAdd(&sm.fixn[k_lane], wrows * kTile);
    if (g < kGroup) break;
  }
  __syncthreads();
  const int nh = min(sm.nheavy, kHeavyCap);
  for (;;) {
    int idx = 0;
    if (lane == 0) idx = atomicAdd(&sm.next_heavy, 1);
    idx = __shfl_sync(full, idx, 0);
    if (idx >= nh) break;
    const int s = sm.heavy[idx];
    const int sr = s / im.ntx;
    process_span<LAYOUT, DIM, MODE>(im, sr, s - sr * im.ntx, sm, wl, it, status);
  }
  block_to_accum(sm, p, 0, im.K, DIM, it % 3);
}

// BATCH: the instance for multi-image launches (no span iterations: a
// batch's images go through the unit loop).
template <int LAYOUT, int DIM, int MODE, bool BATCH = false>
__global__ void __launch_bounds__(kThreads, BATCH ? kBatchMinBlocks : SG_KM_MINBLOCKS)
    kmeans_kernel(Params p) {
  __shared__ Smem sm;
  for (int i = threadIdx.x; i < kWarps * kMaxK * kMaxDim; i += blockDim.x)
    (&sm.acc[0][0])[i] = 0.0f;
  for (int i = threadIdx.x; i < kWarps * kMaxK; i += blockDim.x) (&sm.cnt[0][0])[i] = 0;
  for (int i = threadIdx.x; i < kMaxK * kMaxDim; i += blockDim.x) sm.fix[i] = 0;
  for (int i = threadIdx.x; i < kMaxK; i += blockDim.x) sm.fixn[i] = 0;
  if (LAYOUT == SPLIT_LAYOUT_RGB8)
    for (int i = threadIdx.x; i < 256; i += blockDim.x) sm.lut[i] = (float)i / 255.0f;
  __syncthreads();

  bool stopped = false;   // a single image that converged: no iterations left
  unsigned nbar = 0;      // grid barriers passed (every block passes the same ones)
  for (int it = 0; it < p.max_iter; ++it) {
    if (blockIdx.x == 0 && threadIdx.x == 0) p.hdr->work_counter[(it + 1) & 1] = 0;
    int cached = -1;
    bool more = false;      // the cached image runs this iteration
    if (MODE != kAssignOnly && it > 0) {
      if (p.nimages == 1) {
        // every block forms the single image's centroids (block 0 publishes),
        // so all of them see it converge together
        more = form_centroids<LAYOUT, DIM, MODE>(p, 0, image_of(p, 0), it, sm.cent,
                                                 blockIdx.x == 0, sm.lut);
        cached = 0;
        if (!more) {
          stopped = true;
          break;
        }
      } else {
        // A batch: owners form and publish their images, then a second grid
        // barrier, so that a block switching images (often, with small
        // images) only loads the published centroids.
        for (int img = (int)blockIdx.x; img < p.nimages; img += gridDim.x)
          form_centroids<LAYOUT, DIM, MODE>(p, img, image_of(p, img), it, sm.cent, true,
                                            sm.lut);
        if (!grid_barrier_counted(p.hdr, ++nbar, p.wait_limit, p.wait_skip)) return;
      }
    }
    if constexpr (MODE == kCluster && !BATCH) {
      if (p.nimages == 1 && it > 0 && p.img0.span_sum) {
        span_iteration<LAYOUT, DIM, MODE>(p, sm, it);
        if (!grid_barrier_counted(p.hdr, ++nbar, p.wait_limit, p.wait_skip)) return;
        continue;
      }
    }
    // The first wave is static (block b takes unit b): only later fetches go
    // through the work counter, so blocks do not queue on it as they start.
    int raw = (int)blockIdx.x;
    for (int k = 0; raw < p.total_units; ++k) {
      // odd iterations walk the units backwards: they start on the units the
      // previous iteration touched last, which are still resident in L2
      const int u = (it & 1) ? p.total_units - 1 - raw : raw;
      const int img = find_image(p, u);
      const Image& im = image_of(p, img);
      if (img != cached) {
        if (MODE == kAssignOnly) {
          load_centroids<DIM>(p.cur + (size_t)img * (kMaxK * 8), im.K, sm.cent);
          more = true;
        } else {
          // the published centroids and state of iteration it (a single
          // image reaches this only in iteration 0)
          load_centroids<DIM>(p.cur + acc_slot(p, it & 1, img) * (kMaxK * 8), im.K, sm.cent);
          if (threadIdx.x == 0) sm.more = !__ldcg(&p.state[acc_slot(p, it & 1, img)].done);
        }
        cached = img;
        __syncthreads();
        if (MODE != kAssignOnly) more = sm.more != 0;
      }
      if (more) {
        const int lu = u - im.unit_begin;
        const bool wl = (MODE == kAssignOnly) ||
                        (MODE == kCluster && (im.threshold >= 0.0f || it == im.max_iter - 1));
        const int ty = lu / im.ntx;
        process_span<LAYOUT, DIM, MODE>(im, ty * kWarps + (int)(threadIdx.x >> 5),
                                        lu - ty * im.ntx, sm, wl, it, &p.hdr->status);
        if (MODE != kAssignOnly) block_to_accum(sm, p, img, im.K, DIM, it % 3);
      }
      // the last warp fetches the next unit (slot k & 1 was last read before
      // the barrier that ended unit k - 1)
      if (threadIdx.x == kThreads - 32) {
        if (MODE != kAssignOnly && !more && p.nimages > 1) {
          // a batch image that has stopped: later fetches skip the rest of its
          // units (which only changes who does which unit, not any result)
          const int ub = im.unit_begin, ue = ub + im.nunits;
          const int raw_end = (it & 1) ? p.total_units - ub : ue;
          if (raw_end > (int)gridDim.x)
            atomicMax(&p.hdr->work_counter[it & 1], (unsigned)(raw_end - (int)gridDim.x));
        }
        sm.next[k & 1] = (int)gridDim.x + (int)atomicAdd(&p.hdr->work_counter[it & 1], 1u);
      }
      __syncthreads();
      raw = sm.next[k & 1];
    }
    if (MODE == kAssignOnly) return;
    // the barrier publishes every block's sums (fire-and-forget adds ordered
    // by the block barrier before the arrival's release)
    if (!grid_barrier_counted(p.hdr, ++nbar, p.wait_limit, p.wait_skip)) return;
  }
  if (MODE == kAssignOnly || stopped) return;
  // centroids after the last iteration; every image stops here
  for (int img = (int)blockIdx.x; img < p.nimages; img += gridDim.x)
    form_centroids<LAYOUT, DIM, MODE>(p, img, image_of(p, img), p.max_iter, sm.cent, true,
                                      sm.lut);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

struct Layout {
  unsigned long long* acc_lo;
  unsigned long long* acc_hi;
  unsigned* acc_cnt;
  float* cur;
  ImageState* state;
  Image* images;
  long long* span_sum;   // single image: kept span feature words (after the rest)
  WsHeader* hdr;
  size_t bytes;
};

inline int height_of(int64_t n, int width) { return (int)((n + width - 1) / width); }
inline int tiles_x(int width) { return (width + kTile - 1) / kTile; }
inline int units_of(int64_t n, int width, int rows = kTile) {
  return tiles_x(width) * ((height_of(n, width) + rows - 1) / rows);
}
// Fast spans of an image: full kTile-wide tile columns times full span-row
// slices at the smallest span height (2 rows, 16-row units), which bounds
// every unit height the tuning table may choose.
inline int64_t span_slots(int64_t n, int width) {
  return (int64_t)(width / kTile) * (height_of(n, width) / 2);
}

// The workspace holds per-image state (accumulators, centroids, counters),
// whose size does not depend on the image sizes, and optionally a single
// image's kept span sums (kSpanSums words per fast span, after the rest: a
// workspace without them runs the same clustering, reading every pixel in
// every iteration).
static Layout carve(void* ws, int nimages, int64_t span_entries = 0) {
  Carver c(ws);
  Layout l;
  l.hdr = c.take<WsHeader>(1);
  l.acc_lo = c.take<unsigned long long>((size_t)3 * nimages * kMaxK * kMaxDim);
  l.acc_hi = c.take<unsigned long long>((size_t)3 * nimages * kMaxK * kMaxDim);
  l.acc_cnt = c.take<unsigned>((size_t)3 * nimages * kMaxK);
  l.cur = c.take<float>((size_t)2 * nimages * kMaxK * 8);
  l.state = c.take<ImageState>((size_t)2 * nimages);
  l.images = nimages > 1 ? c.take<Image>((size_t)nimages) : nullptr;
  l.span_sum = span_entries > 0 ? c.take<long long>((size_t)span_entries * kSpanSums) : nullptr;
  l.bytes = c.size();
  return l;
}

// Header words used by the barrier and the work counters and all three
// accumulator slots start every call at zero (a call that stopped early, or
// a workspace used by another call, may have left data there).
static int reset_counters(const Layout& l, int nimages, cudaStream_t st) {
  (void)nimages;
  SG_CUDA_TRY(cudaMemsetAsync(reinterpret_cast<char*>(l.hdr) + sizeof(int), 0,
                              sizeof(unsigned) * 4, st));
  SG_CUDA_TRY(cudaMemsetAsync(l.acc_lo, 0, reinterpret_cast<char*>(l.cur) -
                                               reinterpret_cast<char*>(l.acc_lo), st));
  return SPLIT_OK;
}

// Per-image iteration state (cluster.cu:65-68: delta = 0, old_delta =
// delta + threshold + 1, so the first convergence test always passes).
__global__ void init_kernel(Params p) {
  pdl_wait();
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

// Per-call setup of a single-image clustering in one launch: the header's
// barrier and work counters and all three accumulator slots to zero
// (`zero` .. `zero` + zero_words: the slots and the counts), the iteration
// state (cluster.cu:65-68), and the caller's planar centroids into slot 0.
template <int DIM>
__global__ void setup_kernel(Params p, unsigned* zero, int zero_words) {
  pdl_wait();
  const Image& im = p.img0;
  if (threadIdx.x == 0) {
    p.hdr->barrier_count = 0u;
    p.hdr->barrier_gen = 0u;
    p.hdr->work_counter[0] = 0u;
    p.hdr->work_counter[1] = 0u;
    ImageState st;
    st.delta = 0.0f;
    st.old_delta = st.delta + im.threshold + 1.0f;
    st.iters = 0;
    st.done = im.max_iter <= 0;
    p.state[0] = st;
    if (im.d_iterations && st.done) *im.d_iterations = 0;
  }
  for (int i = threadIdx.x; i < zero_words; i += blockDim.x) zero[i] = 0u;
  for (int idx = threadIdx.x; idx < im.K * DIM; idx += blockDim.x) {
    const int k = idx / DIM, d = idx % DIM;
    p.cur[k * 8 + d] = im.centroids[d * im.K + k];
  }
}

template <int DIM>
__global__ void load_user_centroids(Params p) {
  pdl_wait();
  for (int img = blockIdx.x; img < p.nimages; img += gridDim.x) {
    const Image& im = image_of(p, img);
    float* c0 = p.cur + (size_t)img * (kMaxK * 8);
    for (int idx = threadIdx.x; idx < im.K * DIM; idx += blockDim.x) {
      const int k = idx / DIM, d = idx % DIM;
      c0[k * 8 + d] = im.centroids[d * im.K + k];
    }
  }
}

// ---- tuning table (host side) ----------------------------------------------
// Per image size class: the unit height and the resident blocks per SM of
// the cooperative launch.  A unit height is chosen from the image's own pixel
// count, so an image gets the same reduction tree alone and in a batch.
struct TuneTable {
  std::mutex m;
  std::vector<split_tune_entry> e;
};
static TuneTable& tune_table() {
  static TuneTable t;
  return t;
}
split_tune_entry tuned(int64_t npix) {
  TuneTable& t = tune_table();
  std::lock_guard<std::mutex> g(t.m);
  for (const split_tune_entry& x : t.e)
    if (npix <= x.max_pixels) return x;
  return split_tune_entry{INT64_MAX, kTile, 0};
}

// The float4 kernels stage features in kStageBytes of dynamic shared memory,
// above the default 48 KB limit with their static part: the attribute is set
// once per device, before any launch (and outside any graph capture: batch
// preparation calls this too).
static int stage_attributes() {
  static std::mutex mu;
  static bool done[64] = {false};
  int dev = 0;
  SG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return SPLIT_ERR_CUDA;
  std::lock_guard<std::mutex> lock(mu);
  if (done[dev]) return SPLIT_OK;
  const void* kerns[] = {
      (const void*)kmeans_kernel<SPLIT_LAYOUT_FLOAT4, 3, kCluster>,
      (const void*)kmeans_kernel<SPLIT_LAYOUT_FLOAT4, 5, kCluster>,
      (const void*)kmeans_kernel<SPLIT_LAYOUT_FLOAT4, 3, kUpdateOnly>,
      (const void*)kmeans_kernel<SPLIT_LAYOUT_FLOAT4, 5, kUpdateOnly>,
      (const void*)kmeans_kernel<SPLIT_LAYOUT_FLOAT4, 3, kAssignOnly>,
      (const void*)kmeans_kernel<SPLIT_LAYOUT_FLOAT4, 5, kAssignOnly>,
      (const void*)kmeans_kernel<SPLIT_LAYOUT_FLOAT4, 3, kCluster, true>,
      (const void*)kmeans_kernel<SPLIT_LAYOUT_FLOAT4, 5, kCluster, true>};
  for (const void* k : kerns)
    SG_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kStageBytes));
  done[dev] = true;
  return SPLIT_OK;
}

template <int LAYOUT, int DIM, int MODE>
static int launch(Params& p, cudaStream_t st) {
  DeviceInfo di;
  SG_TRY(device_info(&di));
  auto kern = kmeans_kernel<LAYOUT, DIM, MODE>;
  if constexpr (MODE == kCluster)
    if (p.images) kern = kmeans_kernel<LAYOUT, DIM, MODE, true>;   // a batch
  const size_t dyn = LAYOUT == SPLIT_LAYOUT_FLOAT4 ? kStageBytes : 0;
  if (dyn) SG_TRY(stage_attributes());
  int per_sm = 0;
  SG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, dyn));
  if (per_sm < 1) return SPLIT_ERR_UNSUPPORTED;
  if (p.blocks_per_sm > 0 && p.blocks_per_sm < per_sm) per_sm = p.blocks_per_sm;
  int grid = di.sm_count * per_sm;
  if (grid > p.total_units) grid = p.total_units > 0 ? p.total_units : 1;
  if (MODE == kAssignOnly) {
    kern<<<grid, kThreads, dyn, st>>>(p);
    return launch_status();
  }
  void* args[] = {&p};
  SG_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)kern, dim3(grid), dim3(kThreads),
                                          args, dyn, st));
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
  layout &= ~(SPLIT_FEATURES_UNIT_RANGE | SPLIT_KMEANS_REFERENCE_SHIFT);
  if (!points || n <= 0 || n > 0x7fffffffLL || K < 1 || K > kMaxK) return false;
  if (dim != 3 && dim != 5) return false;
  if (layout < SPLIT_LAYOUT_PLANAR || layout > SPLIT_LAYOUT_RGB8) return false;
  if (width < 1) return false;
  if (layout == SPLIT_LAYOUT_FLOAT4 && (reinterpret_cast<uintptr_t>(points) & 15)) return false;
  return true;
}

// Test setting of the grid barriers of single-image launches
// (split_kmeans_set_wait_test): poll limit (0: kSpinLimit) and skipping block.
static std::atomic<unsigned> g_wait_limit{0};
static std::atomic<int> g_wait_skip{-1};
static void wait_test(unsigned* limit, int* skip) {
  const unsigned l = g_wait_limit.load(std::memory_order_relaxed);
  *limit = l ? l : kSpinLimit;
  *skip = g_wait_skip.load(std::memory_order_relaxed);
}

static int run(int mode, const void* points, int layout, int dim, int64_t n,
               int width, float xy_scale, float* centroids,
               const float* centroids_in, int K, int32_t* labels,
               const int32_t* labels_in, void* ws, size_t ws_bytes, int max_iter,
               float threshold, int32_t* d_iter, cudaStream_t st) {
  if (!valid_features(points, layout, dim, n, width, K)) return SPLIT_ERR_INVALID;
  const int unit_range = (layout & SPLIT_FEATURES_UNIT_RANGE) ? 1 : 0;
  const int ref_shift = (layout & SPLIT_KMEANS_REFERENCE_SHIFT) ? 1 : 0;
  layout &= ~(SPLIT_FEATURES_UNIT_RANGE | SPLIT_KMEANS_REFERENCE_SHIFT);
  // the reference's shift is defined for its own case only: 3-D clustering
  // with every word it reads inside the N x K distance matrix
  if (ref_shift && (mode != kCluster || dim != 3 || K < 3 || n * (K - 2) < 3 * (int64_t)K))
    return SPLIT_ERR_INVALID;
  const split_tune_entry te = tuned(n);
  const int units = units_of(n, width, te.kmeans_unit_rows);
  Layout l = carve(nullptr, 1);
  if (!ws || ws_bytes < l.bytes || (reinterpret_cast<uintptr_t>(ws) & 255))
    return SPLIT_ERR_WORKSPACE;
  // span sums for a clustering of more than one iteration, where the
  // workspace holds them
  const int64_t slots = span_slots(n, width);
  const bool keep = mode == kCluster && max_iter > 1 && slots > 0 &&
                    ws_bytes >= carve(nullptr, 1, slots).bytes;
  l = carve(ws, 1, keep ? slots : 0);
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
  im.height = height_of(n, width);
  im.ntx = tiles_x(width);
  im.unit_rows = te.kmeans_unit_rows;
  im.ref_shift = ref_shift;
  im.span_sum = l.span_sum;
  im.span_cols = width / kTile;
  p.blocks_per_sm = te.kmeans_blocks_per_sm;
  wait_test(&p.wait_limit, &p.wait_skip);
  p.nimages = 1;
  p.images = nullptr;
  p.total_units = units;
  p.max_iter = max_iter;
  p.acc_lo = l.acc_lo;
  p.acc_hi = l.acc_hi;
  p.acc_cnt = l.acc_cnt;
  p.cur = l.cur;
  p.state = l.state;
  p.hdr = l.hdr;
  (void)centroids_in;
  // counters, accumulator slots, state and centroids in one launch (the
  // slots and counts lie between acc_lo and cur, 256-byte aligned pieces)
  unsigned* zero = reinterpret_cast<unsigned*>(l.acc_lo);
  const int zero_words = (int)((reinterpret_cast<char*>(l.cur) -
                                reinterpret_cast<char*>(l.acc_lo)) / sizeof(unsigned));
  if (dim == 3) launch_pdl(setup_kernel<3>, dim3(1), dim3(256), 0, st, p, zero, zero_words);
  else launch_pdl(setup_kernel<5>, dim3(1), dim3(256), 0, st, p, zero, zero_words);
  SG_TRY(launch_status());
  if (max_iter <= 0) return SPLIT_OK;
  if (mode == kCluster) return dispatch<kCluster>(layout, dim, p, st);
  if (mode == kUpdateOnly) return dispatch<kUpdateOnly>(layout, dim, p, st);
  return dispatch<kAssignOnly>(layout, dim, p, st);
}

}  // namespace km
}  // namespace sg

using namespace sg;

namespace sg {
namespace kmw {
// more clusters than the persistent kernel holds (kmeans_wide.cu)
int run(bool cluster, const void* points, int layout, int dim, int64_t n, int width,
        float xy_scale, float* centroids, const float* cent_in, int K, int32_t* labels,
        void* ws, size_t ws_bytes, int max_iter, float threshold, int32_t* d_iter,
        cudaStream_t st);
size_t workspace_bytes(int K, int dim);
}  // namespace kmw
}  // namespace sg

extern "C" void split_kmeans_set_wait_test(unsigned spin_limit, int skip_block) {
  km::g_wait_limit.store(spin_limit, std::memory_order_relaxed);
  km::g_wait_skip.store(skip_block < 0 ? -1 : skip_block, std::memory_order_relaxed);
}

extern "C" size_t split_kmeans_cluster_workspace_size_2d(int64_t npoints, int width,
                                                         int nclusters, int dim) {
  if (npoints <= 0 || width < 1) return 0;
  if (nclusters > km::kMaxK) {
    if (dim != 3 && dim != 5) dim = 5;
    return kmw::workspace_bytes(nclusters, dim);
  }
  // with the kept span sums of a clustering
  return km::carve(nullptr, 1, km::span_slots(npoints, width)).bytes;
}

extern "C" size_t split_kmeans_cluster_workspace_size(int64_t npoints, int nclusters, int dim) {
  // without the image width: room for the span sums at any width
  // ((width / 64) * (height / 2) <= npoints / 64 + 1)
  if (npoints <= 0) return 0;
  if (nclusters > km::kMaxK) return split_kmeans_cluster_workspace_size_2d(npoints, 1, nclusters, dim);
  return km::carve(nullptr, 1, npoints / 64 + 1).bytes;
}

extern "C" int split_kmeans_cluster(const void* points, int layout, int dim, int64_t npoints,
                                    int width, float xy_scale, float* centroids, int nclusters,
                                    int32_t* labels, void* workspace, size_t workspace_bytes,
                                    int max_iter, float threshold, int32_t* d_iterations,
                                    void* stream) {
  if (!centroids || !labels) return SPLIT_ERR_INVALID;
  if (nclusters > km::kMaxK)
    return kmw::run(true, points, layout, dim, npoints, width, xy_scale, centroids, centroids,
                    nclusters, labels, workspace, workspace_bytes, max_iter, threshold,
                    d_iterations, as_stream(stream));
  return km::run(km::kCluster, points, layout, dim, npoints, width, xy_scale, centroids,
                 centroids, nclusters, labels, nullptr, workspace, workspace_bytes, max_iter,
                 threshold, d_iterations, as_stream(stream));
}

extern "C" size_t split_kmeans_assign_workspace_size(int64_t npoints, int nclusters) {
  // one assignment keeps no span sums
  if (npoints <= 0) return 0;
  if (nclusters > km::kMaxK) return split_kmeans_cluster_workspace_size(npoints, nclusters, 5);
  return km::carve(nullptr, 1).bytes;
}

extern "C" int split_kmeans_assign(const void* points, int layout, int dim, int64_t npoints,
                                   int width, float xy_scale, const float* centroids,
                                   int nclusters, int32_t* labels, void* workspace,
                                   size_t workspace_bytes, void* stream) {
  if (!centroids || !labels) return SPLIT_ERR_INVALID;
  if (nclusters > km::kMaxK)
    return kmw::run(false, points, layout, dim, npoints, width, xy_scale, nullptr, centroids,
                    nclusters, labels, workspace, workspace_bytes, 1, -1.0f, nullptr,
                    as_stream(stream));
  return km::run(km::kAssignOnly, points, layout, dim, npoints, width, xy_scale,
                 const_cast<float*>(centroids), centroids, nclusters, labels, nullptr,
                 workspace, workspace_bytes, 1, -1.0f, nullptr, as_stream(stream));
}

namespace sg {
namespace segm {
int run(const int32_t* labels, const void* points, int layout, int dim, int64_t n, int width,
        float xy_scale, float* centroids, int K, void* ws, size_t ws_bytes, cudaStream_t st);
size_t workspace_bytes(int K, int dim);
}  // namespace segm
}  // namespace sg

extern "C" size_t split_kmeans_update_workspace_size(int64_t npoints, int nclusters, int dim) {
  // more clusters than the k-means kernel holds in shared memory: per-cluster
  // accumulators (16 B per feature value + a count)
  if (nclusters > km::kMaxK) {
    if (npoints <= 0 || dim < 1) return 0;
    return segm::workspace_bytes(nclusters, dim);
  }
  if (npoints <= 0) return 0;
  return km::carve(nullptr, 1).bytes;
}

extern "C" int split_kmeans_update(const int32_t* labels, const void* points, int layout,
                                   int dim, int64_t npoints, int width, float xy_scale,
                                   float* centroids, int nclusters, void* workspace,
                                   size_t workspace_bytes, void* stream) {
  if (!centroids || !labels) return SPLIT_ERR_INVALID;
  if (nclusters > km::kMaxK)
    return segm::run(labels, points, layout, dim, npoints, width, xy_scale, centroids,
                     nclusters, workspace, workspace_bytes, as_stream(stream));
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

// ---------------------------------------------------------------------------
// Allocation-free clustering.  Some callers cannot allocate device memory at
// the point where they cluster: a latency-critical serving loop (cudaMalloc
// and cudaFree synchronise the device), and host plugins whose device memory
// is owned by a pool they may not touch.  This variant keeps its scratch in
// one file-scope device array of fixed size, so a call needs no workspace.
//
// Limits and sharing rules:
//   - the array holds the state of one image, whatever its size: three
//     accumulator slots, two centroid slots and the iteration state for up
//     to kMaxK (64) clusters of up to kMaxDim (5) dimensions, 20736 bytes.
//     K above 64, or D other than 3 and 5, is rejected with
//     SPLIT_ERR_INVALID before anything is queued, as the workspace entry
//     point does;
//   - every GPU that loads the library holds the array until the process
//     exits; its device address is looked up once per device, on the first
//     call made with that device current.  A cudaDeviceReset of that device
//     unloads the module and may move the array, so the cached address is
//     stale afterwards: a process that resets a device must not call this
//     entry point on it again;
//   - all calls share the array: two calls whose work overlaps on the GPU
//     (different streams, or different host threads without ordering) race
//     and corrupt each other's results.  Order them on one stream.
// ---------------------------------------------------------------------------
#include <mutex>

namespace sg {
namespace km {

// Size of carve(ws, 1), evaluated at compile time (every piece starts on a
// 256-byte boundary).
constexpr size_t round256(size_t v) { return (v + 255) & ~size_t(255); }
constexpr size_t kStaticBytes =
    round256(round256(round256(round256(round256(round256(sizeof(WsHeader)) +
                                                 (size_t)3 * kMaxK * kMaxDim * 8) +
                                        (size_t)3 * kMaxK * kMaxDim * 8) +
                               (size_t)3 * kMaxK * 4) +
                      (size_t)2 * kMaxK * 8 * 4) +
             (size_t)2 * sizeof(ImageState));

static __device__ __align__(256) unsigned char g_static_scratch[kStaticBytes];

// Device address of g_static_scratch on the current device (looked up once).
static int static_scratch(void** out) {
  static std::mutex mu;
  static void* addr[64] = {nullptr};
  int dev = 0;
  SG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return SPLIT_ERR_CUDA;
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess || !p) return SPLIT_ERR_CUDA;
    addr[dev] = p;
  }
  *out = addr[dev];
  return SPLIT_OK;
}

}  // namespace km
}  // namespace sg

extern "C" int split_kmeans_cluster_noalloc(const void* points, int layout, int dim,
                                            int64_t npoints, int width, float xy_scale,
                                            float* centroids, int nclusters, int32_t* labels,
                                            int max_iter, float threshold,
                                            int32_t* d_iterations, int32_t* d_status,
                                            void* stream) {
  using namespace sg::km;
  if (!centroids || !labels || npoints <= 0 || width < 1) return SPLIT_ERR_INVALID;
  // K, D and the layout first: nothing is queued for a call run() would refuse
  if (!valid_features(points, layout, dim, npoints, width, nclusters)) return SPLIT_ERR_INVALID;
  // one image's state, for any image size, always fits the array
  if (carve(nullptr, 1).bytes > kStaticBytes) return SPLIT_ERR_WORKSPACE;
  void* ws = nullptr;
  SG_TRY(static_scratch(&ws));
  cudaStream_t st = as_stream(stream);
  // The array keeps the previous call's contents: the status word starts at
  // zero here (run() clears the barrier words, counters and accumulators).
  Layout l = carve(ws, 1);
  SG_CUDA_TRY(cudaMemsetAsync(l.hdr, 0, sizeof(WsHeader), st));
  SG_TRY(run(kCluster, points, layout, dim, npoints, width, xy_scale, centroids, centroids,
             nclusters, labels, nullptr, ws, kStaticBytes, max_iter, threshold, d_iterations,
             st));
  if (d_status)
    SG_CUDA_TRY(cudaMemcpyAsync(d_status, &l.hdr->status, sizeof(int), cudaMemcpyDeviceToDevice,
                                st));
  return SPLIT_OK;
}

// ---------------------------------------------------------------------------
// Batches: one cooperative launch clusters every image of a batch (per-image
// K, iteration count and threshold); each image keeps its own tiles, groups,
// reduction tree and convergence test, so its result does not depend on what
// else shares the launch.
// ---------------------------------------------------------------------------
#include "kmeans_batch.h"

namespace sg {

namespace kmb {
struct BatchCounts {
  int units;
};
// Unit and group totals; sized (for the workspace) at the smallest unit
// height, which needs the most records, or at each image's tuned height.
BatchCounts batch_counts(const KmBatchImage* imgs, int n, bool tuned_rows) {
  BatchCounts c{0};
  for (int i = 0; i < n; ++i) {
    const int rows = tuned_rows ? km::tuned(imgs[i].npoints).kmeans_unit_rows : km::kTile;
    const int u = km::units_of(imgs[i].npoints, imgs[i].width, rows);
    c.units += u;
  }
  return c;
}
}  // namespace kmb
using kmb::BatchCounts;
using kmb::batch_counts;

// Kept span sums of a batch's images (those clustered more than once).
static int64_t batch_span_slots(const KmBatchImage* imgs, int nimages) {
  int64_t t = 0;
  for (int i = 0; i < nimages; ++i)
    if (imgs[i].iters > 1) t += km::span_slots(imgs[i].npoints, imgs[i].width);
  return t;
}

size_t kmeans_batch_workspace(const KmBatchImage* imgs, int nimages) {
  (void)batch_counts;
  return km::carve(nullptr, nimages > 1 ? nimages : 2, batch_span_slots(imgs, nimages)).bytes;
}

int kmeans_batch_prepare(const KmBatchImage* imgs, int nimages, int layout, int dim,
                         float xy_scale, void* ws, size_t ws_bytes, cudaStream_t st,
                         KmBatchPlan* plan) {
  using namespace km;
  if (!imgs || nimages < 1 || (dim != 3 && dim != 5)) return SPLIT_ERR_INVALID;
  // kernel attributes now: the batch's launches may be captured into a graph
  SG_TRY(stage_attributes());
  const int unit_range = (layout & SPLIT_FEATURES_UNIT_RANGE) ? 1 : 0;
  if (layout & SPLIT_KMEANS_REFERENCE_SHIFT) return SPLIT_ERR_INVALID;   // single images only
  layout &= ~SPLIT_FEATURES_UNIT_RANGE;
  const BatchCounts c = batch_counts(imgs, nimages, true);
  const int slots = nimages > 1 ? nimages : 2;
  Layout l = carve(nullptr, slots);
  if (!ws || ws_bytes < l.bytes || (reinterpret_cast<uintptr_t>(ws) & 255))
    return SPLIT_ERR_WORKSPACE;
  // the images' kept span sums, where the workspace holds them
  const int64_t span_total = batch_span_slots(imgs, nimages);
  const bool keep = span_total > 0 && ws_bytes >= carve(nullptr, slots, span_total).bytes;
  l = carve(ws, slots, keep ? span_total : 0);
  int64_t span_off = 0;
  std::vector<Image> host(nimages);
  int ub = 0, max_iter = 0;
  int64_t total_px = 0;
  for (int i = 0; i < nimages; ++i) {
    const KmBatchImage& b = imgs[i];
    if (!valid_features(b.points, layout, dim, b.npoints, b.width, b.nclusters) || !b.centroids ||
        !b.labels)
      return SPLIT_ERR_INVALID;
    Image& im = host[i];
    memset(&im, 0, sizeof(im));
    im.points = b.points;
    im.unit_range = unit_range;
    im.npoints = b.npoints;
    im.width = b.width;
    im.xy_scale = xy_scale;
    im.centroids = b.centroids;
    im.labels = b.labels;
    im.K = b.nclusters;
    im.max_iter = b.iters;
    im.threshold = b.threshold;
    im.unit_begin = ub;
    im.unit_rows = tuned(b.npoints).kmeans_unit_rows;
    im.nunits = units_of(b.npoints, b.width, im.unit_rows);
    total_px += b.npoints;
    im.height = height_of(b.npoints, b.width);
    im.ntx = tiles_x(b.width);
    im.span_cols = b.width / kTile;
    if (keep && b.iters > 1) {
      im.span_sum = l.span_sum + span_off * kSpanSums;
      span_off += span_slots(b.npoints, b.width);
    }
    ub += im.nunits;
    max_iter = max_iter > b.iters ? max_iter : b.iters;
  }
  SG_CUDA_TRY(cudaMemcpyAsync(l.images, host.data(), sizeof(Image) * nimages,
                              cudaMemcpyHostToDevice, st));
  // the host copy must outlive the transfer
  SG_CUDA_TRY(cudaStreamSynchronize(st));
  plan->nimages = nimages;
  plan->units = c.units;
  plan->max_iter = max_iter;
  plan->layout = layout;
  plan->dim = dim;
  // the tuning table's residency is measured on single images, whose kernel
  // instance differs: a batch runs as many blocks as fit
  (void)total_px;
  plan->blocks_per_sm = 0;
  return SPLIT_OK;
}

int kmeans_batch_run(const KmBatchPlan& plan, void* ws, cudaStream_t st) {
  using namespace km;
  const int slots = plan.nimages > 1 ? plan.nimages : 2;
  Layout l = carve(ws, slots);
  Params p{};
  p.nimages = plan.nimages;
  p.images = l.images;  // a one-image batch reads its descriptor from the table too
  p.total_units = plan.units;
  p.max_iter = plan.max_iter;
  p.acc_lo = l.acc_lo;
  p.acc_hi = l.acc_hi;
  p.acc_cnt = l.acc_cnt;
  p.cur = l.cur;
  p.state = l.state;
  p.hdr = l.hdr;
  p.blocks_per_sm = plan.blocks_per_sm;
  p.wait_limit = kSpinLimit;   // the wait test applies to single images only
  p.wait_skip = -1;
  SG_TRY(reset_counters(l, plan.nimages, st));
  launch_pdl(init_kernel, dim3((plan.nimages + 255) / 256), dim3(256), 0, st, p);
  SG_TRY(launch_status());
  // one block per image (the kernel strides over images past 1024)
  const int cb = plan.nimages < 1024 ? plan.nimages : 1024;
  if (plan.dim == 3) launch_pdl(load_user_centroids<3>, dim3(cb), dim3(64), 0, st, p);
  else launch_pdl(load_user_centroids<5>, dim3(cb), dim3(64), 0, st, p);
  SG_TRY(launch_status());
  if (plan.max_iter <= 0) return SPLIT_OK;
  return dispatch<kCluster>(plan.layout, plan.dim, p, st);
}

}  // namespace sg

// ---------------------------------------------------------------------------
// Tuning table C API
// ---------------------------------------------------------------------------
extern "C" int split_tune_set(const split_tune_entry* entries, int n) {
  if (n < 0 || n > SPLIT_TUNE_MAX_ENTRIES || (n > 0 && !entries)) return SPLIT_ERR_INVALID;
  for (int i = 0; i < n; ++i) {
    const split_tune_entry& e = entries[i];
    if (e.max_pixels <= 0 || (i > 0 && e.max_pixels <= entries[i - 1].max_pixels))
      return SPLIT_ERR_INVALID;
    if (e.kmeans_unit_rows != 16 && e.kmeans_unit_rows != 32 && e.kmeans_unit_rows != 64 &&
        e.kmeans_unit_rows != 128)
      return SPLIT_ERR_INVALID;
    if (e.kmeans_blocks_per_sm < 0 || e.kmeans_blocks_per_sm > 8) return SPLIT_ERR_INVALID;
  }
  sg::km::TuneTable& t = sg::km::tune_table();
  std::lock_guard<std::mutex> g(t.m);
  t.e.assign(entries, entries + n);
  return SPLIT_OK;
}

extern "C" int split_tune_get(split_tune_entry* out, int capacity) {
  sg::km::TuneTable& t = sg::km::tune_table();
  std::lock_guard<std::mutex> g(t.m);
  const int n = (int)t.e.size();
  for (int i = 0; i < n && i < capacity && out; ++i) out[i] = t.e[i];
  return n;
}

// ---------------------------------------------------------------------------
// Centroids of many clusters (K > kMaxK): calculate_centroids on segment
// labels (samples/src/main.cu:293-294, :306-307 call it with K = the number
// of segments).  Per-cluster sums of the member features in the same 96-bit
// fixed point as the k-means update (each feature rounded to a multiple of
// 2^-24, low and high words added with 64-bit atomics), so the result is the
// same whatever order pixels are added in.  A warp whose 32 pixels share one
// label adds one warp sum; mixed warps add per pixel.  Means in FP64,
// rounded to FP32; a cluster without members keeps its input centroid.
// ---------------------------------------------------------------------------
namespace sg {
namespace segm {

constexpr int kThreads = 256;

struct Layout {
  WsHeader* hdr;
  unsigned long long* lo;   // [K][dim]
  unsigned long long* hi;   // [K][dim]
  unsigned* cnt;            // [K]
  size_t bytes;
};

inline Layout carve(void* ws, int K, int dim) {
  Carver c(ws);
  Layout l;
  l.hdr = c.take<WsHeader>(1);
  l.lo = c.take<unsigned long long>((size_t)K * dim);
  l.hi = c.take<unsigned long long>((size_t)K * dim);
  l.cnt = c.take<unsigned>((size_t)K);
  l.bytes = c.size();
  return l;
}

template <int LAYOUT, int DIM>
__global__ void __launch_bounds__(kThreads)
accumulate_kernel(const int32_t* __restrict__ labels, const void* __restrict__ points,
                  int64_t n, int width, float xy_scale, int K, Layout L) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  // every lane runs the same number of rounds (warp-wide shuffles below)
  const int64_t rounds = (n + stride - 1) / stride;
  for (int64_t r = 0; r < rounds; ++r) {
    const int64_t i = r * stride + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int l = -1;
    float f[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) f[d] = 0.0f;
    if (i < n) {
      l = __ldg(labels + i);
      if (l < 0 || l >= K) l = -1;
    }
    if (l >= 0) {
      if (LAYOUT == SPLIT_LAYOUT_FLOAT4) {
        const float4 v = __ldg(static_cast<const float4*>(points) + i);
        f[0] = v.x;
        f[1] = v.y;
        f[2] = v.z;
      } else if (LAYOUT == SPLIT_LAYOUT_RGB8) {
        const uint8_t* p = static_cast<const uint8_t*>(points) + 3 * i;
#pragma unroll
        for (int c = 0; c < 3; ++c) f[c] = __fdiv_rn((float)__ldg(p + c), 255.0f);
      } else {
        const float* p = static_cast<const float*>(points);
#pragma unroll
        for (int d = 0; d < DIM; ++d) f[d] = __ldg(p + (int64_t)d * n + i);
      }
      if (DIM == 5 && LAYOUT != SPLIT_LAYOUT_PLANAR) {
        const int64_t row = i / width;
        f[3] = __fmul_rn(xy_scale, (float)(i - row * width));
        f[4] = __fmul_rn(xy_scale, (float)row);
      }
    }
    unsigned long long qlo[DIM], qhi[DIM];
    fix::quantize<DIM>(f, l, &L.hdr->status, qlo, qhi);
    fix::warp_add<DIM>(l, qlo, qhi, L.lo, L.hi, L.cnt);
  }
}

__global__ void __launch_bounds__(kThreads)
finish_kernel(Layout L, int K, int dim, float* __restrict__ centroids) {
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < (int64_t)K * dim;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(idx / dim), d = (int)(idx - (int64_t)k * dim);
    const unsigned nk = L.cnt[k];
    if (nk == 0) continue;
    centroids[(int64_t)d * K + k] = fix::mean(L.lo[idx], L.hi[idx], nk);
  }
}

size_t workspace_bytes(int K, int dim) { return carve(nullptr, K, dim).bytes; }

int run(const int32_t* labels, const void* points, int layout, int dim, int64_t n, int width,
        float xy_scale, float* centroids, int K, void* ws, size_t ws_bytes, cudaStream_t st) {
  layout &= ~SPLIT_FEATURES_UNIT_RANGE;
  if (!labels || !points || !centroids || n <= 0 || n > 0x7fffffffLL || K < 1 || width < 1)
    return SPLIT_ERR_INVALID;
  if ((dim != 3 && dim != 5) || layout < SPLIT_LAYOUT_PLANAR || layout > SPLIT_LAYOUT_RGB8)
    return SPLIT_ERR_INVALID;
  if (layout == SPLIT_LAYOUT_FLOAT4 && (reinterpret_cast<uintptr_t>(points) & 15))
    return SPLIT_ERR_INVALID;
  Layout l = carve(nullptr, K, dim);
  if (!ws || ws_bytes < l.bytes || (reinterpret_cast<uintptr_t>(ws) & 255))
    return SPLIT_ERR_WORKSPACE;
  l = carve(ws, K, dim);
  SG_CUDA_TRY(cudaMemsetAsync(reinterpret_cast<char*>(l.hdr) + sizeof(int), 0,
                              l.bytes - sizeof(int), st));
  DeviceInfo di;
  SG_TRY(device_info(&di));
  int64_t blocks = (n + kThreads - 1) / kThreads;
  const int64_t cap = (int64_t)di.sm_count * 8;
  if (blocks > cap) blocks = cap;
#define SG_SEG_CASE(LY, D)                                                                 \
  if (layout == LY && dim == D) {                                                          \
    accumulate_kernel<LY, D><<<(int)blocks, kThreads, 0, st>>>(labels, points, n, width,  \
                                                               xy_scale, K, l);            \
  }
  SG_SEG_CASE(SPLIT_LAYOUT_PLANAR, 3)
  SG_SEG_CASE(SPLIT_LAYOUT_PLANAR, 5)
  SG_SEG_CASE(SPLIT_LAYOUT_FLOAT4, 3)
  SG_SEG_CASE(SPLIT_LAYOUT_FLOAT4, 5)
  SG_SEG_CASE(SPLIT_LAYOUT_RGB8, 3)
  SG_SEG_CASE(SPLIT_LAYOUT_RGB8, 5)
#undef SG_SEG_CASE
  SG_TRY(launch_status());
  int64_t fb = ((int64_t)K * dim + kThreads - 1) / kThreads;
  if (fb > cap) fb = cap;
  finish_kernel<<<(int)fb, kThreads, 0, st>>>(l, K, dim, centroids);
  return launch_status();
}

}  // namespace segm
}  // namespace sg
