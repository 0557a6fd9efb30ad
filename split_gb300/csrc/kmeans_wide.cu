// k-means with more clusters than the persistent kernel keeps in shared
// memory (64 < K <= 2^20): label_points (split/src/split/device/kmeans/
// label.cu:74-106) and cluster (cluster.cu:27-93), which set no limit on K.
//
// Assignment (assign_kernel): a warp takes 128 consecutive pixels per round
// (4 per lane, measured as two packed FP32x2 pairs), the block walks the
// centroids in shared-memory chunks of 32 KB (1024 centroids of 5
// dimensions, 2048 of 3), and each warp prunes them exactly with bounds over
// its pixels' feature box before measuring the survivors.  The squared distance is the reference's sum of
// (x - c)^2 in dimension order (label.cu:23-32) with one rounding per
// operation, and ties go to the lowest cluster index (strict < in ascending
// k, as the reference's argmin over the distance row, label.cu:98-105).  In
// a clustering the same pass adds every pixel's features to its cluster's
// fixed-point sums (fixsum.cuh), so the update reads no pixel again: for
// features below 2^32 as one 64-bit word per dimension, summed first over a
// lane's four pixels where the warp's 128 pixels share one label.
//
// Clustering: per iteration one assignment launch and one forming launch
// (form_kernel, one block), all max_iter pairs queued at once, each launch a
// programmatic dependent of the one before.  The forming launch turns the
// sums into means (FP64 division of the exact sum, rounded once to FP32; a
// cluster without members keeps its centroid), measures the centroid shift,
// and decides on the device whether the next iteration runs (|delta -
// old_delta| > threshold, cluster.cu:65-88).  After the stop, the launches
// still queued return at once.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "common.cuh"
#include "f32x2.cuh"
#include "fixsum.cuh"

namespace sg {
namespace kmw {

constexpr int kMinK = 65;                 // smaller K runs in the persistent kernel
constexpr int kMaxClusters = 1 << 20;
constexpr int kThreads = 256;
constexpr int kPix = 4;                   // pixels per thread and round (two pairs)
constexpr int kChunkF4 = 2048;            // float4 slots of one centroid chunk (32 KB)
constexpr int kFormThreads = 1024;

struct State {
  float delta;   // shift of the last formed iteration (0 before the first)
  int iters;     // iterations formed
  int done;      // no further iteration runs
  int pad;
};

struct Layout {
  WsHeader* hdr;
  State* state;
  float* cur;                // [2][DIM][K] planar: input centroids of odd / even iterations
  unsigned long long* lo;    // [K][DIM] low words of the fixed-point sums
  unsigned long long* hi;    // [K][DIM] high words (signed)
  unsigned* cnt;             // [K] member counts
  float* word;               // [3K] squared terms of the reference's shift
  size_t bytes;
};

inline Layout carve(void* ws, int K, int dim) {
  Carver c(ws);
  Layout l;
  l.hdr = c.take<WsHeader>(1);
  l.state = c.take<State>(1);
  l.cur = c.take<float>((size_t)2 * dim * K);
  l.lo = c.take<unsigned long long>((size_t)K * dim);
  l.hi = c.take<unsigned long long>((size_t)K * dim);
  l.cnt = c.take<unsigned>((size_t)K);
  l.word = c.take<float>((size_t)3 * K);
  l.bytes = c.size();
  return l;
}

struct Points {
  const void* pts;
  int64_t n;
  int width;
  float xy;      // xy_scale: dimension 3 and 4 of 5-D packed features
};

// Features of pixel i (i < n): RGB8 channels / 255, packed float4 .xyz or
// planar rows; 5-D packed features append xy * (column, row) of an image
// `width` pixels wide.
template <int LAYOUT, int DIM>
__device__ __forceinline__ void load_px(const Points& P, int64_t i, float (&f)[DIM]) {
  if (LAYOUT == SPLIT_LAYOUT_PLANAR) {
    const float* p = static_cast<const float*>(P.pts);
#pragma unroll
    for (int d = 0; d < DIM; ++d) f[d] = __ldg(p + d * P.n + i);
    return;
  }
  if (LAYOUT == SPLIT_LAYOUT_FLOAT4) {
    const float4 v = __ldg(static_cast<const float4*>(P.pts) + i);
    f[0] = v.x;
    f[1] = v.y;
    f[2] = v.z;
  } else {
    const uint8_t* p = static_cast<const uint8_t*>(P.pts) + 3 * i;
#pragma unroll
    for (int c = 0; c < 3; ++c) f[c] = __fdiv_rn((float)__ldg(p + c), 255.0f);
  }
  if (DIM == 5) {
    const int row = (int)i / P.width;
    const int col = (int)i - row * P.width;
    f[DIM == 5 ? 3 : 0] = __fmul_rn(P.xy, (float)col);
    f[DIM == 5 ? 4 : 0] = __fmul_rn(P.xy, (float)row);
  }
}

struct AssignArgs {
  Points P;
  int K;
  const float* cent;        // [DIM][K] planar
  int32_t* labels;
  const State* state;       // clustering: the launch returns once done is set
  unsigned long long* lo;
  unsigned long long* hi;
  unsigned* cnt;
  int* status;
};

// Order-preserving float -> int key (warp min / max of the box).
__device__ __forceinline__ int fkey(float x) {
  const int i = __float_as_int(x);
  return i ^ ((i >> 31) & 0x7fffffff);
}
__device__ __forceinline__ float fkey_inv(int k) {
  return __int_as_float(k ^ ((k >> 31) & 0x7fffffff));
}

// Squared distances of the pixel pair (p, q) to one centroid (c.x, c.y, c.z,
// c.w, c4), the reference's sum in dimension order, kept where it is below
// the pair's best so far (ties keep the lower index seen first).
template <int DIM>
__device__ __forceinline__ void closer(const float (&fp)[DIM], const float (&fq)[DIM],
                                       const float4 c, float c4, int k, float& bp, float& bq,
                                       int& kp, int& kq) {
  float2 t = fsub2(make_float2(fp[0], fq[0]), make_float2(c.x, c.x));
  float2 dd = fmul2(t, t);
  t = fsub2(make_float2(fp[1], fq[1]), make_float2(c.y, c.y));
  dd = ffma2(t, t, dd);
  t = fsub2(make_float2(fp[2], fq[2]), make_float2(c.z, c.z));
  dd = ffma2(t, t, dd);
  if (DIM == 5) {
    constexpr int X = DIM == 5 ? 3 : 0, Y = DIM == 5 ? 4 : 0;
    t = fsub2(make_float2(fp[X], fq[X]), make_float2(c.w, c.w));
    dd = ffma2(t, t, dd);
    t = fsub2(make_float2(fp[Y], fq[Y]), make_float2(c4, c4));
    dd = ffma2(t, t, dd);
  }
  if (dd.x < bp) {
    bp = dd.x;
    kp = k;
  }
  if (dd.y < bq) {
    bq = dd.y;
    kq = k;
  }
}

// A warp takes 128 consecutive pixels per round: lane l holds pixels
// base + 32 j + l, j < 4, so each of its four loads is coalesced and labels
// come in runs across the lanes for the fixed-point sums.
//
// Exact pruning per warp and round, over the box [lo, hi] of its 128
// pixels' features: for a centroid, LB = squared distance to the box (below
// every pixel's distance) and UB = squared distance to the farthest corner
// (above it).  thr = the smallest UB seen so far (over this chunk and the
// ones before) bounds every pixel's best distance, so a centroid whose LB
// exceeds thr by more than the 1e-4 relative margin is strictly farther than
// another centroid from every pixel, even after FP32 rounding (a few ulp),
// and is skipped: every argmin, ties included, is unchanged.  Lanes bound 32
// centroids at a time; the survivors of a ballot are then measured against
// the warp's pixels in ascending k, as pairs on the packed FP32x2 pipe.
template <int LAYOUT, int DIM, bool ACC>
__global__ void __launch_bounds__(kThreads, 3) assign_kernel(AssignArgs a) {
  constexpr int CS = DIM == 5 ? 2 : 1;          // float4 slots per centroid
  constexpr int kChunk = kChunkF4 / CS;         // centroids per chunk
  constexpr unsigned full = 0xffffffffu;
  __shared__ float4 cs[kChunkF4];
  __shared__ int stop;
  pdl_wait();
  if (ACC) {
    if (threadIdx.x == 0) stop = __ldcg(&a.state->done);
    __syncthreads();
    if (stop) return;
  }
  const int K = a.K;
  const int lane = threadIdx.x & 31;
  const int nchunks = (K + kChunk - 1) / kChunk;
  const int64_t warps = (int64_t)gridDim.x * (kThreads / 32);
  const int64_t gw = (int64_t)blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5);
  const int64_t rounds = (a.P.n + warps * 128 - 1) / (warps * 128);
  float* csf = reinterpret_cast<float*>(cs);

  auto load_chunk = [&](int ch) {
    const int k0 = ch * kChunk;
    const int kc = min(kChunk, K - k0);
    __syncthreads();
    for (int idx = threadIdx.x; idx < kc * DIM; idx += kThreads) {
      const int d = idx / kc, k = idx - d * kc;
      csf[k * (4 * CS) + d] = __ldg(a.cent + (int64_t)d * K + k0 + k);
    }
    __syncthreads();
  };
  if (nchunks == 1) load_chunk(0);

  for (int64_t r = 0; r < rounds; ++r) {
    const int64_t base = (r * warps + gw) * 128 + lane;
    float f[kPix][DIM];
    bool ok[kPix];
#pragma unroll
    for (int j = 0; j < kPix; ++j) {
      const int64_t i = base + 32 * j;
      ok[j] = i < a.P.n;
#pragma unroll
      for (int d = 0; d < DIM; ++d) f[j][d] = 0.0f;
      if (ok[j]) load_px<LAYOUT, DIM>(a.P, i, f[j]);
    }
    // box of the warp's pixels; fminf / fmaxf skip NaN (a NaN pixel's
    // distances all compare false, so it keeps label 0 whatever is skipped)
    float lo[DIM], hi[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      float x = INFINITY, z = -INFINITY;
#pragma unroll
      for (int j = 0; j < kPix; ++j) {
        if (ok[j]) {
          x = fminf(x, f[j][d]);
          z = fmaxf(z, f[j][d]);
        }
      }
      lo[d] = fkey_inv(__reduce_min_sync(full, fkey(x)));
      hi[d] = fkey_inv(__reduce_max_sync(full, fkey(z)));
    }
    float best[kPix];
    int bk[kPix];
#pragma unroll
    for (int j = 0; j < kPix; ++j) {
      best[j] = INFINITY;
      bk[j] = 0;
    }
    float ub_min = INFINITY;
    for (int ch = 0; ch < nchunks; ++ch) {
      if (nchunks > 1) load_chunk(ch);
      const int k0 = ch * kChunk;
      const int kc = min(kChunk, K - k0);
      // smallest UB over this chunk (and the chunks before)
      float um = ub_min;
      for (int k = lane; k < kc; k += 32) {
        float u = 0.0f;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
          const float c = csf[k * (4 * CS) + d];
          const float e = fmaxf(c - lo[d], hi[d] - c);
          u = __fmaf_rn(e, e, u);
        }
        um = fminf(um, u);
      }
      // UB >= 0: its bit pattern orders like the value
      ub_min = __int_as_float(__reduce_min_sync(full, __float_as_int(um)));
      const float thr = ub_min * 1.0001f;
      for (int g = 0; g < kc; g += 32) {
        const int k = g + lane;
        float l = __int_as_float(0x7fffffff);   // past the chunk: never a candidate
        if (k < kc) {
          l = 0.0f;
#pragma unroll
          for (int d = 0; d < DIM; ++d) {
            const float c = csf[k * (4 * CS) + d];
            const float gg = fmaxf(fmaxf(lo[d] - c, c - hi[d]), 0.0f);
            l = __fmaf_rn(gg, gg, l);
          }
        }
        unsigned m = __ballot_sync(full, l <= thr);
        while (m) {
          const int kk = g + __ffs(m) - 1;
          m &= m - 1;
          const float4 c = cs[kk * CS];
          const float c4 = DIM == 5 ? cs[kk * CS + (CS - 1)].x : 0.0f;
          closer<DIM>(f[0], f[1], c, c4, k0 + kk, best[0], best[1], bk[0], bk[1]);
          closer<DIM>(f[2], f[3], c, c4, k0 + kk, best[2], best[3], bk[2], bk[3]);
        }
      }
    }
#pragma unroll
    for (int j = 0; j < kPix; ++j)
      if (ok[j]) a.labels[base + 32 * j] = bk[j];
    if (ACC) {
      // Features below 2^32 (the common case by far): the narrow fixed-point
      // form, and where all 128 pixels share one label each lane first adds
      // its four pixels' words.  Otherwise the general form, pixel by pixel.
      bool small = true;
#pragma unroll
      for (int j = 0; j < kPix; ++j)
#pragma unroll
        for (int d = 0; d < DIM; ++d) small = small && (!ok[j] || fabsf(f[j][d]) < 4294967296.0f);
      const int b0 = __shfl_sync(full, bk[0], 0);   // every lane, before any branch
      bool one = ok[kPix - 1];                        // (ok[3] implies ok[0..2])
#pragma unroll
      for (int j = 1; j < kPix; ++j) one = one && bk[j] == bk[0];
      if (__all_sync(full, small)) {
        if (__all_sync(full, one && bk[0] == b0)) {
          long long q[DIM];
#pragma unroll
          for (int d = 0; d < DIM; ++d) {
            q[d] = 0;
#pragma unroll
            for (int j = 0; j < kPix; ++j) q[d] += __float2ll_rn(__fmul_rn(f[j][d], fix::kScale));
          }
          fix::warp_add_narrow<DIM>(b0, q, kPix, a.lo, a.hi, a.cnt);
        } else {
#pragma unroll
          for (int j = 0; j < kPix; ++j) {
            const int l = ok[j] ? bk[j] : -1;
            long long q[DIM];
#pragma unroll
            for (int d = 0; d < DIM; ++d)
              q[d] = l >= 0 ? __float2ll_rn(__fmul_rn(f[j][d], fix::kScale)) : 0ll;
            fix::warp_add_narrow<DIM>(l, q, 1u, a.lo, a.hi, a.cnt);
          }
        }
      } else {
#pragma unroll
        for (int j = 0; j < kPix; ++j) {
          unsigned long long qlo[DIM], qhi[DIM];
          const int l = ok[j] ? bk[j] : -1;
          fix::quantize<DIM>(f[j], l, a.status, qlo, qhi);
          fix::warp_add<DIM>(l, qlo, qhi, a.lo, a.hi, a.cnt);
        }
      }
    }
  }
}

// Initial state, the caller's centroids into cur[0], zero sums.
__global__ void setup_kernel(Layout L, int K, int dim, const float* __restrict__ cent,
                             int32_t* d_iter, int max_iter) {
  pdl_wait();
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nt = (int64_t)gridDim.x * blockDim.x;
  if (t == 0) {
    State s;
    s.delta = 0.0f;
    s.iters = 0;
    s.done = max_iter <= 0;
    s.pad = 0;
    *L.state = s;
    if (d_iter && max_iter <= 0) *d_iter = 0;
  }
  const int64_t kd = (int64_t)K * dim;
  for (int64_t i = t; i < kd; i += nt) {
    L.cur[i] = cent[i];
    L.lo[i] = 0ull;
    L.hi[i] = 0ull;
  }
  for (int64_t k = t; k < K; k += nt) L.cnt[k] = 0u;
}

struct FormArgs {
  Layout L;
  Points P;
  int K;
  int i;                    // iteration being formed (1-based)
  int max_iter;
  float threshold;
  int ref_shift;            // the reference's shift measure (3-D only)
  float* centroids;         // the caller's [DIM][K], written when the run stops
  int32_t* d_iter;
};

// Centroids of iteration i from the sums of its assignment, the shift, the
// decision.  One block: every sum is read once and cleared for the next
// iteration.  The L2 shift is summed in a fixed order (per-thread strided
// partials, then a fixed tree), so it does not vary between runs.
//
// With ref_shift the shift is the reference's own measure (cluster.cu:40-50,
// :73-87): it compares the new planar centroids, entry j = d * K + k, with
// the words its workspace holds at float offset 2N at that point, which are
//   j < K:  1 / n_j (centroids.cu:40-63 writes the reciprocal sizes there);
//   j >= K: the distance of point (2N + j) / K to centroid (2N + j) % K of
//           the iteration's input (label.cu:80-88 writes the N x K distance
//           matrix from offset 0), sum of squares in dimension order;
// and sums (c_new[j] - word[j])^2 in FP32 in j order.
template <int LAYOUT, int DIM>
__global__ void __launch_bounds__(kFormThreads) form_kernel(FormArgs a) {
  __shared__ float part[kFormThreads];
  __shared__ int stop, more;
  pdl_wait();
  if (threadIdx.x == 0) stop = __ldcg(&a.L.state->done);
  __syncthreads();
  if (stop) return;
  const int K = a.K;
  const int64_t kd = (int64_t)K * DIM;
  const float* c_old = a.L.cur + (size_t)((a.i - 1) & 1) * kd;
  float* c_new = a.L.cur + (size_t)(a.i & 1) * kd;
  float acc = 0.0f;
  for (int64_t idx = threadIdx.x; idx < kd; idx += kFormThreads) {
    const int d = (int)(idx / K), k = (int)(idx - (int64_t)d * K);
    const float c = c_old[idx];
    const unsigned n = __ldcg(a.L.cnt + k);
    const size_t s = (size_t)k * DIM + d;
    const float cn = n ? fix::mean(__ldcg(a.L.lo + s), __ldcg(a.L.hi + s), n) : c;
    a.L.lo[s] = 0ull;
    a.L.hi[s] = 0ull;
    c_new[idx] = cn;
    const float df = __fsub_rn(cn, c);
    acc = __fadd_rn(acc, __fmul_rn(df, df));
  }
  part[threadIdx.x] = acc;
  __syncthreads();   // every c_new entry written
  if (DIM == 3 && a.ref_shift) {
    const int64_t base = 2 * a.P.n;
    for (int64_t j = threadIdx.x; j < 3 * (int64_t)K; j += kFormThreads) {
      float word;
      if (j < K) {
        word = __fdiv_rn(1.0f, (float)__ldcg(a.L.cnt + j));
      } else {
        const int64_t e = base + j;
        const int64_t px = e / K;
        const int c = (int)(e - px * K);
        float f[DIM];
        load_px<LAYOUT, DIM>(a.P, px, f);
        float w = 0.0f;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
          const float t = __fsub_rn(f[d], c_old[(int64_t)d * K + c]);
          w = d == 0 ? __fmul_rn(t, t) : __fadd_rn(w, __fmul_rn(t, t));
        }
        word = w;
      }
      const float t = __fsub_rn(c_new[j], word);
      a.L.word[j] = __fmul_rn(t, t);
    }
  }
  __syncthreads();
  for (int s = kFormThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) part[threadIdx.x] = __fadd_rn(part[threadIdx.x], part[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    float sq = part[0];
    if (DIM == 3 && a.ref_shift) {
      sq = 0.0f;
      for (int64_t j = 0; j < 3 * (int64_t)K; ++j) sq = __fadd_rn(sq, a.L.word[j]);
    }
    const float delta = sqrtf(sq);
    const float old_delta = a.L.state->delta;
    const bool m = a.i < a.max_iter && fabsf(delta - old_delta) > a.threshold;
    a.L.state->delta = delta;
    a.L.state->iters = a.i;
    if (!m) {
      a.L.state->done = 1;
      if (a.d_iter) *a.d_iter = a.i;
    }
    more = m ? 1 : 0;
  }
  __syncthreads();
  if (!more)
    for (int64_t idx = threadIdx.x; idx < kd; idx += kFormThreads) a.centroids[idx] = c_new[idx];
  for (int k = threadIdx.x; k < K; k += kFormThreads) a.L.cnt[k] = 0u;
}

size_t workspace_bytes(int K, int dim) { return carve(nullptr, K, dim).bytes; }

template <int LAYOUT, int DIM>
static int queue(bool cluster, const Points& P, int K, const float* cent, float* centroids,
                 int32_t* labels, const Layout& L, int max_iter, float threshold, int ref_shift,
                 int32_t* d_iter, cudaStream_t st) {
  DeviceInfo di;
  SG_TRY(device_info(&di));
  int per_sm = 0;
  auto ak = cluster ? assign_kernel<LAYOUT, DIM, true> : assign_kernel<LAYOUT, DIM, false>;
  SG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ak, kThreads, 0));
  if (per_sm < 1) return SPLIT_ERR_UNSUPPORTED;
  int64_t blocks = (P.n + (int64_t)kThreads * kPix - 1) / ((int64_t)kThreads * kPix);
  const int64_t cap = (int64_t)di.sm_count * per_sm;
  if (blocks > cap) blocks = cap;
  AssignArgs aa{};
  aa.P = P;
  aa.K = K;
  aa.labels = labels;
  aa.state = L.state;
  aa.lo = L.lo;
  aa.hi = L.hi;
  aa.cnt = L.cnt;
  aa.status = &L.hdr->status;
  if (!cluster) {
    aa.cent = cent;
    SG_CUDA_TRY(launch_pdl(ak, dim3((unsigned)blocks), dim3(kThreads), 0, st, aa));
    return launch_status();
  }
  int64_t sb = ((int64_t)K * DIM + 255) / 256;
  if (sb > di.sm_count * 4) sb = di.sm_count * 4;
  SG_CUDA_TRY(launch_pdl(setup_kernel, dim3((unsigned)sb), dim3(256), 0, st, L, K, DIM, cent,
                         d_iter, max_iter));
  SG_TRY(launch_status());
  FormArgs fa{};
  fa.L = L;
  fa.P = P;
  fa.K = K;
  fa.max_iter = max_iter;
  fa.threshold = threshold;
  fa.ref_shift = ref_shift;
  fa.centroids = centroids;
  fa.d_iter = d_iter;
  const size_t kd = (size_t)K * DIM;
  for (int i = 1; i <= max_iter; ++i) {
    aa.cent = L.cur + (size_t)((i - 1) & 1) * kd;
    SG_CUDA_TRY(launch_pdl(ak, dim3((unsigned)blocks), dim3(kThreads), 0, st, aa));
    SG_TRY(launch_status());
    fa.i = i;
    SG_CUDA_TRY(launch_pdl(form_kernel<LAYOUT, DIM>, dim3(1), dim3(kFormThreads), 0, st, fa));
    SG_TRY(launch_status());
  }
  return SPLIT_OK;
}

int run(bool cluster, const void* points, int layout, int dim, int64_t n, int width,
        float xy_scale, float* centroids, const float* cent_in, int K, int32_t* labels,
        void* ws, size_t ws_bytes, int max_iter, float threshold, int32_t* d_iter,
        cudaStream_t st) {
  const int ref_shift = (layout & SPLIT_KMEANS_REFERENCE_SHIFT) ? 1 : 0;
  layout &= ~(SPLIT_FEATURES_UNIT_RANGE | SPLIT_KMEANS_REFERENCE_SHIFT);
  if (!points || !cent_in || !labels || n <= 0 || n > 0x7fffffffLL || width < 1)
    return SPLIT_ERR_INVALID;
  if (K < kMinK || K > kMaxClusters || (dim != 3 && dim != 5)) return SPLIT_ERR_INVALID;
  if (layout < SPLIT_LAYOUT_PLANAR || layout > SPLIT_LAYOUT_RGB8) return SPLIT_ERR_INVALID;
  if (layout == SPLIT_LAYOUT_FLOAT4 && (reinterpret_cast<uintptr_t>(points) & 15))
    return SPLIT_ERR_INVALID;
  // the reference's shift: 3-D clustering, every word it reads inside the
  // N x K distance matrix
  if (ref_shift && (!cluster || dim != 3 || n * (K - 2) < 3 * (int64_t)K))
    return SPLIT_ERR_INVALID;
  Layout l = carve(nullptr, K, dim);
  if (!ws || ws_bytes < l.bytes || (reinterpret_cast<uintptr_t>(ws) & 255))
    return SPLIT_ERR_WORKSPACE;
  l = carve(ws, K, dim);
  const Points P{points, n, width, xy_scale};
  if (cluster && max_iter <= 0) max_iter = 0;
#define SG_KMW_CASE(LY, D)                                                                  \
  if (layout == LY && dim == D)                                                             \
    return queue<LY, D>(cluster, P, K, cent_in, centroids, labels, l, max_iter, threshold,  \
                        ref_shift, d_iter, st);
  SG_KMW_CASE(SPLIT_LAYOUT_PLANAR, 3)
  SG_KMW_CASE(SPLIT_LAYOUT_PLANAR, 5)
  SG_KMW_CASE(SPLIT_LAYOUT_FLOAT4, 3)
  SG_KMW_CASE(SPLIT_LAYOUT_FLOAT4, 5)
  SG_KMW_CASE(SPLIT_LAYOUT_RGB8, 3)
  SG_KMW_CASE(SPLIT_LAYOUT_RGB8, 5)
#undef SG_KMW_CASE
  return SPLIT_ERR_INVALID;
}

}  // namespace kmw
}  // namespace sg
