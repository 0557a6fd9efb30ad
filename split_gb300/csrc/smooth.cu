// Smooth-boundary merge: segments join the adjacent segment across whose
// shared boundary the features change least.
//
// Restates the documented behaviour of split/src/split/device/ccl/
// merge_smooth_boundaries.cu:134-243:
//   * directed 8-neighbour edges (p, q) between pixels of different labels,
//     the image border excluded (segment_adjacency.cu:112-142, :170-254);
//   * per segment pair (s, t): the number of such edges and the mean over
//     them of |x_p - x_q| (Euclidean norm of feature rows 0..2, in FP32,
//     VecNorm :25-35), averaged per pair (:176-186);
//   * pairs with mean >= D or with 15 edges or fewer are dropped (:197-205),
//     D = threshold * max_i |x_i| (:193-195, max_colwise_norm :37-55);
//   * every segment with candidates maps to the one with the smallest
//     (mean, id) (:207-226: "if we are faced with multiple options, we take
//     the smallest scalar"); mutual pairs keep the larger id
//     (fix_map_cycles.cuh:14-44) and labels follow their map chains to the
//     end (map_until_converged.cuh:14-31).
// The reference file does not compile as written (its reduce_by_key is given
// thrust::less, a predicate, as the reduction), so the stated intent above
// is what this restates.
//
// Pair statistics live in an open-addressing table (key (s, t), edge count,
// 96-bit fixed-point sum of the edge norms at scale 2^32), so the means do
// not depend on the order edges are added in.  Bids are one 64-bit atomicMax
// per pair on ~((bits(mean) << 32) | t).
#include "geom.cuh"

namespace sg {
namespace smooth {

constexpr int kThreads = 256;
constexpr int kProbeCap = 1 << 16;
constexpr unsigned kChainCap = 1u << 24;

struct Layout {
  WsHeader* hdr;
  unsigned* maxsq;              // bits of the largest |x|^2 (non-negative float)
  unsigned* list_count;
  unsigned long long* best;     // [n] winning bid per segment, 0 = none
  int32_t* map;                 // [n]
  int32_t* fin;                 // [n]
  unsigned long long* keys;     // [cap]
  unsigned* counts;             // [cap]
  unsigned long long* dlo;      // [cap] low 32-bit words of the norm sums
  unsigned long long* dhi;      // [cap] high words
  int32_t* list;                // [cap] claimed slots
  int cap_log2;
  size_t bytes;
};

inline int cap_log2_for(int64_t n) {
  int l = 12;
  while ((1ll << l) < 2 * n && l < 31) ++l;
  return l;
}

inline Layout carve(void* ws, int64_t n) {
  Carver c(ws);
  Layout l;
  l.hdr = c.take<WsHeader>(1);
  l.maxsq = c.take<unsigned>(1);
  l.list_count = c.take<unsigned>(1);
  l.best = c.take<unsigned long long>((size_t)n);
  l.map = c.take<int32_t>((size_t)n);
  l.fin = c.take<int32_t>((size_t)n);
  l.cap_log2 = cap_log2_for(n);
  const size_t cap = (size_t)1 << l.cap_log2;
  l.keys = c.take<unsigned long long>(cap);
  l.counts = c.take<unsigned>(cap);
  l.dlo = c.take<unsigned long long>(cap);
  l.dhi = c.take<unsigned long long>(cap);
  l.list = c.take<int32_t>(cap);
  l.bytes = c.size();
  return l;
}

__device__ __forceinline__ unsigned long long pair_key(int s, int t) {
  return (((unsigned long long)(unsigned)s << 32) | (unsigned)t) + 1ull;
}
__device__ __forceinline__ int key_s(unsigned long long k) { return (int)((k - 1ull) >> 32); }
__device__ __forceinline__ int key_t(unsigned long long k) {
  return (int)(unsigned)((k - 1ull) & 0xffffffffull);
}

// |x_p - x_q| over feature rows 0..2, the sum of squares in row order
__device__ __forceinline__ float edge_norm(const float* pts, long long n, long long p,
                                           long long q) {
  float s = 0.0f;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float v = __fsub_rn(__ldg(pts + d * n + p), __ldg(pts + d * n + q));
    s = __fadd_rn(s, __fmul_rn(v, v));
  }
  return __fsqrt_rn(s);
}

__device__ void insert(const Layout& L, int s, int t, unsigned m, unsigned long long lo,
                       unsigned long long hi, int* status) {
  const unsigned long long key = pair_key(s, t);
  const unsigned mask = (1u << L.cap_log2) - 1u;
  unsigned h = (unsigned)((key * 0x9E3779B97F4A7C15ull) >> (64 - L.cap_log2));
  for (int probe = 0; probe < kProbeCap; ++probe, h = (h + 1) & mask) {
    unsigned long long k = *(volatile unsigned long long*)(L.keys + h);
    if (k == 0ull) {
      k = atomicCAS(L.keys + h, 0ull, key);
      if (k == 0ull) {
        const unsigned idx = atomicAdd(L.list_count, 1u);
        L.list[idx] = (int)h;
        k = key;
      }
    }
    if (k == key) {
      atomicAdd(L.counts + h, m);
      atomicAdd(L.dlo + h, lo);
      atomicAdd(L.dhi + h, hi);
      return;
    }
  }
  set_status(status, SPLIT_ERR_OVERFLOW);
}

__global__ void __launch_bounds__(kThreads)
maxnorm_kernel(const float* __restrict__ pts, long long n, Layout L) {
  unsigned best = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    float s = 0.0f;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const float v = __ldg(pts + d * n + i);
      s = __fadd_rn(s, __fmul_rn(v, v));
    }
    // non-negative floats order like their bit patterns (NaN is skipped)
    if (s >= 0.0f) best = max(best, __float_as_uint(s));
  }
  best = __reduce_max_sync(0xffffffffu, best);
  if ((threadIdx.x & 31) == 0) atomicMax(L.maxsq, best);
}

// one block per 32 x 64 tile: every pixel adds its out-going boundary edges,
// aggregated per distinct neighbour label
__global__ void __launch_bounds__(kThreads)
edge_kernel(const int32_t* __restrict__ lab, const float* __restrict__ pts, Geoms gs, Layout L,
            int* status) {
  const long long n = gs.total_px;
  const TileRef tr = tile_ref(gs, blockIdx.x);
  const int W = tr.W, H = tr.H;
  for (int q = threadIdx.x; q < kTileH * kTileW; q += blockDim.x) {
    const int x = tr.tx0 + q % kTileW, y = tr.ty0 + q / kTileW;
    if (x >= W || y >= H) continue;
    const long long i = tr.off + (long long)y * W + x;
    const int s = __ldg(lab + i);
    if (s < 0 || s >= n) {
      set_status(status, SPLIT_ERR_INVALID);
      continue;
    }
    int t[8];
    long long j[8];
    int nt = 0;
#pragma unroll
    for (int d = 0; d < 8; ++d) {
      const int dx = (d == 0 || d == 3 || d == 5) ? -1 : (d == 2 || d == 4 || d == 7) ? 1 : 0;
      const int dy = d < 3 ? -1 : d > 4 ? 1 : 0;
      const int nx = x + dx, ny = y + dy;
      if (nx < 0 || ny < 0 || nx >= W || ny >= H) continue;
      const long long k = tr.off + (long long)ny * W + nx;
      const int v = __ldg(lab + k);
      if (v < 0 || v >= n) {
        set_status(status, SPLIT_ERR_INVALID);
        continue;
      }
      if (v != s) {
        t[nt] = v;
        j[nt] = k;
        ++nt;
      }
    }
    for (int a = 0; a < nt; ++a) {
      bool first = true;
      for (int b = 0; b < a; ++b) first &= (t[b] != t[a]);
      if (!first) continue;
      unsigned m = 0;
      unsigned long long slo = 0, shi = 0;
      for (int b = a; b < nt; ++b) {
        if (t[b] != t[a]) continue;
        ++m;
        const float e = edge_norm(pts, n, i, j[b]);
        if (!(e < 1073741824.0f)) set_status(status, SPLIT_ERR_OVERFLOW);   // 2^30, or NaN
        const long long q = __float2ll_rn(__fmul_rn(e, 4294967296.0f));
        slo += (unsigned long long)q & 0xffffffffull;
        shi += (unsigned long long)(q >> 32);
      }
      insert(L, s, t[a], m, slo, shi, status);
    }
  }
}

// mean edge norm of a slot, rounded to FP32 (the reference keeps it as real);
// edge norms are below 2^30, so the high words sum to below 2^62
__device__ __forceinline__ float slot_mean(const Layout& L, int h) {
  const double hi = (double)(long long)L.dhi[h];
  const double lo = (double)L.dlo[h];
  const double S = __dadd_rn(__dmul_rn(hi, 4294967296.0), lo);
  return __double2float_rn(__ddiv_rn(__dmul_rn(S, 1.0 / 4294967296.0), (double)L.counts[h]));
}

__device__ void bid_phase(const Layout& L, float threshold) {
  const unsigned cnt = *(volatile unsigned*)L.list_count;
  const float D = __fmul_rn(threshold, __fsqrt_rn(__uint_as_float(*(volatile unsigned*)L.maxsq)));
  for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < cnt; j += gridDim.x * blockDim.x) {
    const int h = L.list[j];
    const unsigned long long k = L.keys[h];
    const int s = key_s(k), t = key_t(k);
    const float d = slot_mean(L, h);
    if (!(d < D) || L.counts[h] <= 15u) continue;
    atomicMax(L.best + s, ~(((unsigned long long)__float_as_uint(d) << 32) | (unsigned)t));
  }
}

__device__ __forceinline__ int bid_target(unsigned long long b) {
  return (int)(unsigned)((~b) & 0xffffffffull);
}

__device__ void decide_phase(const Layout& L) {
  const unsigned cnt = *(volatile unsigned*)L.list_count;
  for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < cnt; j += gridDim.x * blockDim.x) {
    const unsigned long long k = L.keys[L.list[j]];
    const int s = key_s(k), t = key_t(k);
    const unsigned long long b = L.best[s];
    if (b && bid_target(b) == t) L.map[s] = t;
  }
}

__device__ __forceinline__ int next_of(const Layout& L, int n, int r) {
  if (*(volatile unsigned long long*)(L.best + r) == 0ull) return r;
  const int nx = *(volatile int*)(L.map + r);
  if (nx < 0 || nx >= n) {
    set_status(&L.hdr->status, SPLIT_ERR_INVALID);
    return r;
  }
  return nx;
}

// mutual pairs: the larger id keeps itself
__device__ void cycle_phase(const Layout& L, int n) {
  const unsigned cnt = *(volatile unsigned*)L.list_count;
  for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < cnt; j += gridDim.x * blockDim.x) {
    const unsigned long long k = L.keys[L.list[j]];
    const int s = key_s(k), t = key_t(k);
    const unsigned long long b = L.best[s];
    if (!b || bid_target(b) != t) continue;
    if (next_of(L, n, t) == s && s > t) *(volatile int*)(L.map + s) = s;
  }
}

__device__ void resolve_phase(const Layout& L, int n) {
  const unsigned cnt = *(volatile unsigned*)L.list_count;
  for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < cnt; j += gridDim.x * blockDim.x) {
    const unsigned long long k = L.keys[L.list[j]];
    const int s = key_s(k), t = key_t(k);
    const unsigned long long b = L.best[s];
    if (!b || bid_target(b) != t) continue;
    int r = s;
    for (unsigned steps = 0;; ++steps) {
      const int nx = next_of(L, n, r);
      if (nx == r) break;
      r = nx;
      if (steps > kChainCap) {
        set_status(&L.hdr->status, SPLIT_ERR_NOT_CONVERGED);
        break;
      }
    }
    L.fin[s] = r;
  }
}

// The decision over the (segment, neighbour) list, one cooperative launch (one
// block per SM): bids, decisions, mutual-pair fix, chains, each phase behind a
// bounded grid barrier.
__global__ void __launch_bounds__(kThreads) list_kernel(Layout L, float threshold, int n) {
  bid_phase(L, threshold);
  if (!grid_barrier(L.hdr)) return;
  decide_phase(L);
  if (!grid_barrier(L.hdr)) return;
  cycle_phase(L, n);
  if (!grid_barrier(L.hdr)) return;
  resolve_phase(L, n);
}

__global__ void __launch_bounds__(kThreads)
relabel_kernel(int32_t* __restrict__ lab, long long n, Layout L) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int v = lab[i];
    if (v < 0 || v >= n) continue;
    if (L.best[v]) lab[i] = L.fin[v];
  }
}

// table slots and bids back to zero for the next call
__global__ void cleanup_kernel(Layout L) {
  const unsigned cnt = *(volatile unsigned*)L.list_count;
  for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < cnt; j += gridDim.x * blockDim.x) {
    const int h = L.list[j];
    const int s = key_s(L.keys[h]);
    L.best[s] = 0ull;
    L.keys[h] = 0ull;
    L.counts[h] = 0u;
    L.dlo[h] = 0ull;
    L.dhi[h] = 0ull;
  }
}

}  // namespace smooth
}  // namespace sg

using namespace sg;

extern "C" size_t split_merge_smooth_workspace_size(int width, int height) {
  if (width < 1 || height < 1) return 0;
  return smooth::carve(nullptr, (int64_t)width * height).bytes;
}

extern "C" int split_merge_smooth(int32_t* labels, int width, int height, const float* points,
                                  float threshold, void* workspace, size_t workspace_bytes,
                                  void* stream) {
  using namespace sg::smooth;
  if (!labels || !points || width < 1 || height < 1) return SPLIT_ERR_INVALID;
  const int64_t n = (int64_t)width * height;
  if (n > 0x7fffffffLL || !(threshold >= 0.0f)) return SPLIT_ERR_INVALID;
  Layout l = carve(nullptr, n);
  if (!workspace || workspace_bytes < l.bytes || (reinterpret_cast<uintptr_t>(workspace) & 255))
    return SPLIT_ERR_WORKSPACE;
  l = carve(workspace, n);
  cudaStream_t st = as_stream(stream);
  // header words after the status, the norm maximum and the slot counter
  // start at zero; the table and the bids are kept clean by cleanup_kernel
  // (a fresh workspace is zero-filled by its owner)
  SG_CUDA_TRY(cudaMemsetAsync(reinterpret_cast<char*>(l.hdr) + sizeof(int), 0,
                              reinterpret_cast<char*>(l.best) -
                                  reinterpret_cast<char*>(l.hdr) - sizeof(int), st));
  DeviceInfo di;
  SG_TRY(device_info(&di));
  const Geoms gs = single_geom(width, height);
  int64_t blocks = (n + kThreads - 1) / kThreads;
  const int64_t cap = (int64_t)di.sm_count * 8;
  if (blocks > cap) blocks = cap;
  maxnorm_kernel<<<(int)blocks, kThreads, 0, st>>>(points, n, l);
  SG_TRY(launch_status());
  edge_kernel<<<gs.total_tiles, kThreads, 0, st>>>(labels, points, gs, l, &l.hdr->status);
  SG_TRY(launch_status());
  const int grid = di.sm_count * 4;
  {
    // one co-resident block per SM; the header clear above zeroed the barrier
    int per_sm = 0;
    SG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, list_kernel, kThreads, 0));
    if (per_sm < 1) return SPLIT_ERR_UNSUPPORTED;
    float thr = threshold;
    int n32 = (int)n;
    void* args[] = {&l, &thr, &n32};
    SG_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)list_kernel, dim3(di.sm_count),
                                            dim3(kThreads), args, 0, st));
  }
  SG_TRY(launch_status());
  relabel_kernel<<<(int)blocks, kThreads, 0, st>>>(labels, n, l);
  SG_TRY(launch_status());
  cleanup_kernel<<<grid, kThreads, 0, st>>>(l);
  return launch_status();
}
