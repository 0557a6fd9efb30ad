// Connected-component labelling of an int32 label image, 4- or 8-connected,
// by block-local union-find in shared memory followed by a global root merge
// across tile borders and a path-compression pass.
//
// Restates the fixed point of split/src/split/device/ccl/
// connected_components.cu:80-181 (iterated max propagation along row runs and
// column runs, i.e. 4-connectivity, until every pixel holds the maximum
// linear index of its component).  Union-find reaches that fixed point in
// three passes instead of one round per path turn.  The label of a component
// is its minimum (SPLIT_LABEL_MIN_INDEX) or maximum (SPLIT_LABEL_MAX_INDEX,
// the reference) linear pixel index.
//
// Passes (labels_out doubles as the global parent array):
//   tile   : one block per TH x TW tile; labels staged in shared memory; local
//            union-find on shared parents; every pixel writes the global
//            index of its local root; local roots clear their size counter.
//   border : per tile, edges to earlier tiles (W, NW, N, NE across the tile
//            edge) are merged with lock-free atomicMin/atomicMax hooking.
//   flatten: every pixel follows its parent chain to the root and stores it
//            (in place; a concurrent reader sees an ancestor either way);
//            optional per-component pixel counts, aggregated per warp.
//
// compress_labels (compress_labels.cu:10-35) is a flag / scan / gather over
// the label range [-1, n).
#include "geom.cuh"

namespace sg {
namespace ccl {

constexpr int TH = kTileH, TW = kTileW, kThreads = 256;
constexpr unsigned kUnionCap = 1u << 22;

template <bool MAXC>
__device__ __forceinline__ bool better(int a, int b) {
  return MAXC ? a > b : a < b;
}

// ---- shared-memory union-find --------------------------------------------
// Find with path halving.  Safe next to concurrent hooking: a halving store
// only ever points a node at one of its ancestors, and a hook that loses such
// a race is retried by sunite with the node's new parent.
__device__ __forceinline__ int sfind(volatile int* par, int x) {
  int p = par[x];
  while (p != x) {
    const int gp = par[p];
    if (gp != p) par[x] = gp;
    x = p;
    p = par[x];
  }
  return x;
}

template <bool MAXC>
__device__ __forceinline__ void sunite(int* par, int a, int b, int* status) {
  volatile int* vp = par;
  for (unsigned it = 0; it < kUnionCap; ++it) {
    a = sfind(vp, a);
    b = sfind(vp, b);
    if (a == b) return;
    // hook the worse root under the better one
    const int lo = better<MAXC>(a, b) ? a : b;
    const int hi = better<MAXC>(a, b) ? b : a;
    const int old = MAXC ? atomicMax(par + hi, lo) : atomicMin(par + hi, lo);
    if (old == hi) return;
    a = old;
    b = lo;
  }
  set_status(status, SPLIT_ERR_NOT_CONVERGED);
}

// ---- global union-find (parents in labels_out) -----------------------------
__device__ __forceinline__ int gfind(const int* P, int x, unsigned& budget) {
  int p = __ldcg(P + x);
  while (p != x && budget) {
    x = p;
    p = __ldcg(P + x);
    --budget;
  }
  return x;
}

template <bool MAXC>
__device__ void gunite(int* P, int a, int b, int* status) {
  unsigned budget = kUnionCap;
  for (unsigned it = 0; it < kUnionCap && budget; ++it) {
    a = gfind(P, a, budget);
    b = gfind(P, b, budget);
    if (a == b) return;
    const int lo = better<MAXC>(a, b) ? a : b;
    const int hi = better<MAXC>(a, b) ? b : a;
    const int old = MAXC ? atomicMax(P + hi, lo) : atomicMin(P + hi, lo);
    if (old == hi) return;
    a = old;
    b = lo;
  }
  set_status(status, SPLIT_ERR_NOT_CONVERGED);
}

// Tile pass.  Thread t owns 8 consecutive pixels of row t / 8; runs of equal
// label inside those 8 pixels are linked without atomics, and a union is only
// issued where run adjacency does not already imply it:
//   W  : only at the first pixel of a thread's 8 (other W links are runs);
//   N  : unless W and NW both carry the label (the NW/N run already joins);
//   NW : only if neither W nor N carries the label;
//   NE : only if N does not carry the label and E (in the tile) does not
//        either (E's own N link covers NE).
template <bool MAXC, int CONN>
__global__ void __launch_bounds__(kThreads)
tile_kernel(const int32_t* __restrict__ in, Geoms gs, int* __restrict__ P,
            int32_t* __restrict__ sizes, int* status) {
  static_assert(TW == 64 && TH * TW == kThreads * 8, "8 pixels per thread");
  __shared__ int lab[TH * TW];
  __shared__ int par[TH * TW];
  const TileRef t = tile_ref(gs, blockIdx.x);
  const int W = t.W, H = t.H, tx0 = t.tx0, ty0 = t.ty0;
  const long long off = t.off;
  const int tw = min(TW, W - tx0), th = min(TH, H - ty0);
  for (int i = threadIdx.x; i < TH * TW; i += kThreads) {
    const int r = i / TW, c = i % TW;
    lab[i] = (r < th && c < tw) ? __ldg(in + off + (long long)(ty0 + r) * W + tx0 + c) : 0;
  }
  __syncthreads();
  const int r = threadIdx.x >> 3, c0 = (threadIdx.x & 7) * 8;
  const int base = r * TW + c0;
  {
    // runs point at their best pixel: the first (minimum index convention)
    // or the last (maximum index convention)
    const bool ok_row = r < th;
    if (!MAXC) {
      int run = base;
      par[base] = base;
#pragma unroll
      for (int j = 1; j < 8; ++j) {
        const int i = base + j;
        if (!(ok_row && c0 + j < tw) || lab[i] != lab[i - 1]) run = i;
        par[i] = run;
      }
    } else {
      int run = base + 7;
      par[base + 7] = base + 7;
#pragma unroll
      for (int j = 6; j >= 0; --j) {
        const int i = base + j;
        if (!(ok_row && c0 + j + 1 < tw) || lab[i] != lab[i + 1]) run = i;
        par[i] = run;
      }
    }
  }
  __syncthreads();
  if (r < th) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int c = c0 + j;
      if (c >= tw) break;
      const int i = base + j;
      const int v = lab[i];
      const bool hasW = c > 0 && lab[i - 1] == v;
      if (j == 0 && hasW) sunite<MAXC>(par, i, i - 1, status);
      if (r > 0) {
        const bool n = lab[i - TW] == v;
        const bool nw = c > 0 && lab[i - TW - 1] == v;
        if (n && !(hasW && nw)) sunite<MAXC>(par, i, i - TW, status);
        if (CONN == 8) {
          if (nw && !hasW && !n) sunite<MAXC>(par, i, i - TW - 1, status);
          const bool ne = c + 1 < tw && lab[i - TW + 1] == v;
          const bool e = c + 1 < tw && lab[i + 1] == v;
          if (ne && !n && !e) sunite<MAXC>(par, i, i - TW + 1, status);
        }
      }
    }
  }
  __syncthreads();
  if (r < th) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int c = c0 + j;
      if (c >= tw) break;
      const int i = base + j;
      const int root = sfind(par, i);
      const long long g = off + (long long)(ty0 + r) * W + tx0 + c;
      P[g] = (int)(off + (long long)(ty0 + root / TW) * W + tx0 + root % TW);
      if (sizes && root == i) sizes[g] = 0;
    }
  }
}

template <bool MAXC, int CONN>
__global__ void __launch_bounds__(kThreads)
border_kernel(const int32_t* __restrict__ in, Geoms gs, int* P, int* status) {
  const TileRef t = tile_ref(gs, blockIdx.x);
  const int W = t.W, tx0 = t.tx0, ty0 = t.ty0;
  const long long off = t.off;
  const int tw = min(TW, W - tx0), th = min(TH, t.H - ty0);
  // top row (tw pixels), left column (th - 1 pixels), right column (th - 1)
  const int nb = tw + 2 * (th - 1);
  for (int j = threadIdx.x; j < nb; j += kThreads) {
    int r, c;
    if (j < tw) { r = 0; c = j; }
    else if (j < tw + th - 1) { r = j - tw + 1; c = 0; }
    else { r = j - tw - th + 2; c = tw - 1; }
    const int x = tx0 + c, y = ty0 + r;
    const int g = (int)(off + (long long)y * W + x);
    const int v = __ldg(in + g);
    // backward neighbours that lie in another tile
    if (c == 0 && x > 0 && __ldg(in + g - 1) == v) gunite<MAXC>(P, g, g - 1, status);
    if (y > 0) {
      if (r == 0 && __ldg(in + g - W) == v) gunite<MAXC>(P, g, g - W, status);
      if (CONN == 8) {
        if ((r == 0 || c == 0) && x > 0 && __ldg(in + g - W - 1) == v)
          gunite<MAXC>(P, g, g - W - 1, status);
        if ((r == 0 || c == tw - 1) && x + 1 < W && __ldg(in + g - W + 1) == v)
          gunite<MAXC>(P, g, g - W + 1, status);
      }
    }
  }
}

// Flatten pass, one block per tile (only image pixels are touched, so batch
// arenas may carry padding between images).
__global__ void __launch_bounds__(kThreads)
flatten_kernel(int* P, Geoms gs, int32_t* __restrict__ sizes, int* status) {
  const unsigned full = 0xffffffffu;
  const TileRef t = tile_ref(gs, blockIdx.x);
  for (int q = threadIdx.x; q < TH * TW; q += kThreads) {
    const int x = t.tx0 + q % TW, y = t.ty0 + q / TW;
    int root = -1;
    if (x < t.W && y < t.H) {
      const long long g = t.off + (long long)y * t.W + x;
      unsigned budget = kUnionCap;
      const int lr = __ldcg(P + g);
      root = gfind(P, lr, budget);
      if (!budget) set_status(status, SPLIT_ERR_NOT_CONVERGED);
      P[g] = root;
      if (lr != root) P[lr] = root;  // later pixels of this local tree: one hop
    }
    if (sizes) {
      const unsigned peers = __match_any_sync(full, root);
      const int leader = __ffs(peers) - 1;
      if (root >= 0 && (threadIdx.x & 31) == leader) atomicAdd(sizes + root, __popc(peers));
    }
  }
}

struct Layout {
  WsHeader* hdr;
  size_t bytes;
};

static Layout carve(void* ws) {
  Carver c(ws);
  Layout l;
  l.hdr = c.take<WsHeader>(1);
  l.bytes = c.size();
  return l;
}

template <bool MAXC, int CONN>
static int run(const int32_t* in, const Geoms& gs, int32_t* out, int32_t* sizes, WsHeader* hdr,
               cudaStream_t st) {
  tile_kernel<MAXC, CONN><<<gs.total_tiles, kThreads, 0, st>>>(in, gs, out, sizes, &hdr->status);
  SG_TRY(launch_status());
  border_kernel<MAXC, CONN><<<gs.total_tiles, kThreads, 0, st>>>(in, gs, out, &hdr->status);
  SG_TRY(launch_status());
  flatten_kernel<<<gs.total_tiles, kThreads, 0, st>>>(out, gs, sizes, &hdr->status);
  return launch_status();
}

}  // namespace ccl

// Labelling over a geometry table (one image or a batch arena).  Labels are
// arena-global linear indices.
int ccl_geoms(const int32_t* in, const Geoms& gs, int connectivity, int convention, int32_t* out,
              int32_t* sizes, WsHeader* hdr, cudaStream_t st) {
  const bool mx = convention == SPLIT_LABEL_MAX_INDEX;
  if (connectivity == 4)
    return mx ? ccl::run<true, 4>(in, gs, out, sizes, hdr, st)
              : ccl::run<false, 4>(in, gs, out, sizes, hdr, st);
  return mx ? ccl::run<true, 8>(in, gs, out, sizes, hdr, st)
            : ccl::run<false, 8>(in, gs, out, sizes, hdr, st);
}

// ---- label compression ----------------------------------------------------
namespace cmp {

constexpr int kThreads = 256;
constexpr int kTile = 4096;  // elements per scan tile

struct Layout {
  WsHeader* hdr;
  int32_t* flags;       // [n + 1] -> ranks after the scan
  int32_t* tile_sums;   // [ntiles]
  size_t bytes;
};

static Layout carve(void* ws, int64_t n) {
  Carver c(ws);
  Layout l;
  l.hdr = c.take<WsHeader>(1);
  l.flags = c.take<int32_t>((size_t)n + 1);
  const int64_t tiles = (n + 1 + kTile - 1) / kTile;
  l.tile_sums = c.take<int32_t>((size_t)tiles + 1);
  l.bytes = c.size();
  return l;
}

__global__ void mark_kernel(const int32_t* __restrict__ labels, int64_t n,
                            int32_t* __restrict__ flags, int* status) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int v = labels[i];
    if (v < -1 || v >= n) {
      set_status(status, SPLIT_ERR_INVALID);
      continue;
    }
    flags[v + 1] = 1;
  }
}

__device__ __forceinline__ int block_exclusive_scan(int v, int* warp_tot, int& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int t = lane < (kThreads / 32) ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < kThreads / 32) warp_tot[lane] = t;
  }
  __syncthreads();
  total = warp_tot[kThreads / 32 - 1];
  const int before = warp ? warp_tot[warp - 1] : 0;
  __syncthreads();
  return before + x - v;
}

// per-tile totals of the flags
__global__ void tile_sum_kernel(const int32_t* __restrict__ flags, int64_t m,
                                int32_t* __restrict__ sums) {
  __shared__ int red[kThreads / 32];
  const int64_t t0 = (int64_t)blockIdx.x * kTile;
  int s = 0;
  for (int i = threadIdx.x; i < kTile; i += kThreads) {
    const int64_t j = t0 + i;
    if (j < m) s += flags[j];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < kThreads / 32; ++w) t += red[w];
    sums[blockIdx.x] = t;
  }
}

// exclusive scan of the tile totals (one block, sequential chunks)
__global__ void scan_sums_kernel(int32_t* sums, int64_t ntiles, int32_t* d_count) {
  __shared__ int warp_tot[kThreads / 32];
  int carry = 0;
  for (int64_t base = 0; base < ntiles; base += kThreads) {
    const int64_t i = base + threadIdx.x;
    const int v = i < ntiles ? sums[i] : 0;
    int total;
    const int ex = block_exclusive_scan(v, warp_tot, total);
    if (i < ntiles) sums[i] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) {
    sums[ntiles] = carry;
    if (d_count) *d_count = carry;
  }
}

// flags -> exclusive ranks, tile by tile
__global__ void tile_scan_kernel(int32_t* flags, int64_t m, const int32_t* __restrict__ sums) {
  __shared__ int warp_tot[kThreads / 32];
  const int64_t t0 = (int64_t)blockIdx.x * kTile;
  int carry = sums[blockIdx.x];
  for (int base = 0; base < kTile; base += kThreads) {
    const int64_t j = t0 + base + threadIdx.x;
    const int v = j < m ? flags[j] : 0;
    int total;
    const int ex = block_exclusive_scan(v, warp_tot, total);
    if (j < m) flags[j] = carry + ex;
    carry += total;
  }
}

__global__ void gather_kernel(int32_t* labels, int64_t n, const int32_t* __restrict__ ranks) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int v = labels[i];
    if (v >= -1 && v < n) labels[i] = __ldg(ranks + v + 1);
  }
}

}  // namespace cmp
}  // namespace sg

using namespace sg;

extern "C" size_t split_ccl_workspace_size(int width, int height) {
  (void)width;
  (void)height;
  return ccl::carve(nullptr).bytes;
}

extern "C" int split_ccl(const int32_t* labels_in, int width, int height, int connectivity,
                         int convention, int32_t* labels_out, int32_t* d_sizes, void* workspace,
                         size_t workspace_bytes, void* stream) {
  if (!labels_in || !labels_out || width < 1 || height < 1) return SPLIT_ERR_INVALID;
  if ((int64_t)width * height > 0x7fffffffLL) return SPLIT_ERR_INVALID;
  if (connectivity != 4 && connectivity != 8) return SPLIT_ERR_INVALID;
  if (convention != SPLIT_LABEL_MIN_INDEX && convention != SPLIT_LABEL_MAX_INDEX)
    return SPLIT_ERR_INVALID;
  if (labels_in == labels_out) return SPLIT_ERR_INVALID;
  ccl::Layout l = ccl::carve(nullptr);
  if (!workspace || workspace_bytes < l.bytes || (reinterpret_cast<uintptr_t>(workspace) & 255))
    return SPLIT_ERR_WORKSPACE;
  l = ccl::carve(workspace);
  return ccl_geoms(labels_in, single_geom(width, height), connectivity, convention, labels_out,
                   d_sizes, l.hdr, as_stream(stream));
}

extern "C" size_t split_compress_labels_workspace_size(int64_t n) {
  if (n <= 0) return 0;
  return cmp::carve(nullptr, n).bytes;
}

extern "C" int split_compress_labels(int32_t* labels, int64_t n, int32_t* d_count,
                                     void* workspace, size_t workspace_bytes, void* stream) {
  if (!labels || n <= 0 || n > 0x7fffffffLL) return SPLIT_ERR_INVALID;
  cmp::Layout l = cmp::carve(nullptr, n);
  if (!workspace || workspace_bytes < l.bytes || (reinterpret_cast<uintptr_t>(workspace) & 255))
    return SPLIT_ERR_WORKSPACE;
  l = cmp::carve(workspace, n);
  cudaStream_t st = as_stream(stream);
  DeviceInfo di;
  SG_TRY(device_info(&di));
  const int64_t m = n + 1;
  const int64_t ntiles = (m + cmp::kTile - 1) / cmp::kTile;
  int64_t blocks = (n + 255) / 256;
  if (blocks > (int64_t)di.sm_count * 16) blocks = (int64_t)di.sm_count * 16;
  SG_CUDA_TRY(cudaMemsetAsync(l.flags, 0, sizeof(int32_t) * (size_t)m, st));
  cmp::mark_kernel<<<(int)blocks, 256, 0, st>>>(labels, n, l.flags, &l.hdr->status);
  SG_TRY(launch_status());
  cmp::tile_sum_kernel<<<(int)ntiles, cmp::kThreads, 0, st>>>(l.flags, m, l.tile_sums);
  SG_TRY(launch_status());
  cmp::scan_sums_kernel<<<1, cmp::kThreads, 0, st>>>(l.tile_sums, ntiles, d_count);
  SG_TRY(launch_status());
  cmp::tile_scan_kernel<<<(int)ntiles, cmp::kThreads, 0, st>>>(l.flags, m, l.tile_sums);
  SG_TRY(launch_status());
  cmp::gather_kernel<<<(int)blocks, 256, 0, st>>>(labels, n, l.flags);
  return launch_status();
}
