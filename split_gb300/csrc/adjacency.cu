// Segment adjacency: the edge list of pixels that border another segment
// (8-neighbourhood) and the sorted list of distinct (segment, neighbouring
// segment) pairs.
//
// Restates split/src/split/device/ccl/segment_adjacency.cu:
//   segment_adjacency_edges (:170-254): for every pixel i in index order and
//     every in-image neighbour j in the order NW, N, NE, W, E, SW, S, SE
//     (NeighbourKeys, :112-142) with labels[i] != labels[j] (the remove_if
//     at :239-243 keeps the survivors in order), one edge (i, j); the m
//     sources go to edges[0, m), the targets to edges[m, 2m) (:249-251).
//   segment_adjacency (:256-289): the label pairs (labels[i], labels[j]) of
//     those edges, sorted by key then value (:279-284), without repeats
//     (:286).
//
// No N x 16 edge array and no comparison sort: the edges are written by an
// order-preserving compaction (per-block counts, one scan, a write pass that
// recomputes each item's outputs), and the pairs are sorted as 64-bit keys
// by a stable LSD radix sort (8-bit digits; a digit equal in every key is
// skipped), after which the same compaction keeps the first pair of every
// run of equal pairs.  Counts come back through device words.
#include "common.cuh"

namespace sg {
namespace adj {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kItems = 16;                    // items per thread
constexpr int kTile = kThreads * kItems;      // items per block
constexpr int kScanThreads = 1024;
// 16 n edge words must stay addressable with int32 (as in the reference)
constexpr int64_t kMaxPixels = (1ll << 27) - 1;

enum Mode { kEdges = 0, kPairs = 1, kUnique = 2 };

struct Layout {
  WsHeader* hdr;
  int* block_sum;                   // [blocks + 1]: per-block counts, then their prefix
  int* total;                       // [2]: edges (or pairs), distinct pairs
  unsigned long long* bits;         // [2]: OR and AND of every pair key
  unsigned long long* keys[2];      // [8 n] each: pair keys, sort ping-pong
  unsigned* hist;                   // [256 * sort blocks]: digit counts, then offsets
  size_t bytes;
};

__host__ __device__ inline int blocks_of(int64_t items) {
  return (int)((items + kTile - 1) / kTile);
}

static Layout carve(void* ws, int64_t n, bool pairs) {
  Carver c(ws);
  Layout l{};
  l.hdr = c.take<WsHeader>(1);
  const int64_t items = pairs ? 8 * n : n;
  l.block_sum = c.take<int>((size_t)blocks_of(items) + 1);
  l.total = c.take<int>(2);
  l.bits = c.take<unsigned long long>(2);
  if (pairs) {
    l.keys[0] = c.take<unsigned long long>((size_t)(8 * n));
    l.keys[1] = c.take<unsigned long long>((size_t)(8 * n));
    l.hist = c.take<unsigned>((size_t)256 * blocks_of(8 * n));
  }
  l.bytes = c.size();
  return l;
}

// neighbour d of pixel (x, y) in the reference's order, or -1 outside
__device__ __forceinline__ int neighbour(int x, int y, int w, int h, int d) {
  const int dx = (d == 0 || d == 3 || d == 5) ? -1 : (d == 2 || d == 4 || d == 7) ? 1 : 0;
  const int dy = d < 3 ? -1 : d > 4 ? 1 : 0;
  const int nx = x + dx, ny = y + dy;
  return (nx >= 0 && nx < w && ny >= 0 && ny < h) ? ny * w + nx : -1;
}

// A pair key whose unsigned order is the (key, value) order of signed ints.
__device__ __forceinline__ unsigned long long pair_key(int a, int b) {
  return ((unsigned long long)((unsigned)a ^ 0x80000000u) << 32) |
         (unsigned long long)((unsigned)b ^ 0x80000000u);
}

// ---- stable LSD radix sort bookkeeping ---------------------------------------
// Pass p sorts on bits [8 p, 8 p + 8).  A pass whose digit is equal in every
// key is skipped; the buffer a pass reads is keys[q & 1], q the number of
// passes before it that were not skipped.
__device__ __forceinline__ bool pass_runs(const unsigned long long* bits, int p) {
  return (((bits[0] ^ bits[1]) >> (8 * p)) & 0xffull) != 0ull;
}
__device__ __forceinline__ int pass_parity(const unsigned long long* bits, int p) {
  int q = 0;
  for (int k = 0; k < p; ++k) q += pass_runs(bits, k);
  return q & 1;
}

struct Items {
  const int32_t* labels;   // kEdges / kPairs
  int w, h;
  // kUnique: the sort buffers and the key bits that name the sorted one
  const unsigned long long* keys0;
  const unsigned long long* keys1;
  const unsigned long long* bits;
  __device__ __forceinline__ const unsigned long long* sorted() const {
    return pass_parity(bits, 8) ? keys1 : keys0;
  }
};

// Outputs of item i: the bitmask of neighbours that border another segment
// (kEdges / kPairs), or whether a sorted pair starts a run (kUnique).
template <int MODE>
__device__ __forceinline__ unsigned item_mask(const Items& it, int i) {
  if (MODE == kUnique) {
    const unsigned long long* s = it.sorted();
    return (i == 0 || s[i] != s[i - 1]) ? 1u : 0u;
  }
  const int x = i % it.w, y = i / it.w, v = __ldg(it.labels + i);
  unsigned m = 0;
#pragma unroll
  for (int d = 0; d < 8; ++d) {
    const int j = neighbour(x, y, it.w, it.h, d);
    if (j >= 0 && __ldg(it.labels + j) != v) m |= 1u << d;
  }
  return m;
}

__device__ __forceinline__ int n_items(const int* d_n, int n) { return d_n ? *d_n : n; }

// Block totals of the items' outputs (contiguous kItems per thread).
template <int MODE>
__global__ void __launch_bounds__(kThreads) count_kernel(Items it, int n, const int* d_n,
                                                          int* block_sum) {
  pdl_wait();
  const int nn = n_items(d_n, n);
  const int base = blockIdx.x * kTile;
  if (base >= nn) return;
  int c = 0;
  for (int k = 0; k < kItems; ++k) {
    const int i = base + threadIdx.x * kItems + k;
    if (i < nn) c += __popc(item_mask<MODE>(it, i));
  }
  __shared__ int ws[kWarps];
  c = __reduce_add_sync(0xffffffffu, c);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int w = 0; w < kWarps; ++w) s += ws[w];
    block_sum[blockIdx.x] = s;
  }
}

// Exclusive scan of `count` words in place by one block, in tiles of
// kScanThreads with a carried prefix; the grand total goes to *total (when
// given).
template <typename T>
__device__ void block_scan(T* a, int count, int* total) {
  __shared__ T part[kScanThreads / 32];
  __shared__ T carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int t0 = 0; t0 < count; t0 += kScanThreads) {
    const int i = t0 + threadIdx.x;
    const T v = i < count ? a[i] : 0;
    T s = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const T u = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += u;
    }
    if (lane == 31) part[warp] = s;
    __syncthreads();
    if (warp == 0) {
      T p = lane < kScanThreads / 32 ? part[lane] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const T u = __shfl_up_sync(0xffffffffu, p, o);
        if (lane >= o) p += u;
      }
      if (lane < kScanThreads / 32) part[lane] = p;
    }
    __syncthreads();
    const T before = carry + (warp ? part[warp - 1] : 0) + s - v;
    if (i < count) a[i] = before;
    __syncthreads();
    if (threadIdx.x == kScanThreads - 1) carry = before + v;
    __syncthreads();
  }
  if (threadIdx.x == 0 && total) *total = (int)carry;
}

// Prefix of the block totals (their total to *total); with `bits`, also
// resets the key OR / AND words that the write pass then fills.
__global__ void __launch_bounds__(kScanThreads) scan_blocks_kernel(int n, const int* d_n,
                                                                   int* block_sum, int* total,
                                                                   unsigned long long* bits) {
  pdl_wait();
  const int nb = blocks_of(n_items(d_n, n));
  if (bits && threadIdx.x == 0) {
    bits[0] = 0ull;
    bits[1] = ~0ull;
  }
  block_scan<int>(block_sum, nb, total);
}

// Writes every item's outputs at its place in the order of the items (a
// block-wide exclusive scan of the threads' counts, plus the block prefix).
template <int MODE>
__global__ void __launch_bounds__(kThreads) write_kernel(Items it, int n, const int* d_n,
                                                          const int* block_sum, const int* total,
                                                          int32_t* out0, int32_t* out1,
                                                          unsigned long long* keys,
                                                          unsigned long long* bits) {
  pdl_wait();
  const int nn = n_items(d_n, n);
  const int base = blockIdx.x * kTile;
  if (base >= nn) return;
  const int first = base + threadIdx.x * kItems;
  int c = 0;
  for (int k = 0; k < kItems; ++k)
    if (first + k < nn) c += __popc(item_mask<MODE>(it, first + k));
  // exclusive scan of c over the block
  __shared__ int ws[kWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int s = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, s, o);
    if (lane >= o) s += u;
  }
  if (lane == 31) ws[warp] = s;
  __syncthreads();
  int before = block_sum[blockIdx.x] + s - c;
  for (int w = 0; w < warp; ++w) before += ws[w];
  const int m = *total;
  unsigned long long o_or = 0ull, o_and = ~0ull;
  for (int k = 0; k < kItems; ++k) {
    const int i = first + k;
    if (i >= nn) break;
    unsigned mask = item_mask<MODE>(it, i);
    if (MODE == kUnique) {
      if (mask) {
        const unsigned long long key = it.sorted()[i];
        out0[before] = (int)((unsigned)(key >> 32) ^ 0x80000000u);
        out1[before] = (int)((unsigned)key ^ 0x80000000u);
        ++before;
      }
      continue;
    }
    const int x = i % it.w, y = i / it.w;
    const int v = MODE == kPairs ? __ldg(it.labels + i) : 0;
    while (mask) {
      const int d = __ffs(mask) - 1;
      mask &= mask - 1;
      const int j = neighbour(x, y, it.w, it.h, d);
      if (MODE == kEdges) {
        out0[before] = i;
        out0[m + before] = j;
      } else {
        const unsigned long long key = pair_key(v, __ldg(it.labels + j));
        keys[before] = key;
        o_or |= key;
        o_and &= key;
      }
      ++before;
    }
  }
  if (MODE == kPairs) {
    // digits that differ between keys (a digit equal in all is not sorted on)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      o_or |= __shfl_xor_sync(0xffffffffu, o_or, o);
      o_and &= __shfl_xor_sync(0xffffffffu, o_and, o);
    }
    if (lane == 0) {
      atomicOr(bits, o_or);
      atomicAnd(bits + 1, o_and);
    }
  }
}

// ---- stable LSD radix sort of the pair keys ----------------------------------
// Digit counts per block, digit-major (hist[d * nb + b]).
__global__ void __launch_bounds__(kThreads) hist_kernel(const Layout l, int p) {
  pdl_wait();
  const int n = *l.total;
  const int nb = blocks_of(n), b = blockIdx.x;
  if (b >= nb || !pass_runs(l.bits, p)) return;
  const unsigned long long* in = l.keys[pass_parity(l.bits, p)];
  __shared__ unsigned h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  for (int k = 0; k < kItems; ++k) {
    const int i = b * kTile + k * kThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(in[i] >> (8 * p)) & 0xff], 1u);
  }
  __syncthreads();
  l.hist[threadIdx.x * nb + b] = h[threadIdx.x];
}

__global__ void __launch_bounds__(kScanThreads) hist_scan_kernel(const Layout l, int p) {
  pdl_wait();
  if (!pass_runs(l.bits, p)) return;
  block_scan<unsigned>(l.hist, 256 * blocks_of(*l.total), nullptr);
}

// Stable scatter: a block moves its items in index order, kThreads at a
// time; an item's place is its digit's offset for the block, plus the items
// of that digit in earlier rounds, in earlier warps of this round, and in
// earlier lanes of its warp.
__global__ void __launch_bounds__(kThreads) scatter_kernel(const Layout l, int p) {
  pdl_wait();
  const int n = *l.total;
  const int nb = blocks_of(n), b = blockIdx.x;
  if (b >= nb || !pass_runs(l.bits, p)) return;
  const int q = pass_parity(l.bits, p);
  const unsigned long long* in = l.keys[q];
  unsigned long long* out = l.keys[q ^ 1];
  __shared__ unsigned off[256];
  __shared__ unsigned wc[kWarps][256];
  const int warp = threadIdx.x >> 5;
  off[threadIdx.x] = l.hist[threadIdx.x * nb + b];
  for (int w = 0; w < kWarps; ++w) wc[w][threadIdx.x] = 0;
  __syncthreads();
  unsigned lt;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
  for (int k = 0; k < kItems; ++k) {
    const int i = b * kTile + k * kThreads + threadIdx.x;
    const bool ok = i < n;
    const unsigned long long key = ok ? in[i] : 0ull;
    const int digit = ok ? (int)((key >> (8 * p)) & 0xff) : 256;
    const unsigned peers = __match_any_sync(0xffffffffu, digit);
    const int rank = __popc(peers & lt);
    if (ok && rank == 0) wc[warp][digit] = __popc(peers);
    __syncthreads();
    if (ok) {
      unsigned pos = off[digit] + rank;
      for (int w = 0; w < warp; ++w) pos += wc[w][digit];
      out[pos] = key;
    }
    __syncthreads();
    // the round's counts move into the digit offsets
    unsigned t = 0;
    for (int w = 0; w < kWarps; ++w) {
      t += wc[w][threadIdx.x];
      wc[w][threadIdx.x] = 0;
    }
    off[threadIdx.x] += t;
    __syncthreads();
  }
}

template <int MODE>
static int compaction(const Items& it, int n, const int* d_n, int max_blocks, const Layout& l,
                      int* total, int32_t* out0, int32_t* out1, unsigned long long* keys,
                      unsigned long long* bits, cudaStream_t st) {
  launch_pdl(count_kernel<MODE>, dim3(max_blocks), dim3(kThreads), 0, st, it, n, d_n,
             l.block_sum);
  SG_TRY(launch_status());
  launch_pdl(scan_blocks_kernel, dim3(1), dim3(kScanThreads), 0, st, n, d_n, l.block_sum, total,
             bits);
  SG_TRY(launch_status());
  launch_pdl(write_kernel<MODE>, dim3(max_blocks), dim3(kThreads), 0, st, it, n, d_n,
             (const int*)l.block_sum, (const int*)total, out0, out1, keys, bits);
  return launch_status();
}

}  // namespace adj
}  // namespace sg

using namespace sg;

extern "C" size_t split_segment_adjacency_edges_workspace_size(int width, int height) {
  if (width < 1 || height < 1) return 0;
  return adj::carve(nullptr, (int64_t)width * height, false).bytes;
}

extern "C" int split_segment_adjacency_edges(const int32_t* labels, int width, int height,
                                             int32_t* edges, int32_t* d_count, void* workspace,
                                             size_t workspace_bytes, void* stream) {
  if (!labels || !edges || !d_count || width < 1 || height < 1) return SPLIT_ERR_INVALID;
  const int64_t n = (int64_t)width * height;
  if (n > adj::kMaxPixels) return SPLIT_ERR_INVALID;
  adj::Layout l = adj::carve(nullptr, n, false);
  if (!workspace || workspace_bytes < l.bytes || (reinterpret_cast<uintptr_t>(workspace) & 255))
    return SPLIT_ERR_WORKSPACE;
  l = adj::carve(workspace, n, false);
  cudaStream_t st = as_stream(stream);
  adj::Items it{labels, width, height, nullptr, nullptr, nullptr};
  return adj::compaction<adj::kEdges>(it, (int)n, nullptr, adj::blocks_of(n), l, d_count, edges,
                                      nullptr, nullptr, nullptr, st);
}

extern "C" size_t split_segment_adjacency_workspace_size(int width, int height) {
  if (width < 1 || height < 1) return 0;
  return adj::carve(nullptr, (int64_t)width * height, true).bytes;
}

extern "C" int split_segment_adjacency(const int32_t* labels, int width, int height,
                                       int32_t* keys, int32_t* adjacency, int32_t* d_count,
                                       void* workspace, size_t workspace_bytes, void* stream) {
  if (!labels || !keys || !adjacency || !d_count || width < 1 || height < 1)
    return SPLIT_ERR_INVALID;
  const int64_t n = (int64_t)width * height;
  if (n > adj::kMaxPixels) return SPLIT_ERR_INVALID;
  adj::Layout l = adj::carve(nullptr, n, true);
  if (!workspace || workspace_bytes < l.bytes || (reinterpret_cast<uintptr_t>(workspace) & 255))
    return SPLIT_ERR_WORKSPACE;
  l = adj::carve(workspace, n, true);
  cudaStream_t st = as_stream(stream);
  // 1: the pair key of every edge, in edge order, and the digits that vary
  adj::Items it{labels, width, height, nullptr, nullptr, nullptr};
  SG_TRY(adj::compaction<adj::kPairs>(it, (int)n, nullptr, adj::blocks_of(n), l, l.total, nullptr,
                                      nullptr, l.keys[0], l.bits, st));
  // 2: stable radix passes
  const int sort_blocks = adj::blocks_of(8 * n);
  for (int p = 0; p < 8; ++p) {
    launch_pdl(adj::hist_kernel, dim3(sort_blocks), dim3(adj::kThreads), 0, st, l, p);
    SG_TRY(launch_status());
    launch_pdl(adj::hist_scan_kernel, dim3(1), dim3(adj::kScanThreads), 0, st, l, p);
    SG_TRY(launch_status());
    launch_pdl(adj::scatter_kernel, dim3(sort_blocks), dim3(adj::kThreads), 0, st, l, p);
    SG_TRY(launch_status());
  }
  // 3: the first pair of every run of equal pairs (which buffer holds the
  // sorted keys depends on the passes that ran: named on the device)
  adj::Items u{nullptr, width, height, l.keys[0], l.keys[1], l.bits};
  return adj::compaction<adj::kUnique>(u, 0, l.total, sort_blocks, l, d_count, keys, adjacency,
                                       nullptr, nullptr, st);
}
