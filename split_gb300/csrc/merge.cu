// Small-segment merge: a boundary-histogram pass plus a relabel.
//
// Restates split/src/split/device/ccl/merge_small_segments.cu:92-196 with its
// helpers segment_adjacency.cu:112-142 (8-neighbour edge set),
// detail/fix_map_cycles.cuh:14-44 (mutual pairs keep the larger id) and
// detail/map_until_converged.cuh:14-31 (every label follows its map chain to
// the end).  Instead of materialising 16 ints per pixel of edges and radix
// sorting them, pixels of small segments insert their (segment, neighbour
// segment) pairs into a hash table with multiplicities; each pair then bids
// for its segment with one 64-bit atomicMax:
//   MOST_BOUNDARY: (edge count << 32) | ~neighbour      (most edges, lowest id)
//   REF_CHROMA   : ~((bits(d2) << 32) | neighbour)       (least d2, lowest id)
// and the winning pair writes the segment's map entry.
//
// Workspace state (kept clean between calls):
//   table keys / counts / slot list   zero outside a call
//   best[n]                            zero outside a call
// Per-call arrays: size[n] (unless the caller passes component sizes),
// map[n], fin[n] (final target of every small segment), sum[n] (chroma),
// dec[n] (segments decided by the overflow path).
//
// The table holds at most half its capacity (2^ceil(log2 n) slots) of pairs.
// An image cut into very many small segments can have more distinct pairs
// than that (up to about 8 per pixel).  Then the pair pass stops inserting and
// flags the overflow, and the decision kernel takes the overflow path: the
// small segments are split into classes by the top bits of a hash of their
// id, and each class goes through its own round of pair pass, bids and
// decisions in the emptied table; a class whose pairs still do not fit is
// split in two again.  Bids only compare pairs of one segment, so rounds over
// disjoint classes decide exactly what one pass over a large enough table
// would.  The chains then resolve over the decided segments.
#include <algorithm>

#include "geom.cuh"
#include "merge_state.cuh"

namespace sg {
namespace mrg {

constexpr int kThreads = 256;
static_assert(kTileH * kTileW % kThreads == 0, "whole pixels per thread in a tile");
constexpr int kProbeCap = 1 << 16;
constexpr unsigned kChainCap = 1u << 24;
// overflow path: pending classes (level, class) on a stack, and a bound on rounds
constexpr int kStackCap = 64;
constexpr unsigned kRoundCap = 1u << 20;

struct Layout {
  WsHeader* hdr;
  State* state;
  int32_t* size;
  int32_t* map;
  int32_t* fin;
  unsigned long long* best;
  double* sum;
  unsigned long long* keys;
  unsigned* counts;
  int32_t* list;
  int32_t* dec;
  int* stack;   // [1 + 2 * kStackCap]: depth, then (level, class) pairs
  int cap_log2;
  size_t bytes;
};

inline int cap_log2_for(int64_t n) {
  int l = 12;
  while ((1ll << l) < n && l < 31) ++l;
  return l;
}

inline Layout carve(void* ws, int64_t n) {
  Carver c(ws);
  Layout l;
  l.hdr = c.take<WsHeader>(1);
  l.state = c.take<State>(1);
  l.size = c.take<int32_t>((size_t)n);
  l.map = c.take<int32_t>((size_t)n);
  l.fin = c.take<int32_t>((size_t)n);
  l.best = c.take<unsigned long long>((size_t)n);
  l.sum = c.take<double>((size_t)n);
  l.cap_log2 = cap_log2_for(n);
  const size_t cap = (size_t)1 << l.cap_log2;
  l.keys = c.take<unsigned long long>(cap);
  l.counts = c.take<unsigned>(cap);
  l.list = c.take<int32_t>(cap);
  l.dec = c.take<int32_t>((size_t)n);
  l.stack = c.take<int>(1 + 2 * kStackCap);
  l.bytes = c.size();
  return l;
}

__device__ __forceinline__ unsigned long long pair_key(int s, int t) {
  return (((unsigned long long)(unsigned)s << 32) | (unsigned)t) + 1ull;
}
__device__ __forceinline__ int key_s(unsigned long long k) { return (int)((k - 1ull) >> 32); }
__device__ __forceinline__ int key_t(unsigned long long k) { return (int)(unsigned)((k - 1ull) & 0xffffffffull); }

// Inserts (s, t) with multiplicity m.  A new pair that takes the table past
// half its capacity (or a probe sequence that runs out) flags the overflow
// and returns true: the caller then stops inserting (the pass decides class
// by class instead), and so does every tile that starts after the flag is
// set, so the table never grows past half by more than the lanes running at
// once.  Every claimed slot is listed (the list holds as many entries as the
// table), so the table can always be cleared through the list.  The list
// counter is one word that every new pair increments: the lanes of a warp
// that claim slots in the same step take their list places with one atomic,
// and nothing else reads that word during the pass.
__device__ bool insert(const Layout& L, int s, int t, unsigned m) {
  const unsigned long long key = pair_key(s, t);
  const unsigned mask = (1u << L.cap_log2) - 1u;
  unsigned h = (unsigned)((key * 0x9E3779B97F4A7C15ull) >> (64 - L.cap_log2));
  for (int probe = 0; probe < kProbeCap; ++probe, h = (h + 1) & mask) {
    unsigned long long k = *(volatile unsigned long long*)(L.keys + h);
    if (k == 0ull) {
      k = atomicCAS(L.keys + h, 0ull, key);
      if (k == 0ull) {
        atomicAdd(L.counts + h, m);
        const unsigned am = __activemask();
        const int lane = threadIdx.x & 31, leader = __ffs(am) - 1;
        unsigned base = 0;
        if (lane == leader) base = atomicAdd(&L.state->list_count, (unsigned)__popc(am));
        base = __shfl_sync(am, base, leader);
        const unsigned idx = base + __popc(am & ((1u << lane) - 1u));
        L.list[idx] = (int)h;
        if (idx < (mask >> 1)) return false;
        *(volatile int*)&L.state->overflow = 1;
        return true;
      }
    }
    if (k == key) {
      atomicAdd(L.counts + h, m);
      return false;
    }
  }
  *(volatile int*)&L.state->overflow = 1;
  return true;
}

// Class of segment s at split level `lev`: the top lev bits of a hash of s
// (level 0: every segment in class 0).
__device__ __forceinline__ unsigned seg_class(int s, int lev) {
  return lev == 0 ? 0u : ((unsigned)s * 2654435761u) >> (32 - lev);
}

// sizes (generic path) and chroma sums; REF_CHROMA also notes whether the
// labels were already sorted (merge_small_segments.cu:124-126, :192-195)
__global__ void __launch_bounds__(kThreads)
size_kernel(const int32_t* __restrict__ lab, int64_t n, Layout L, bool count_sizes,
            const float* __restrict__ chroma, int* status) {
  pdl_wait();
  const unsigned full = 0xffffffffu;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = base + threadIdx.x;
    int s = -1;
    if (i < n) {
      s = __ldg(lab + i);
      if (s < 0 || s >= n) {
        set_status(status, SPLIT_ERR_INVALID);
        s = -1;
      } else if (chroma && i + 1 < n && __ldg(lab + i + 1) < s) {
        L.state->unsorted = 1;
      }
    }
    const unsigned peers = __match_any_sync(full, s);
    const int leader = __ffs(peers) - 1;
    if (count_sizes && s >= 0 && (threadIdx.x & 31) == leader) atomicAdd(L.size + s, __popc(peers));
    if (chroma && s >= 0) atomicAdd(L.sum + s, (double)__ldg(chroma + i));
  }
}

// boundary histogram of the small segments (of class (lev, cls) when CLASSES)
// in one 32 x 64 tile, by the block
template <bool CLASSES>
__device__ __forceinline__ void pair_tile(const int32_t* __restrict__ lab, const Geoms& gs,
                                          const Layout& L, const int32_t* sizes, int P, int tile,
                                          int lev, unsigned cls, int* status) {
  const long long n = gs.total_px;
  const TileRef tr = tile_ref(gs, tile);
  const int W = tr.W, H = tr.H;
  // an overflow flagged before the tile starts: nothing more to insert
  __shared__ int stopped;
  if (threadIdx.x == 0) stopped = *(volatile int*)&L.state->overflow;
  __syncthreads();
  bool go = stopped == 0;
  // all label loads, then all size gathers, before any pixel is examined:
  // the eight pixels' dependent load pairs overlap instead of serialising
  constexpr int kPer = kTileH * kTileW / kThreads;
  int seg[kPer], sz[kPer];
#pragma unroll
  for (int j = 0; j < kPer; ++j) {
    const int q = threadIdx.x + j * kThreads;
    const int x = tr.tx0 + q % kTileW, y = tr.ty0 + q / kTileW;
    seg[j] = (x < W && y < H) ? __ldg(lab + tr.off + (long long)y * W + x) : -1;
  }
#pragma unroll
  for (int j = 0; j < kPer; ++j) sz[j] = (seg[j] >= 0 && seg[j] < n) ? __ldg(sizes + seg[j]) : P;
  for (int j = 0; j < kPer; ++j) {
    if (sz[j] >= P || (CLASSES && seg_class(seg[j], lev) != cls)) continue;
    const int q = threadIdx.x + j * kThreads;
    const int x = tr.tx0 + q % kTileW, y = tr.ty0 + q / kTileW;
    const int s = seg[j];
    L.fin[s] = s;
    int t[8];
    int nt = 0;
#pragma unroll
    for (int d = 0; d < 8; ++d) {
      const int dx = (d == 0 || d == 3 || d == 5) ? -1 : (d == 2 || d == 4 || d == 7) ? 1 : 0;
      const int dy = d < 3 ? -1 : d > 4 ? 1 : 0;
      const int nx = x + dx, ny = y + dy;
      int v = -1;
      if (nx >= 0 && ny >= 0 && nx < W && ny < H) v = __ldg(lab + tr.off + (long long)ny * W + nx);
      if (v >= n) {
        set_status(status, SPLIT_ERR_INVALID);
        v = -1;
      }
      if (v != s && v >= 0) t[nt++] = v;
    }
    for (int a = 0; a < nt; ++a) {
      bool first = true;
      unsigned m = 1;
      for (int b = 0; b < a; ++b) first &= (t[b] != t[a]);
      if (!first) continue;
      for (int b = a + 1; b < nt; ++b) m += (t[b] == t[a]);
      if (go && insert(L, s, t[a], m)) go = false;
    }
  }
}

// boundary histogram of small segments, one block per 32 x 64 tile
__global__ void __launch_bounds__(kThreads, 4)
pair_kernel(const int32_t* __restrict__ lab, Geoms gs, Layout L, const int32_t* sizes, int P,
            int* status) {
  pdl_wait();
  pair_tile<false>(lab, gs, L, sizes, P, blockIdx.x, 0, 0u, status);
}

__device__ __forceinline__ float seg_mean(const Layout& L, const int32_t* sizes, int s) {
  return (float)L.sum[s] / (float)__ldg(sizes + s);
}

__device__ void bid_phase(const Layout& L, const int32_t* sizes, int policy) {
  const unsigned cnt = *(volatile unsigned*)&L.state->list_count;
  for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < cnt; j += gridDim.x * blockDim.x) {
    const int h = L.list[j];
    const unsigned long long k = L.keys[h];
    const int s = key_s(k), t = key_t(k);
    unsigned long long bid;
    if (policy == SPLIT_MERGE_MOST_BOUNDARY) {
      bid = ((unsigned long long)L.counts[h] << 32) | (unsigned)(0xffffffffu - (unsigned)t);
    } else {
      const float x = seg_mean(L, sizes, s) - seg_mean(L, sizes, t);
      const float d2 = __fadd_rn(__fmul_rn(x, x), __fmul_rn(x, x));
      bid = ~(((unsigned long long)__float_as_uint(d2) << 32) | (unsigned)t);
    }
    atomicMax(L.best + s, bid);
  }
}

__device__ __forceinline__ int bid_target(unsigned long long b, int policy) {
  if (policy == SPLIT_MERGE_MOST_BOUNDARY) return (int)(0xffffffffu - (unsigned)(b & 0xffffffffull));
  return (int)(unsigned)((~b) & 0xffffffffull);
}

__device__ void decide_phase(const Layout& L, int policy) {
  const unsigned cnt = *(volatile unsigned*)&L.state->list_count;
  for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < cnt; j += gridDim.x * blockDim.x) {
    const unsigned long long k = L.keys[L.list[j]];
    const int s = key_s(k), t = key_t(k);
    if (bid_target(L.best[s], policy) == t) L.map[s] = t;
  }
}

// next segment along the map: small segments with a winning neighbour move
__device__ __forceinline__ int next_of(const Layout& L, const int32_t* sizes, int P, int r) {
  if (__ldg(sizes + r) >= P) return r;
  if (*(volatile unsigned long long*)(L.best + r) == 0ull) return r;
  const int nx = *(volatile int*)(L.map + r);
  // map entries come from winning pairs, so they are segment ids; anything
  // else is a corrupted workspace: stop the chain here
  if (nx < 0 || nx >= L.state->n) {
    set_status(&L.hdr->status, SPLIT_ERR_INVALID);
    return r;
  }
  return nx;
}

// mutual pairs: the larger id keeps itself (fix_map_cycles.cuh:28-43)
__device__ void cycle_phase(const Layout& L, const int32_t* sizes, int P, int policy) {
  const unsigned cnt = *(volatile unsigned*)&L.state->list_count;
  for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < cnt; j += gridDim.x * blockDim.x) {
    const unsigned long long k = L.keys[L.list[j]];
    const int s = key_s(k), t = key_t(k);
    if (bid_target(L.best[s], policy) != t) continue;
    if (next_of(L, sizes, P, t) == s && s > t) *(volatile int*)(L.map + s) = s;
  }
}

__device__ void resolve_phase(const Layout& L, const int32_t* sizes, int P, int policy,
                              int* status) {
  const unsigned cnt = *(volatile unsigned*)&L.state->list_count;
  for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < cnt; j += gridDim.x * blockDim.x) {
    const unsigned long long k = L.keys[L.list[j]];
    const int s = key_s(k), t = key_t(k);
    if (bid_target(L.best[s], policy) != t) continue;
    int r = s;
    unsigned steps = 0;
    for (;;) {
      const int nx = next_of(L, sizes, P, r);
      if (nx == r) break;
      r = nx;
      if (++steps > kChainCap) {
        set_status(status, SPLIT_ERR_NOT_CONVERGED);
        break;
      }
    }
    L.fin[s] = r;
  }
}

// return the table and the bids to zero
__device__ void cleanup_phase(const Layout& L) {
  const unsigned cnt = *(volatile unsigned*)&L.state->list_count;
  for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < cnt; j += gridDim.x * blockDim.x) {
    const int h = L.list[j];
    const unsigned long long k = L.keys[h];
    L.best[key_s(k)] = 0ull;
    L.keys[h] = 0ull;
    L.counts[h] = 0u;
  }
}

// ---- overflow path -----------------------------------------------------
// empties the table slots listed in the claimed-slot list
__device__ void clear_table(const Layout& L) {
  const unsigned cnt = *(volatile unsigned*)&L.state->list_count;
  for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < cnt; j += gridDim.x * blockDim.x) {
    const int h = L.list[j];
    L.keys[h] = 0ull;
    L.counts[h] = 0u;
  }
}

// decisions of one round, also listing the decided segments
__device__ void decide_list_phase(const Layout& L, int policy) {
  const unsigned cnt = *(volatile unsigned*)&L.state->list_count;
  for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < cnt; j += gridDim.x * blockDim.x) {
    const unsigned long long k = L.keys[L.list[j]];
    const int s = key_s(k), t = key_t(k);
    if (bid_target(L.best[s], policy) == t) {
      L.map[s] = t;
      L.dec[atomicAdd(&L.state->dec_count, 1u)] = s;
    }
  }
}

__device__ void cycle_dec_phase(const Layout& L, const int32_t* sizes, int P) {
  const unsigned cnt = *(volatile unsigned*)&L.state->dec_count;
  for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < cnt; j += gridDim.x * blockDim.x) {
    const int s = L.dec[j];
    const int t = *(volatile int*)(L.map + s);
    if (next_of(L, sizes, P, t) == s && s > t) *(volatile int*)(L.map + s) = s;
  }
}

__device__ void resolve_dec_phase(const Layout& L, const int32_t* sizes, int P, int* status) {
  const unsigned cnt = *(volatile unsigned*)&L.state->dec_count;
  for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < cnt; j += gridDim.x * blockDim.x) {
    const int s = L.dec[j];
    int r = s;
    unsigned steps = 0;
    for (;;) {
      const int nx = next_of(L, sizes, P, r);
      if (nx == r) break;
      r = nx;
      if (++steps > kChainCap) {
        set_status(status, SPLIT_ERR_NOT_CONVERGED);
        break;
      }
    }
    L.fin[s] = r;
  }
}

// The pair pass overflowed: decide class by class (see the top of the file).
// Runs inside the cooperative decision launch; every phase sits behind a
// bounded grid barrier and the round count is bounded.
__device__ void overflow_path(const Layout& L, const int32_t* lab, const Geoms& gs,
                              const int32_t* sizes, int P, int policy,
                              unsigned long long stamp, unsigned& nbar) {
  WsHeader* h = L.hdr;
  State* st = L.state;
  const bool lead = blockIdx.x == 0 && threadIdx.x == 0;
  clear_table(L);
  if (!grid_barrier_counted(h, ++nbar)) return;
  if (lead) {
    st->list_count = 0;
    st->overflow = 0;
    st->dec_count = 0;
    L.stack[0] = 2;            // the two halves of level 1
    L.stack[1] = 1, L.stack[2] = 1;
    L.stack[3] = 1, L.stack[4] = 0;
  }
  if (!grid_barrier_counted(h, ++nbar)) return;
  __shared__ int lev, cls;
  for (unsigned round = 0;; ++round) {
    if (threadIdx.x == 0) {
      const int depth = *(volatile int*)L.stack;
      lev = depth > 0 && round < kRoundCap ? *(volatile int*)(L.stack + 2 * depth - 1) : -1;
      cls = depth > 0 ? *(volatile int*)(L.stack + 2 * depth) : 0;
    }
    __syncthreads();
    if (lev < 0) break;   // the same decision in every block
    for (int t = blockIdx.x; t < gs.total_tiles; t += gridDim.x)
      pair_tile<true>(lab, gs, L, sizes, P, t, lev, (unsigned)cls, &h->status);
    if (!grid_barrier_counted(h, ++nbar)) return;
    const bool split = *(volatile int*)&st->overflow != 0;
    if (!split) {
      bid_phase(L, sizes, policy);
      if (!grid_barrier_counted(h, ++nbar)) return;
      decide_list_phase(L, policy);
      if (!grid_barrier_counted(h, ++nbar)) return;
    }
    clear_table(L);
    if (!grid_barrier_counted(h, ++nbar)) return;
    if (lead) {
      int depth = L.stack[0] - 1;   // pop (lev, cls)
      if (split) {
        if (lev >= 31 || depth + 2 > kStackCap) {
          set_status(&h->status, SPLIT_ERR_OVERFLOW);
          depth = 0;
        } else {
          L.stack[1 + 2 * depth] = lev + 1, L.stack[2 + 2 * depth] = 2 * cls + 1;
          L.stack[3 + 2 * depth] = lev + 1, L.stack[4 + 2 * depth] = 2 * cls;
          depth += 2;
        }
      }
      L.stack[0] = depth;
      st->list_count = 0;
      st->overflow = 0;
      if (round + 1 >= kRoundCap) set_status(&h->status, SPLIT_ERR_NOT_CONVERGED);
    }
    if (!grid_barrier_counted(h, ++nbar)) return;
  }
  cycle_dec_phase(L, sizes, P);
  if (!grid_barrier_counted(h, ++nbar)) return;
  resolve_dec_phase(L, sizes, P, &h->status);
  if (!grid_barrier_counted(h, ++nbar)) return;
  const unsigned cnt = *(volatile unsigned*)&st->dec_count;
  for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < cnt; j += gridDim.x * blockDim.x)
    L.best[L.dec[j]] = 0ull;
  if (lead) h->stamp = stamp;
}

// The decision over the pair list, one cooperative launch (one block per
// SM): bids, decisions, mutual-pair fix, chains, cleanup, each phase behind a
// bounded grid barrier.  The last step records the layout the guard cleared for.
// When the pair pass overflowed, the overflow path decides instead.
__global__ void __launch_bounds__(kThreads)
list_kernel(Layout L, const int32_t* lab, Geoms gs, const int32_t* sizes, int P, int policy,
            unsigned long long stamp) {
  WsHeader* h = L.hdr;
  // grid barriers passed (the guard zeroed the counter they count on)
  unsigned nbar = 0;
  if (*(volatile int*)&L.state->overflow) {   // set before this launch: the same in every block
    overflow_path(L, lab, gs, sizes, P, policy, stamp, nbar);
    return;
  }
  bid_phase(L, sizes, policy);
  if (!grid_barrier_counted(h, ++nbar)) return;
  decide_phase(L, policy);
  if (!grid_barrier_counted(h, ++nbar)) return;
  cycle_phase(L, sizes, P, policy);
  if (!grid_barrier_counted(h, ++nbar)) return;
  resolve_phase(L, sizes, P, policy, &h->status);
  if (!grid_barrier_counted(h, ++nbar)) return;
  cleanup_phase(L);
  if (blockIdx.x == 0 && threadIdx.x == 0) h->stamp = stamp;
}

__global__ void relabel_kernel(int32_t* lab, int64_t n, const State* stp, const int32_t* fin) {
  pdl_wait();
  const State st = *stp;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    lab[i] = relabel(st, fin, lab[i]);
}

// Sets the run's parameters (block 0) and clears the state that every call
// leaves at zero (hash table, bids) when the workspace was last used with
// another layout (or never): reusing one workspace for images of different
// sizes moves these regions.  list_kernel records the new layout at its end.
__global__ void guard_kernel(WsHeader* h, unsigned long long stamp, Layout L, long long n,
                             const int32_t* sizes, int P, int policy) {
  pdl_wait();
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    State* st = L.state;
    st->n = (int)n;
    st->sizes = sizes;
    st->P = P;
    st->policy = policy;
    st->unsorted = 0;
    st->list_count = 0;
    st->cap_log2 = L.cap_log2;
    st->overflow = 0;
    st->dec_count = 0;
    h->barrier_count = 0;
  }
  if (*(volatile const unsigned long long*)&h->stamp == stamp) return;
  const long long cap = 1ll << L.cap_log2;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cap; i += stride) {
    L.keys[i] = 0ull;
    L.counts[i] = 0u;
  }
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride)
    L.best[i] = 0ull;
}

}  // namespace mrg

int merge_view_n(const void* ws, int64_t n, MergeView* out) {
  if (!ws || n < 1) return SPLIT_ERR_INVALID;
  mrg::Layout l = mrg::carve(const_cast<void*>(ws), n);
  out->state = l.state;
  out->fin = l.fin;
  return SPLIT_OK;
}

int merge_view(const void* ws, int width, int height, MergeView* out) {
  if (!ws || width < 1 || height < 1) return SPLIT_ERR_INVALID;
  mrg::Layout l = mrg::carve(const_cast<void*>(ws), (int64_t)width * height);
  out->state = l.state;
  out->fin = l.fin;
  return SPLIT_OK;
}

}  // namespace sg

using namespace sg;

extern "C" size_t split_merge_small_workspace_size(int width, int height) {
  if (width < 1 || height < 1) return 0;
  return mrg::carve(nullptr, (int64_t)width * height).bytes;
}

// Runs the decision passes over a geometry table (labels are arena-global
// segment ids); the labels are relabelled unless `relabel_labels` is false
// (the fused erosion relabels instead).
static int merge_run(int32_t* labels, const Geoms& gs, int P, int policy, const float* chroma,
                     const int32_t* d_sizes, void* workspace, size_t workspace_bytes,
                     cudaStream_t st, bool relabel_labels) {
  const int64_t n = gs.total_px;
  if (!labels || n < 1 || n > 0x7fffffffLL) return SPLIT_ERR_INVALID;
  if (policy != SPLIT_MERGE_MOST_BOUNDARY && policy != SPLIT_MERGE_REF_CHROMA)
    return SPLIT_ERR_INVALID;
  if (policy == SPLIT_MERGE_REF_CHROMA && !chroma) return SPLIT_ERR_INVALID;
  mrg::Layout l = mrg::carve(nullptr, n);
  if (!workspace || workspace_bytes < l.bytes || (reinterpret_cast<uintptr_t>(workspace) & 255))
    return SPLIT_ERR_WORKSPACE;
  l = mrg::carve(workspace, n);
  DeviceInfo di;
  SG_TRY(device_info(&di));
  int64_t blocks = (n + mrg::kThreads - 1) / mrg::kThreads;
  if (blocks > (int64_t)di.sm_count * 8) blocks = (int64_t)di.sm_count * 8;
  const int grid = (int)blocks;
  const int32_t* sizes = d_sizes ? d_sizes : l.size;
  const bool ref = policy == SPLIT_MERGE_REF_CHROMA;
  const unsigned long long stamp = ((unsigned long long)l.cap_log2 << 40) | (unsigned long long)n;
  // the guard usually finds the stamp unchanged and exits: one block per SM
  // is enough for the rare full clear
  launch_pdl(mrg::guard_kernel, dim3(di.sm_count), dim3(mrg::kThreads), 0, st, l.hdr, stamp, l,
             (long long)n, sizes, P, policy);
  SG_TRY(launch_status());
  if (!d_sizes) SG_CUDA_TRY(cudaMemsetAsync(l.size, 0, sizeof(int32_t) * (size_t)n, st));
  if (ref) SG_CUDA_TRY(cudaMemsetAsync(l.sum, 0, sizeof(double) * (size_t)n, st));
  if (!d_sizes || ref) {
    launch_pdl(mrg::size_kernel, dim3(grid), dim3(mrg::kThreads), 0, st, labels, n, l, !d_sizes,
               ref ? chroma : nullptr, &l.hdr->status);
    SG_TRY(launch_status());
  }
  launch_pdl(mrg::pair_kernel, dim3(gs.total_tiles), dim3(mrg::kThreads), 0, st, labels, gs, l,
             sizes, P, &l.hdr->status);
  SG_TRY(launch_status());
  {
    // One co-resident block per SM: the lists of most images are short and
    // the decision is bound by its grid barriers, which slow with the block
    // count.  Images and arenas of 2^24 pixels and more can hold lists of
    // millions of pairs, walked with a dependent load or two per entry:
    // there as many blocks as fit, up to 4 per SM.
    int per_sm = 0;
    SG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mrg::list_kernel,
                                                              mrg::kThreads, 0));
    if (per_sm < 1) return SPLIT_ERR_UNSUPPORTED;
    const int list_blocks = di.sm_count * (n >= ((int64_t)1 << 24) ? std::min(per_sm, 4) : 1);
    unsigned long long stamp_arg = stamp;
    int P_arg = P, policy_arg = policy;
    const int32_t* sizes_arg = sizes;
    const int32_t* lab_arg = labels;
    Geoms gs_arg = gs;
    void* args[] = {&l, &lab_arg, &gs_arg, &sizes_arg, &P_arg, &policy_arg, &stamp_arg};
    SG_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)mrg::list_kernel, dim3(list_blocks),
                                            dim3(mrg::kThreads), args, 0, st));
  }
  SG_TRY(launch_status());
  if (relabel_labels) {
    launch_pdl(mrg::relabel_kernel, dim3(grid), dim3(mrg::kThreads), 0, st, labels, n,
               (const mrg::State*)l.state, (const int32_t*)l.fin);
    SG_TRY(launch_status());
  }
  return SPLIT_OK;
}

static int merge_decide(int32_t* labels, int width, int height, int P, int policy,
                        const float* chroma, const int32_t* d_sizes, void* workspace,
                        size_t workspace_bytes, cudaStream_t st, bool relabel_labels) {
  if (!labels || width < 1 || height < 1) return SPLIT_ERR_INVALID;
  if ((int64_t)width * height > 0x7fffffffLL) return SPLIT_ERR_INVALID;
  return merge_run(labels, single_geom(width, height), P, policy, chroma, d_sizes, workspace,
                   workspace_bytes, st, relabel_labels);
}

namespace sg {
int merge_geoms(const int32_t* labels, const Geoms& gs, int P, int policy, const int32_t* d_sizes,
                void* workspace, size_t workspace_bytes, cudaStream_t st) {
  return merge_run(const_cast<int32_t*>(labels), gs, P, policy, nullptr, d_sizes, workspace,
                   workspace_bytes, st, false);
}
size_t merge_workspace_bytes(int64_t n) { return mrg::carve(nullptr, n).bytes; }
}  // namespace sg

extern "C" int split_merge_small(int32_t* labels, int width, int height, int P, int policy,
                                 const float* chroma, const int32_t* d_sizes, void* workspace,
                                 size_t workspace_bytes, void* stream) {
  return merge_decide(labels, width, height, P, policy, chroma, d_sizes, workspace,
                      workspace_bytes, as_stream(stream), true);
}

namespace sg {
int merge_decide_only(const int32_t* labels, int width, int height, int P, int policy,
                      const float* chroma, const int32_t* d_sizes, void* workspace,
                      size_t workspace_bytes, cudaStream_t st) {
  return merge_decide(const_cast<int32_t*>(labels), width, height, P, policy, chroma, d_sizes,
                      workspace, workspace_bytes, st, false);
}
}  // namespace sg
