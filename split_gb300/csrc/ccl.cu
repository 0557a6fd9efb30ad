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
//            union-find on shared parents.  A local root stores its own
//            global index, every other pixel the bitwise complement of its
//            local root's (a negative entry), and local roots store their
//            tile-local pixel count as their size.  A tile holding one value
//            everywhere is one component: it stores only its root's entry and
//            records the root in a per-tile word of the workspace (the other
//            passes read that word instead of the tile's entries).
//   border : per tile, edges to earlier tiles (W, NW, N, NE across the tile
//            edge) are merged with lock-free atomicMin/atomicMax hooking of
//            local roots (entries read at edge pixels are decoded first).
//   flatten: every pixel follows its local root's chain to the final root
//            and stores it (in place; a concurrent reader sees an ancestor
//            either way); a local root hooked under another adds its count
//            to the final root's size.
//
// compress_labels (compress_labels.cu:10-35) is a flag / scan / gather over
// the label range [-1, n).
#include "geom.cuh"

namespace sg {
namespace ccl {

constexpr int TH = kTileH, TW = kTileW, kThreads = 256;
constexpr int kWarpsPerTile = kThreads / 32;
constexpr int kRowsPerWarp = TH / kWarpsPerTile;   // 4 rows per warp, 2 pixels per lane
// Bounds on union retries and on find chains (a tile forest has fewer than
// TH * TW nodes; global chains are short after halving).  Running out sets
// SPLIT_ERR_NOT_CONVERGED in the workspace status and returns.
constexpr unsigned kUnionCap = 1u << 16;
constexpr unsigned kFindCap = 1u << 20;
constexpr unsigned kFull = 0xffffffffu;
static_assert(TW == 64 && TH % kWarpsPerTile == 0, "a warp covers whole 64-pixel rows");

template <bool MAXC>
__device__ __forceinline__ bool better(int a, int b) {
  return MAXC ? a > b : a < b;
}

__device__ __forceinline__ unsigned lanemask_le() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_le;" : "=r"(m));
  return m;
}
__device__ __forceinline__ unsigned lanemask_ge() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_ge;" : "=r"(m));
  return m;
}

// ---- shared-memory union-find --------------------------------------------
// Find with path halving.  Safe next to concurrent hooking: a halving store
// only ever points a node at one of its ancestors, and a hook that loses such
// a race is retried by sunite with the node's new parent.
__device__ __forceinline__ int sfind(volatile int* par, int x) {
  int p = par[x];
  for (int hop = 0; p != x && hop < TH * TW; ++hop) {
    const int gp = par[p];
    if (gp != p) par[x] = gp;
    x = p;
    p = par[x];
  }
  return x;
}

// Root of x without writes (for phases where nothing hooks any more).
__device__ __forceinline__ int sroot(const int* par, int x) {
  int p = par[x];
  for (int hop = 0; p != x && hop < TH * TW; ++hop) {
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

// ---- global union-find over local roots (parents in labels_out) ----------
// Parents only move towards the better end (atomicMin / atomicMax hooks, and
// halving stores of a grandparent), so every store points a node at one of
// its ancestors and concurrent finds stay correct.
__device__ __forceinline__ int gfind(int* P, int x, unsigned& budget) {
  int p = __ldcg(P + x);
  while (p != x) {
    if (!budget) return x;
    --budget;
    const int gp = __ldcg(P + p);
    if (gp == p) return p;
    __stcg(P + x, gp);   // path halving
    x = gp;
    p = __ldcg(P + x);
  }
  return x;
}

template <bool MAXC>
__device__ void gunite(int* P, int a, int b, int* status) {
  unsigned budget = kFindCap;
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

// Links that must be unioned between a pixel p (label v) and the row above,
// given equality flags with its neighbours.  Skipped links are implied by
// earlier ones (runs in a row are joined; W + NW cover N; W or N cover NW;
// N or E cover NE), which keeps the number of atomics near the number of
// run overlaps.
struct Links {
  bool n, nw, ne;
};
template <int CONN>
__device__ __forceinline__ Links needed(bool N, bool W, bool NW, bool NE, bool E) {
  Links l;
  l.n = N && !(W && NW);
  l.nw = CONN == 8 && NW && !W && !N;
  l.ne = CONN == 8 && NE && !N && !E;
  return l;
}

// Tile pass.  Warp w owns rows [4w, 4w + 4) of a 32 x 64 tile; lane l holds
// columns l and l + 32 of each row.  Row runs come from warp ballots: the
// node of a run is its first pixel (minimum convention) or its last
// (maximum), and every pixel records its node.  Unions run on nodes only, in
// a shared-memory union-find; after one find per node every pixel reads its
// root in one step and stores the global index of that local root.  Local
// roots clear their size counter.
template <bool MAXC, int CONN>
__global__ void __launch_bounds__(kThreads, 5)
tile_kernel(const int32_t* __restrict__ in, Geoms gs, int* __restrict__ P,
            int32_t* __restrict__ sizes, int* __restrict__ tword, int* __restrict__ tval,
            int* status) {
  pdl_wait();
  __shared__ int lab[TH * TW];
  __shared__ int par[TH * TW];
  const TileRef t = tile_ref(gs, blockIdx.x);
  const int W = t.W, tx0 = t.tx0, ty0 = t.ty0;
  const long long off = t.off;
  const int tw = min(TW, W - tx0), th = min(TH, t.H - ty0);
  const int lane = threadIdx.x & 31, r0 = (threadIdx.x >> 5) * kRowsPerWarp;
  const bool ca = lane < tw, cb = lane + 32 < tw;
  int va[kRowsPerWarp], vb[kRowsPerWarp], na[kRowsPerWarp], nb[kRowsPerWarp];
  // the tile's first pixel: a tile holding one value everywhere is one
  // component, written without the run / union machinery below
  const int v0 = __ldg(in + off + (long long)ty0 * W + tx0);
  bool same = true;
#pragma unroll
  for (int k = 0; k < kRowsPerWarp; ++k) {
    const int r = r0 + k;
    const bool rok = r < th;
    const int32_t* row = in + off + (long long)(ty0 + (rok ? r : 0)) * W + tx0;
    va[k] = (rok && ca) ? __ldg(row + lane) : v0;
    vb[k] = (rok && cb) ? __ldg(row + lane + 32) : v0;
    same = same && va[k] == v0 && vb[k] == v0;
  }
  if (__syncthreads_and(same)) {
    // local root: the first pixel (minimum convention) or the last (maximum);
    // only its entry is stored, the tile word names it for the other passes
    if (threadIdx.x == 0) {
      const long long gr = off + (long long)(ty0 + (MAXC ? th - 1 : 0)) * W + tx0 +
                           (MAXC ? tw - 1 : 0);
      __stcg(P + gr, (int)gr);
      tword[blockIdx.x] = (int)gr + 1;
      tval[blockIdx.x] = v0;
      if (sizes) sizes[gr] = tw * th;
    }
    return;
  }
  if (threadIdx.x == 0) tword[blockIdx.x] = 0;
#pragma unroll
  for (int k = 0; k < kRowsPerWarp; ++k) {
    const int r = r0 + k;
    const bool rok = r < th;
    va[k] = (rok && ca) ? va[k] : 0;
    vb[k] = (rok && cb) ? vb[k] : 0;
    lab[r * TW + lane] = va[k];
    lab[r * TW + lane + 32] = vb[k];
    // run nodes of this row
    const bool oa = rok && ca, ob = rok && cb;
    int nda, ndb;
    if (!MAXC) {
      const int la = __shfl_up_sync(kFull, va[k], 1);
      const int a31 = __shfl_sync(kFull, va[k], 31);
      const int lb0 = __shfl_up_sync(kFull, vb[k], 1);
      const int lb = lane == 0 ? a31 : lb0;
      const unsigned ma = __ballot_sync(kFull, oa && (lane == 0 || la != va[k]));
      const unsigned mb = __ballot_sync(kFull, ob && lb != vb[k]);
      const unsigned le = lanemask_le();
      nda = 31 - __clz(ma & le | 1u);
      const unsigned mbl = mb & le;
      ndb = mbl ? 63 - __clz(mbl) : 31 - __clz(ma | 1u);
    } else {
      const int ra0 = __shfl_down_sync(kFull, va[k], 1);
      const int b0 = __shfl_sync(kFull, vb[k], 0);
      const int ra = lane == 31 ? b0 : ra0;
      const int rb = __shfl_down_sync(kFull, vb[k], 1);
      const unsigned ma = __ballot_sync(kFull, oa && (lane + 1 >= tw || ra != va[k]));
      const unsigned mb = __ballot_sync(kFull, ob && (lane + 33 >= tw || rb != vb[k]));
      const unsigned ge = lanemask_ge();
      const unsigned mag = ma & ge, mbg = mb & ge;
      nda = mag ? __ffs(mag) - 1 : 31 + __ffs(mb | 0x80000000u);
      ndb = 31 + __ffs(mbg | 0x80000000u);
    }
    na[k] = oa ? r * TW + nda : r * TW + lane;
    nb[k] = ob ? r * TW + ndb : r * TW + lane + 32;
    par[r * TW + lane] = na[k];
    par[r * TW + lane + 32] = nb[k];
  }
  __syncthreads();
  // links with the row above (rows 1 .. th - 1 of the tile).  All warp
  // shuffles happen first, with every lane converged, and the needed links
  // are kept as bits; the unions (divergent, retried) come afterwards with
  // no warp-synchronous instruction behind them.
  unsigned links = 0;   // bit 6k + 3h + j: row k, half h, link j (N, NW, NE)
  // bit 2k + h: the pixel that counts its row run (the run's last pixel for
  // the minimum convention, whose node is the first; the first for maximum)
  unsigned counts = 0;
#pragma unroll
  for (int k = 0; k < kRowsPerWarp; ++k) {
    const int r = r0 + k;
    const bool rok = r > 0 && r < th;              // warp-uniform
    const int ua = r > 0 ? lab[(r - 1) * TW + lane] : 0;
    const int ub = r > 0 ? lab[(r - 1) * TW + lane + 32] : 0;
    const int a = va[k], b = vb[k];
    // row neighbours of the pixel and of the pixel above
    const int la = __shfl_up_sync(kFull, a, 1), a31 = __shfl_sync(kFull, a, 31);
    const int lb0 = __shfl_up_sync(kFull, b, 1);
    const int ra0 = __shfl_down_sync(kFull, a, 1), b0 = __shfl_sync(kFull, b, 0);
    const int rb = __shfl_down_sync(kFull, b, 1);
    const int ula = __shfl_up_sync(kFull, ua, 1), ua31 = __shfl_sync(kFull, ua, 31);
    const int ulb0 = __shfl_up_sync(kFull, ub, 1);
    const int ura0 = __shfl_down_sync(kFull, ua, 1), ub0 = __shfl_sync(kFull, ub, 0);
    const int urb = __shfl_down_sync(kFull, ub, 1);
    const int lb = lane == 0 ? a31 : lb0, ulb = lane == 0 ? ua31 : ulb0;
    const int ra = lane == 31 ? b0 : ra0, ura = lane == 31 ? ub0 : ura0;
    if (r < th) {
      const bool xa = ca && (MAXC ? (lane == 0 || la != a) : (lane + 1 >= tw || ra != a));
      const bool xb = cb && (MAXC ? lb != b : (lane + 33 >= tw || rb != b));
      counts |= ((unsigned)xa | ((unsigned)xb << 1)) << (2 * k);
    }
    if (rok && ca) {
      const bool hasW = lane > 0, hasE = lane + 1 < tw;
      const Links l = needed<CONN>(ua == a, hasW && la == a, hasW && ula == a,
                                   hasE && ura == a, hasE && ra == a);
      links |= (unsigned)(l.n | (l.nw << 1) | (l.ne << 2)) << (6 * k);
    }
    if (rok && cb) {
      const bool hasE = lane + 33 < tw;
      const Links l = needed<CONN>(ub == b, lb == b, ulb == b, hasE && urb == b,
                                   hasE && rb == b);
      links |= (unsigned)(l.n | (l.nw << 1) | (l.ne << 2)) << (6 * k + 3);
    }
  }
  while (links) {
    const int bit = __ffs(links) - 1;
    links &= links - 1;
    const int k = bit / 6, h = (bit % 6) / 3, j = bit % 3;
    const int up = (r0 + k - 1) * TW + lane + 32 * h + (j == 1 ? -1 : j == 2 ? 1 : 0);
    int nd = na[0];
#pragma unroll
    for (int q = 0; q < kRowsPerWarp; ++q)
      if (q == k) nd = h ? nb[q] : na[q];
    sunite<MAXC>(par, nd, par[up], status);
  }
  __syncwarp();
  __syncthreads();
  // one find per node (read-only, so concurrent finds see a fixed forest),
  // then every node points straight at its root
  int roota[kRowsPerWarp], rootb[kRowsPerWarp];
#pragma unroll
  for (int k = 0; k < kRowsPerWarp; ++k) {
    const int r = r0 + k;
    const int ia = r * TW + lane, ib = ia + 32;
    roota[k] = (r < th && ca && na[k] == ia) ? sroot(par, ia) : -1;
    rootb[k] = (r < th && cb && nb[k] == ib) ? sroot(par, ib) : -1;
    lab[ia] = 0;   // labels are no longer read: lab counts pixels per root
    lab[ib] = 0;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kRowsPerWarp; ++k) {
    const int ia = (r0 + k) * TW + lane;
    if (roota[k] >= 0) par[ia] = roota[k];
    if (rootb[k] >= 0) par[ia + 32] = rootb[k];
  }
  __syncthreads();
  unsigned isroot = 0;   // bit 2k + h
#pragma unroll
  for (int k = 0; k < kRowsPerWarp; ++k) {
    const int r = r0 + k;
    if (r >= th) continue;
    const long long rowg = off + (long long)(ty0 + r) * W + tx0;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (!(h ? cb : ca)) continue;
      const int c = lane + 32 * h, nd = h ? nb[k] : na[k];
      const int root = par[nd];
      const int gr = (int)(off + (long long)(ty0 + root / TW) * W + tx0 + root % TW);
      const bool own = root == r * TW + c;
      __stcg(P + rowg + c, own ? gr : ~gr);
      isroot |= (unsigned)own << (2 * k + h);
      if (sizes && ((counts >> (2 * k + h)) & 1u)) {
        const int ndc = nd - r * TW;
        atomicAdd(&lab[root], MAXC ? ndc - c + 1 : c - ndc + 1);
      }
    }
  }
  if (sizes) {
    __syncthreads();
    while (isroot) {
      const int bit = __ffs(isroot) - 1;
      isroot &= isroot - 1;
      const int r = r0 + (bit >> 1), c = lane + 32 * (bit & 1);
      sizes[off + (long long)(ty0 + r) * W + tx0 + c] = lab[r * TW + c];
    }
  }
}

// Border pass, one warp per tile: the edges to the tile above (N, NW, NE
// links of the top row), to the tile on the left (W, NW links of the left
// column) and, for 8-connectivity, the NE links of the right column into the
// tile on the right.  Unions start at the local roots the tile pass stored
// and skip links implied by others (the same rules as inside a tile, with
// neighbours read across the edge).
//
// An edge between two one-value tiles is decided from their tile words
// alone: their components join if the values are equal, and no other link
// crosses the edge except at the top row's two corners (8-connectivity),
// whose diagonal links are checked pixel by pixel.  The right column of a
// one-value tile needs no NE link (its N neighbour carries the label).
constexpr int kBorderThreads = 128;
constexpr int kBorderTiles = kBorderThreads / 32;

// The local root named by a tile-pass entry (a non-root pixel stores its local
// root's complement; a local root, hooked or not, stores a root index).
__device__ __forceinline__ int local_root(int e) { return e < 0 ? ~e : e; }

// The local root of pixel g of tile t: the tile word of a one-value tile, the
// pixel's entry otherwise.
__device__ __forceinline__ int lroot(const int* P, const int* tword, long long g, int t) {
  const int w = __ldcg(tword + t);
  return w ? w - 1 : local_root(__ldcg(P + g));
}

template <bool MAXC, int CONN>
__global__ void __launch_bounds__(kBorderThreads)
border_kernel(const int32_t* __restrict__ in, Geoms gs, int* P, const int* __restrict__ tword,
              const int* __restrict__ tval, int* status) {
  pdl_wait();
  const int me = blockIdx.x * kBorderTiles + (threadIdx.x >> 5);
  if (me >= gs.total_tiles) return;
  const int lane = threadIdx.x & 31;
  const TileRef t = tile_ref(gs, me);
  const int up = me - t.tiles_x;
  const int W = t.W, tx0 = t.tx0, ty0 = t.ty0;
  const long long off = t.off;
  const int tw = min(TW, W - tx0), th = min(TH, t.H - ty0);
  bool top_px = ty0 > 0, left_px = tx0 > 0;
  bool right_px = CONN == 8 && tx0 + tw < W;
  const int wme = __ldcg(tword + me);
  if (wme) {
    right_px = false;
    int flags = 0;   // bit 0: the top edge, bit 1: the left edge go pixel by pixel
    if (lane == 0) {
      const int root = wme - 1, v = __ldcg(tval + me);
      const long long g = off + (long long)ty0 * W + tx0;   // the top-left pixel
      if (left_px) {
        const int wl = __ldcg(tword + me - 1);
        if (wl) {
          if (__ldcg(tval + me - 1) == v) gunite<MAXC>(P, root, wl - 1, status);
        } else {
          flags |= 2;
        }
      }
      if (top_px) {
        const int wu = __ldcg(tword + up);
        if (wu) {
          const bool N = __ldcg(tval + up) == v;
          if (N) gunite<MAXC>(P, root, wu - 1, status);
          if (CONN == 8 && !N) {
            // the corners: NW of the first column, NE of the last
            if (tx0 > 0 && __ldg(in + g - 1) != v && __ldg(in + g - W - 1) == v)
              gunite<MAXC>(P, root, lroot(P, tword, g - W - 1, up - 1), status);
            const long long gr = g + tw - 1;
            if (tx0 + tw < W && __ldg(in + gr + 1) != v && __ldg(in + gr - W + 1) == v)
              gunite<MAXC>(P, root, lroot(P, tword, gr - W + 1, up + 1), status);
          }
        } else {
          flags |= 1;
        }
      }
    }
    flags = __shfl_sync(0xffffffffu, flags, 0);
    top_px = flags & 1;
    left_px = flags & 2;
  }
  if (top_px) {
    // the top row with the row above, columns lane and lane + 32
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int c = h * 32 + lane;
      if (c >= tw) break;
      const int x = tx0 + c;
      const long long g = off + (long long)ty0 * W + x;
      const int v = __ldg(in + g);
      const bool hasW = x > 0, hasE = x + 1 < W;
      const bool N = __ldg(in + g - W) == v;
      const bool Wq = hasW && __ldg(in + g - 1) == v;
      const bool NW = hasW && __ldg(in + g - W - 1) == v;
      const bool NE = hasE && __ldg(in + g - W + 1) == v;
      const bool E = hasE && __ldg(in + g + 1) == v;
      // at the tile's first column the W link crosses into the left tile and
      // is made by that edge's lanes; the rule still holds across tiles
      const Links l = needed<CONN>(N, Wq, NW, NE, E);
      if (l.n || l.nw || l.ne) {
        const int a = lroot(P, tword, g, me);
        if (l.n) gunite<MAXC>(P, a, lroot(P, tword, g - W, up), status);
        if (l.nw) gunite<MAXC>(P, a, lroot(P, tword, g - W - 1, c == 0 ? up - 1 : up), status);
        if (l.ne) gunite<MAXC>(P, a, lroot(P, tword, g - W + 1, c == tw - 1 ? up + 1 : up), status);
      }
    }
  }
  if (left_px && lane < th) {
    const int y = ty0 + lane;
    const long long g = off + (long long)y * W + tx0;
    const int v = __ldg(in + g);
    const bool Wq = __ldg(in + g - 1) == v;
    if (lane == 0) {
      // the corner pixel: its N / NW links belong to the top edge
      if (Wq) gunite<MAXC>(P, lroot(P, tword, g, me), lroot(P, tword, g - 1, me - 1), status);
    } else {
      const bool N = __ldg(in + g - W) == v;
      const bool NW = __ldg(in + g - W - 1) == v;
      // W is implied when N and NW carry the label (both columns are joined
      // one row up, and N joins inside this tile)
      const bool lw = Wq && !(N && NW);
      const bool lnw = CONN == 8 && NW && !Wq && !N;
      if (lw || lnw) {
        const int a = lroot(P, tword, g, me);
        if (lw) gunite<MAXC>(P, a, lroot(P, tword, g - 1, me - 1), status);
        if (lnw) gunite<MAXC>(P, a, lroot(P, tword, g - W - 1, me - 1), status);
      }
    }
  }
  if (right_px && lane > 0 && lane < th) {
    // right column, rows 1 .. th - 1: the NE link into the tile to the right
    const int x = tx0 + tw - 1;
    const long long g = off + (long long)(ty0 + lane) * W + x;
    const int v = __ldg(in + g);
    const bool NE = __ldg(in + g - W + 1) == v;
    if (NE && __ldg(in + g - W) != v && __ldg(in + g + 1) != v)
      gunite<MAXC>(P, lroot(P, tword, g, me), lroot(P, tword, g - W + 1, me + 1), status);
  }
}

// Flatten pass, one block per tile, same pixel mapping as the tile pass.
// Every pixel starts from its local root (its complemented entry, or itself
// when the entry is a root index) and follows root entries to the final
// root: one hop for components that stay within the tile or whose local
// root is the final root.  Pixels of one local component chase the same
// chain, so the loads go through L1; entries are only ever replaced by
// ancestors, so a stale line still leads to the final root.  Non-root entries
// are never on a chain, so storing their final roots in place is safe.  A
// local root hooked under another adds its tile-local count to the final
// root's size (nobody adds to a hooked root, so its count is final).
__global__ void __launch_bounds__(kThreads)
flatten_kernel(int* P, Geoms gs, int32_t* __restrict__ sizes, const int* __restrict__ tword,
               int* status) {
  pdl_wait();
  const TileRef t = tile_ref(gs, blockIdx.x);
  const int W = t.W, tx0 = t.tx0, ty0 = t.ty0;
  const int tw = min(TW, W - tx0), th = min(TH, t.H - ty0);
  const int lane = threadIdx.x & 31, r0 = (threadIdx.x >> 5) * kRowsPerWarp;
  const int base = (int)(t.off + (long long)ty0 * W + tx0);
  // a one-value tile: its root's chain is resolved once and every pixel
  // stored without reading the (unwritten) entries
  const int word = __ldcg(tword + blockIdx.x);
  if (word) {
    __shared__ int final_root;
    if (threadIdx.x == 0) {
      const int root = word - 1;
      int f = root, q = P[f];
      unsigned budget = kFindCap;
      while (q != f && budget) {
        --budget;
        f = q;
        q = P[f];
      }
      if (!budget) set_status(status, SPLIT_ERR_NOT_CONVERGED);
      // a root hooked under another adds its count to the final root
      if (sizes && f != root) atomicAdd(sizes + f, __ldcg(sizes + root));
      final_root = f;
    }
    __syncthreads();
    const int f = final_root;
#pragma unroll
    for (int k = 0; k < kRowsPerWarp; ++k) {
      const int r = r0 + k;
      if (r >= th) break;
      if (lane < tw) P[base + r * W + lane] = f;
      if (lane + 32 < tw) P[base + r * W + lane + 32] = f;
    }
    return;
  }
  if (r0 >= th) return;   // the warp's rows lie below the image
  int g[2 * kRowsPerWarp], e[2 * kRowsPerWarp], x[2 * kRowsPerWarp], p[2 * kRowsPerWarp];
#pragma unroll
  for (int k = 0; k < 2 * kRowsPerWarp; ++k) {
    const int r = r0 + (k >> 1), c = lane + 32 * (k & 1);
    g[k] = (r < th && c < tw) ? base + r * W + c : -1;
    e[k] = g[k] >= 0 ? __ldcg(P + g[k]) : 0;
    x[k] = local_root(e[k]);
  }
  unsigned budget = kFindCap;
  // A warp whose pixels all name one local root (a uniform stretch of the
  // image) resolves that root's chain once, in lane 0, and broadcasts it.
  // Lane 0's first pixel is inside the image whenever the warp's rows are.
  const int xr = __shfl_sync(0xffffffffu, x[0], 0);
  bool same = true;
#pragma unroll
  for (int k = 0; k < 2 * kRowsPerWarp; ++k) same = same && (g[k] < 0 || x[k] == xr);
  if (__all_sync(0xffffffffu, same)) {
    int f = xr;
    if (lane == 0) {
      int q = P[f];
      while (q != f && budget) {
        --budget;
        f = q;
        q = P[f];
      }
    }
    f = __shfl_sync(0xffffffffu, f, 0);
#pragma unroll
    for (int k = 0; k < 2 * kRowsPerWarp; ++k) {
      if (g[k] < 0 || e[k] == g[k]) continue;   // outside, or a final root
      P[g[k]] = f;
      if (sizes && e[k] >= 0) atomicAdd(sizes + f, __ldcg(sizes + g[k]));
    }
    if (!budget) set_status(status, SPLIT_ERR_NOT_CONVERGED);
    return;
  }
#pragma unroll
  for (int k = 0; k < 2 * kRowsPerWarp; ++k)
    p[k] = g[k] >= 0 && x[k] != g[k] ? P[x[k]] : x[k];
#pragma unroll
  for (int k = 0; k < 2 * kRowsPerWarp; ++k) {
    if (g[k] < 0 || e[k] == g[k]) continue;   // outside, or a final root
    while (p[k] != x[k] && budget) {
      --budget;
      x[k] = p[k];
      p[k] = P[x[k]];
    }
    P[g[k]] = x[k];
    if (sizes && e[k] >= 0) atomicAdd(sizes + x[k], __ldcg(sizes + g[k]));
  }
  if (!budget) set_status(status, SPLIT_ERR_NOT_CONVERGED);
}

struct Layout {
  WsHeader* hdr;
  int* tword;   // [tiles]: root + 1 of a one-value tile, else 0 (written every run)
  int* tval;    // [tiles]: the value of a one-value tile (written with its word)
  size_t bytes;
};

static Layout carve(void* ws, int tiles) {
  Carver c(ws);
  Layout l;
  l.hdr = c.take<WsHeader>(1);
  l.tword = c.take<int>((size_t)tiles);
  l.tval = c.take<int>((size_t)tiles);
  l.bytes = c.size();
  return l;
}

template <bool MAXC, int CONN>
static int run(const int32_t* in, const Geoms& gs, int32_t* out, int32_t* sizes, WsHeader* hdr,
               cudaStream_t st) {
  const Layout l = carve(hdr, gs.total_tiles);
  int* tword = l.tword;
  launch_pdl(tile_kernel<MAXC, CONN>, dim3(gs.total_tiles), dim3(kThreads), 0, st, in, gs, out,
             sizes, tword, l.tval, &hdr->status);
  SG_TRY(launch_status());
  launch_pdl(border_kernel<MAXC, CONN>, dim3((gs.total_tiles + kBorderTiles - 1) / kBorderTiles),
             dim3(kBorderThreads), 0, st, in, gs, out, (const int*)tword, (const int*)l.tval,
             &hdr->status);
  SG_TRY(launch_status());
  launch_pdl(flatten_kernel, dim3(gs.total_tiles), dim3(kThreads), 0, st, out, gs, sizes,
             (const int*)tword, &hdr->status);
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

// Ranks from a bitmask over the value range [-1, n): bit v + 1 is set when
// some label equals v; the rank of v is the number of set bits below v + 1,
// a per-word exclusive prefix of popcounts plus a popcount within the word.
// The mask and the prefix are 1/32 of the label array each, so the scan is
// short and the gather's lookups stay in L2.
constexpr int kThreads = 256;
constexpr int kTile = 4096;  // words per scan tile

struct Layout {
  WsHeader* hdr;
  uint32_t* bits;       // [nwords]
  int32_t* prefix;      // [nwords]: set bits in the words before
  int32_t* tile_sums;   // [ntiles + 1]
  size_t bytes;
};

inline int64_t words_of(int64_t n) { return (n + 1 + 31) / 32; }

static Layout carve(void* ws, int64_t n) {
  Carver c(ws);
  Layout l;
  const int64_t nw = words_of(n);
  l.hdr = c.take<WsHeader>(1);
  l.bits = c.take<uint32_t>((size_t)nw);
  l.prefix = c.take<int32_t>((size_t)nw);
  const int64_t tiles = (nw + kTile - 1) / kTile;
  l.tile_sums = c.take<int32_t>((size_t)tiles + 1);
  l.bytes = c.size();
  return l;
}

// Sets the bit of every label value.  Only the first lane of a run of equal
// values in the warp touches the mask, and only when it reads the bit clear
// (a stale read just costs a redundant atomicOr).
__global__ void mark_kernel(const int32_t* __restrict__ labels, int64_t n,
                            uint32_t* bits, int* status) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
    const int64_t i = base + threadIdx.x;
    int v = i < n ? labels[i] : -2;
    if (i < n && (v < -1 || v >= n)) {
      set_status(status, SPLIT_ERR_INVALID);
      v = -2;
    }
    const int prev = __shfl_up_sync(0xffffffffu, v, 1);
    if (v >= -1 && ((threadIdx.x & 31) == 0 || prev != v)) {
      const int p = v + 1;
      const uint32_t bit = 1u << (p & 31);
      if (!(bits[p >> 5] & bit)) atomicOr(bits + (p >> 5), bit);
    }
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

// per-tile totals of the set bits
__global__ void tile_sum_kernel(const uint32_t* __restrict__ bits, int64_t nw,
                                int32_t* __restrict__ sums) {
  __shared__ int red[kThreads / 32];
  const int64_t t0 = (int64_t)blockIdx.x * kTile;
  int s = 0;
  for (int i = threadIdx.x; i < kTile; i += kThreads) {
    const int64_t j = t0 + i;
    if (j < nw) s += __popc(bits[j]);
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

// per-word exclusive prefix of the popcounts, tile by tile
__global__ void tile_scan_kernel(const uint32_t* __restrict__ bits, int64_t nw,
                                 const int32_t* __restrict__ sums, int32_t* __restrict__ prefix) {
  __shared__ int warp_tot[kThreads / 32];
  const int64_t t0 = (int64_t)blockIdx.x * kTile;
  int carry = sums[blockIdx.x];
  for (int base = 0; base < kTile; base += kThreads) {
    const int64_t j = t0 + base + threadIdx.x;
    const int v = j < nw ? __popc(bits[j]) : 0;
    int total;
    const int ex = block_exclusive_scan(v, warp_tot, total);
    if (j < nw) prefix[j] = carry + ex;
    carry += total;
  }
}

__global__ void gather_kernel(int32_t* labels, int64_t n, const uint32_t* __restrict__ bits,
                              const int32_t* __restrict__ prefix) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int v = labels[i];
    if (v >= -1 && v < n) {
      const int p = v + 1;
      labels[i] = __ldg(prefix + (p >> 5)) + __popc(__ldg(bits + (p >> 5)) & ((1u << (p & 31)) - 1u));
    }
  }
}

}  // namespace cmp
}  // namespace sg

using namespace sg;

extern "C" size_t split_ccl_workspace_size(int width, int height) {
  if (width < 1 || height < 1) return 0;
  return ccl::carve(nullptr, tiles_of(width, height)).bytes;
}

namespace sg {
// the labelling workspace of a geometry table with `tiles` tiles (batches)
size_t ccl_workspace_bytes(int tiles) { return ccl::carve(nullptr, tiles).bytes; }
}  // namespace sg

extern "C" int split_ccl(const int32_t* labels_in, int width, int height, int connectivity,
                         int convention, int32_t* labels_out, int32_t* d_sizes, void* workspace,
                         size_t workspace_bytes, void* stream) {
  if (!labels_in || !labels_out || width < 1 || height < 1) return SPLIT_ERR_INVALID;
  if ((int64_t)width * height > 0x7fffffffLL) return SPLIT_ERR_INVALID;
  if (connectivity != 4 && connectivity != 8) return SPLIT_ERR_INVALID;
  if (convention != SPLIT_LABEL_MIN_INDEX && convention != SPLIT_LABEL_MAX_INDEX)
    return SPLIT_ERR_INVALID;
  if (labels_in == labels_out) return SPLIT_ERR_INVALID;
  const int tiles = tiles_of(width, height);
  ccl::Layout l = ccl::carve(nullptr, tiles);
  if (!workspace || workspace_bytes < l.bytes || (reinterpret_cast<uintptr_t>(workspace) & 255))
    return SPLIT_ERR_WORKSPACE;
  l = ccl::carve(workspace, tiles);
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
  const int64_t nw = cmp::words_of(n);
  const int64_t ntiles = (nw + cmp::kTile - 1) / cmp::kTile;
  int64_t blocks = (n + 255) / 256;
  if (blocks > (int64_t)di.sm_count * 16) blocks = (int64_t)di.sm_count * 16;
  SG_CUDA_TRY(cudaMemsetAsync(l.bits, 0, sizeof(uint32_t) * (size_t)nw, st));
  cmp::mark_kernel<<<(int)blocks, 256, 0, st>>>(labels, n, l.bits, &l.hdr->status);
  SG_TRY(launch_status());
  cmp::tile_sum_kernel<<<(int)ntiles, cmp::kThreads, 0, st>>>(l.bits, nw, l.tile_sums);
  SG_TRY(launch_status());
  cmp::scan_sums_kernel<<<1, cmp::kThreads, 0, st>>>(l.tile_sums, ntiles, d_count);
  SG_TRY(launch_status());
  cmp::tile_scan_kernel<<<(int)ntiles, cmp::kThreads, 0, st>>>(l.bits, nw, l.tile_sums,
                                                              l.prefix);
  SG_TRY(launch_status());
  cmp::gather_kernel<<<(int)blocks, 256, 0, st>>>(labels, n, l.bits, l.prefix);
  return launch_status();
}
