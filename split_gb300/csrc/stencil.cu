// 2-D stencils of the segmentation path, staged through shared memory by the
// tensor memory accelerator (one cp.async.bulk.tensor tile + halo per block,
// completion on an mbarrier), with a plain-load variant for buffers TMA cannot
// address (row pitch not a multiple of 16 bytes, unaligned base):
//   - square (2r+1)^2 label erosion, optionally fused with the merge relabel;
//   - Sobel normals from a height map or straight from RGB8 (luminance L*/100
//     computed in shared memory, never written);
//   - RGB8 feature packing (float4 features, luminance).
#include <math.h>

#include "geom.cuh"
#include "merge_state.cuh"
#include "tma.cuh"

namespace sg {

static PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

int make_tmap_2d(CUtensorMap* map, CUtensorMapDataType dtype, int elem_bytes, const void* base,
                 uint64_t width, uint64_t height, uint64_t row_bytes, uint32_t box_w,
                 uint32_t box_h) {
  if ((reinterpret_cast<uintptr_t>(base) & 15) || (row_bytes & 15)) return SPLIT_ERR_INVALID;
  if (box_w > 256 || box_h > 256 || (box_w * elem_bytes) % 16) return SPLIT_ERR_INVALID;
  auto enc = tmap_encoder();
  if (!enc) return SPLIT_ERR_UNSUPPORTED;
  cuuint64_t dims[2] = {width, height};
  cuuint64_t strides[1] = {row_bytes};
  cuuint32_t box[2] = {box_w, box_h};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(map, dtype, 2, const_cast<void*>(base), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? SPLIT_OK : SPLIT_ERR_INVALID;
}

namespace stn {

constexpr int TH = kTileH, TW = kTileW, kThreads = 256;
constexpr unsigned kWaitLimit = 1u << 24;

// Stage a box of `sw` x `sh` elements starting at (x0, y0) into `dst`: TMA
// when a tensor map is given, plain coalesced loads (zero outside) otherwise.
template <typename T>
__device__ __forceinline__ bool stage(T* dst, const CUtensorMap* map, const T* src, int W, int H,
                                      int x0, int y0, int sw, int sh, uint64_t* bar, int* status) {
  if (map) {
    if (threadIdx.x == 0) {
      mbar_init(bar, 1);
      mbar_arrive_expect_tx(bar, (unsigned)(sw * sh * sizeof(T)));
      tma_load_2d(dst, map, x0, y0, bar);
    }
    __syncthreads();
    if (!mbar_wait(bar, 0, kWaitLimit)) {
      set_status(status, SPLIT_ERR_TIMEOUT);
      mbar_wait(bar, 0, kWaitLimit);  // let the copy land before leaving
      return false;
    }
    return true;
  }
  if (sizeof(T) == 1 && sw % 4 == 0) {
    // bytes: a warp per staged row, 4 bytes per lane and load.  A group wholly
    // inside the image row is read as one 32-bit word (two words and a funnel
    // shift when the row is not 4-byte aligned; both words hold bytes of the
    // row, so they lie in mapped memory); edge groups go byte by byte.
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int r = threadIdx.x >> 5; r < sh; r += nw) {
      const int gy = y0 + r;
      uint32_t* drow = reinterpret_cast<uint32_t*>(dst + r * sw);
      if (gy < 0 || gy >= H) {
        for (int c = lane; c < sw / 4; c += 32) drow[c] = 0u;
        continue;
      }
      const unsigned char* srow = reinterpret_cast<const unsigned char*>(src) + (size_t)gy * W;
      for (int c = lane; c < sw / 4; c += 32) {
        const int gx = x0 + 4 * c;
        uint32_t v;
        if (gx >= 0 && gx + 3 < W) {
          const uintptr_t a = reinterpret_cast<uintptr_t>(srow + gx);
          const uint32_t* w = reinterpret_cast<const uint32_t*>(a & ~(uintptr_t)3);
          const unsigned sh8 = 8u * (unsigned)(a & 3);
          v = sh8 ? __funnelshift_r(__ldg(w), __ldg(w + 1), sh8) : __ldg(w);
        } else {
          v = 0u;
#pragma unroll
          for (int q = 0; q < 4; ++q)
            if (gx + q >= 0 && gx + q < W) v |= (uint32_t)srow[gx + q] << (8 * q);
        }
        drow[c] = v;
      }
    }
  } else {
    for (int i = threadIdx.x; i < sw * sh; i += blockDim.x) {
      const int r = i / sw, c = i % sw;
      const int gx = x0 + c, gy = y0 + r;
      dst[i] = (gx >= 0 && gy >= 0 && gx < W && gy < H) ? src[(size_t)gy * W + gx] : T(0);
    }
  }
  __syncthreads();
  return true;
}

// ---- erosion ---------------------------------------------------------------
struct ErodeArgs {
  const int32_t* in;    // arena
  int32_t* out;         // arena
  int R, XP;
  const mrg::State* mstate;  // fused relabel when not null
  const int32_t* mfin;
  int local_labels;     // write labels minus the image's arena offset
  int* status;
};

// TMA bits of ImgGeom::tma_ok
constexpr int kTmaLabels = 1, kTmaRgb = 2;

__device__ __forceinline__ const CUtensorMap* pick_map(const Geoms& gs, const TileRef& t,
                                                       const CUtensorMap* single, int bit) {
  if (gs.n == 1) return single;
  return (gs.maps && (t.tma_ok & bit)) ? gs.maps + t.img : nullptr;
}

template <bool R1>
__global__ void __launch_bounds__(kThreads)
erode_kernel(const __grid_constant__ CUtensorMap tmap, bool use_tma, ErodeArgs a, Geoms gs) {
  pdl_wait();
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t bar;
  const int R = R1 ? 1 : a.R, XP = R1 ? 4 : a.XP;
  const int SW = TW + 2 * XP, SH = TH + 2 * R;
  int32_t* lab = reinterpret_cast<int32_t*>(smem);
  const TileRef t = tile_ref(gs, blockIdx.x);
  const int W = t.W, H = t.H, tx0 = t.tx0, ty0 = t.ty0;
  const CUtensorMap* map = pick_map(gs, t, use_tma ? &tmap : nullptr, kTmaLabels);
  if (!stage<int32_t>(lab, map, a.in + t.off, W, H, tx0 - XP, ty0 - R, SW, SH, &bar, a.status))
    return;
  if (a.mstate) {
    const mrg::State ms = *a.mstate;
    if (R1) {
      // 72 x 34 entries, four consecutive ones per step (the staged tile is
      // 16-byte aligned); an entry equal to the one before it takes that
      // one's result instead of gathering again
      static_assert((TW + 8) * (TH + 2) % 4 == 0, "whole int4 steps");
      int4* l4 = reinterpret_cast<int4*>(lab);
      for (int i = threadIdx.x; i < SW * SH / 4; i += blockDim.x) {
        const int4 v = l4[i];
        int4 o;
        o.x = mrg::relabel(ms, a.mfin, v.x);
        o.y = v.y == v.x ? o.x : mrg::relabel(ms, a.mfin, v.y);
        o.z = v.z == v.y ? o.y : mrg::relabel(ms, a.mfin, v.z);
        o.w = v.w == v.z ? o.z : mrg::relabel(ms, a.mfin, v.w);
        l4[i] = o;
      }
    } else {
      for (int i = threadIdx.x; i < SW * SH; i += blockDim.x)
        lab[i] = mrg::relabel(ms, a.mfin, lab[i]);
    }
    __syncthreads();
  }
  const int base = a.local_labels ? (int)t.off : 0;
  int32_t* out = a.out + t.off;
  if (R1) {
    // thread: column c of the tile, rows [r0, r0 + kStrip); the 3 x 3 window
    // slides down the column in registers, each row as its centre value and
    // a flag for "left == centre == right"
    constexpr int kGroups = kThreads / TW, kStrip = TH / kGroups;
    static_assert(kThreads % TW == 0 && TH % kGroups == 0, "whole column strips");
    const int c = threadIdx.x % TW, r0 = (threadIdx.x / TW) * kStrip;
    const int x = tx0 + c;
    if (x >= W) return;
    const bool xin = x >= 1 && x + 1 < W;
    const int* q = lab + r0 * SW + (c + XP);   // staged row r0 = image row ty0 + r0 - 1
    int up = q[0], cu = q[SW];
    bool tu = q[-1] == up && q[1] == up;
    bool tc = q[SW - 1] == cu && q[SW + 1] == cu;
#pragma unroll
    for (int k = 0; k < kStrip; ++k) {
      const int y = ty0 + r0 + k;
      if (y >= H) break;
      const int* d = q + (k + 2) * SW;
      const int dn = d[0];
      const bool td = d[-1] == dn && d[1] == dn;
      const bool keep = xin && y >= 1 && y + 1 < H && tu && tc && td && up == cu && dn == cu;
      out[(size_t)y * W + x] = keep ? cu - base : -1;
      up = cu;
      cu = dn;
      tu = tc;
      tc = td;
    }
    return;
  }
  // separable square window: vertical run test per staged column, then the
  // horizontal test over the vertical flags
  unsigned char* vert = smem + (size_t)SW * SH * sizeof(int32_t);
  for (int i = threadIdx.x; i < TH * SW; i += blockDim.x) {
    const int r = i / SW, c = i % SW;
    const int* p = lab + (r + R) * SW + c;
    const int v = p[0];
    bool ok = true;
    for (int dy = -R; dy <= R && ok; ++dy) ok = p[dy * SW] == v;
    vert[i] = ok;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < TH * TW; i += blockDim.x) {
    const int r = i / TW, c = i % TW;
    const int x = tx0 + c, y = ty0 + r;
    if (x >= W || y >= H) continue;
    const int* p = lab + (r + R) * SW + (c + XP);
    const unsigned char* f = vert + r * SW + (c + XP);
    const int v = p[0];
    bool keep = x >= R && y >= R && x + R < W && y + R < H;
    for (int dx = -R; dx <= R && keep; ++dx) keep = p[dx] == v && f[dx];
    out[(size_t)y * W + x] = keep ? v - base : -1;
  }
}

inline int erode_halo(int R) { return (R + 3) / 4 * 4; }

static int erode_geoms_launch(const int32_t* in, int32_t* out, const Geoms& gs, int R,
                              const mrg::State* ms, const int32_t* mfin, int local_labels,
                              int* status, cudaStream_t st) {
  const int XP = erode_halo(R);
  const int SW = TW + 2 * XP, SH = TH + 2 * R;
  CUtensorMap map;
  memset(&map, 0, sizeof(map));
  bool use_tma = false;
  if (gs.n == 1)
    use_tma = make_tmap_2d(&map, CU_TENSOR_MAP_DATA_TYPE_INT32, 4, in, (uint64_t)gs.one.W,
                           (uint64_t)gs.one.H, (uint64_t)gs.one.W * 4, (uint32_t)SW,
                           (uint32_t)SH) == SPLIT_OK;
  ErodeArgs a{in, out, R, XP, ms, mfin, local_labels, status};
  size_t smem = (size_t)SW * SH * sizeof(int32_t);
  if (R == 1) {
    launch_pdl(erode_kernel<true>, dim3(gs.total_tiles), dim3(kThreads), smem, st, map, use_tma, a,
               gs);
  } else {
    smem += (size_t)TH * SW;
    if (smem > 48 * 1024)
      SG_CUDA_TRY(cudaFuncSetAttribute(erode_kernel<false>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    launch_pdl(erode_kernel<false>, dim3(gs.total_tiles), dim3(kThreads), smem, st, map, use_tma,
               a, gs);
  }
  return launch_status();
}

static int erode_launch(const int32_t* in, int32_t* out, int W, int H, int R,
                        const mrg::State* ms, const int32_t* mfin, int* status, cudaStream_t st) {
  return erode_geoms_launch(in, out, single_geom(W, H), R, ms, mfin, 0, status, st);
}

// ---- luminance ----------------------------------------------------------------
// sRGB byte -> linear * 100 after the sample's clamp to >= 1/255
// (samples/src/main.cu:170-173, conversion.inl:15-20).
__device__ __forceinline__ float lin100(int byte) {
  float v = (float)byte / 255.0f;
  v = fmaxf(v, 1.0f / 255.0f);
  const float r1 = 1.0f / 1.055f, r2 = 1.0f / 12.92f;
  const float l = v > 0.04045f ? powf(__fmul_rn(__fadd_rn(v, 0.055f), r1), 2.4f) : __fmul_rn(v, r2);
  return __fmul_rn(l, 100.0f);
}

// L* / 100 from linear channels (conversion.inl:22-24 Y row, :46-64 L*).
__device__ __forceinline__ float lum_from_lin(float r, float g, float b) {
  const float Y = __fadd_rn(__fadd_rn(__fmul_rn(r, 0.2126729f), __fmul_rn(g, 0.7151522f)),
                            __fmul_rn(b, 0.0721750f));
  const float y = __fmul_rn(Y, 0.01f);
  const float fy = y > 0.008856f ? cbrtf(y) : __fadd_rn(__fmul_rn(7.787f, y), 16.0f / 116.0f);
  return __fmul_rn(__fsub_rn(__fmul_rn(116.0f, fy), 16.0f), 0.01f);
}

// ---- Sobel normals --------------------------------------------------------------
// h is a (TH + 2) x (TW + 2) tile of heights with a one-pixel halo; outside
// the image the accessor returns 0 (row/column ends are zero-extended) and
// the differencing rows/columns are clamped (sobel_normals.cu:49-83).
__device__ __forceinline__ void sobel_tile(const float* h, int hp, int tx0, int ty0, int W, int H,
                                           float zinv, float* out) {
  const size_t n = (size_t)W * H;
  if (tx0 >= 1 && ty0 >= 1 && tx0 + TW < W && ty0 + TH < H) {
    // the tile and its one-pixel ring lie inside the image: no clamping and
    // no bounds checks; the same sums in the same order as below.  Thread:
    // column c, rows [r0, r0 + kStrip); the 3 x 3 window and the rows'
    // horizontal [1 2 1] sums slide down the column in registers.
    constexpr int kGroups = kThreads / TW, kStrip = TH / kGroups;
    static_assert(kThreads % TW == 0 && TH % kGroups == 0, "whole column strips");
    const float zz = __fmul_rn(zinv, zinv), za = fabsf(zinv);
    const int c = threadIdx.x % TW, r0 = (threadIdx.x / TW) * kStrip;
    const float* q = h + r0 * hp + (c + 1);   // the row above pixel row r0
    float al = q[-1], ar = q[1];
    float bl = q[hp - 1], bm = q[hp], br = q[hp + 1];
    float sa = __fadd_rn(__fadd_rn(al, __fmul_rn(2.0f, q[0])), ar);
    float sbm = __fadd_rn(__fadd_rn(bl, __fmul_rn(2.0f, bm)), br);
    size_t g = (size_t)(ty0 + r0) * W + tx0 + c;
#pragma unroll
    for (int k = 0; k < kStrip; ++k, g += W) {
      const float* d = q + (k + 2) * hp;   // the row below pixel row r0 + k
      const float dl = d[-1], dm = d[0], dr = d[1];
      const float sd = __fadd_rn(__fadd_rn(dl, __fmul_rn(2.0f, dm)), dr);
      const float tr = __fadd_rn(__fadd_rn(ar, __fmul_rn(2.0f, br)), dr);
      const float tl = __fadd_rn(__fadd_rn(al, __fmul_rn(2.0f, bl)), dl);
      const float gy = __fsub_rn(sd, sa);
      const float gx = __fsub_rn(tr, tl);
      const float rm = rsqrtf(__fmaf_rn(gx, gx, __fmaf_rn(gy, gy, zz)));
      out[g] = __fmul_rn(gx, rm);
      out[n + g] = __fmul_rn(gy, rm);
      out[2 * n + g] = __fmul_rn(za, rm);
      al = bl;
      ar = br;
      bl = dl;
      bm = dm;
      br = dr;
      sa = sbm;
      sbm = sd;
    }
    return;
  }
  for (int i = threadIdx.x; i < TH * TW; i += blockDim.x) {
    const int r = i / TW, c = i % TW;
    const int x = tx0 + c, y = ty0 + r;
    if (x >= W || y >= H) continue;
    auto hz = [&](int xx, int yy) -> float {
      if (xx < 0 || xx >= W || yy < 0 || yy >= H) return 0.0f;
      return h[(yy - ty0 + 1) * hp + (xx - tx0 + 1)];
    };
    const int yb = min(y + 1, H - 1), yt = max(y - 1, 0);
    const int xr = min(x + 1, W - 1), xl = max(x - 1, 0);
    const float sb = __fadd_rn(__fadd_rn(hz(x - 1, yb), __fmul_rn(2.0f, hz(x, yb))), hz(x + 1, yb));
    const float st = __fadd_rn(__fadd_rn(hz(x - 1, yt), __fmul_rn(2.0f, hz(x, yt))), hz(x + 1, yt));
    const float tr = __fadd_rn(__fadd_rn(hz(xr, y - 1), __fmul_rn(2.0f, hz(xr, y))), hz(xr, y + 1));
    const float tl = __fadd_rn(__fadd_rn(hz(xl, y - 1), __fmul_rn(2.0f, hz(xl, y))), hz(xl, y + 1));
    const float gy = __fsub_rn(sb, st);
    const float gx = __fsub_rn(tr, tl);
    const float m2 = __fmaf_rn(gx, gx, __fmaf_rn(gy, gy, __fmul_rn(zinv, zinv)));
    const float rm = rsqrtf(m2);
    const size_t g = (size_t)y * W + x;
    out[g] = __fmul_rn(gx, rm);
    out[n + g] = __fmul_rn(gy, rm);
    out[2 * n + g] = __fmul_rn(fabsf(zinv), rm);
  }
}

struct NormArgs {
  const float* heights;  // arena
  const uint8_t* rgb;    // arena (3 bytes per pixel)
  float* out;            // per image: 3 planes at 3 * (arena offset)
  float zinv;
  int* status;
  float4* features;      // optional, arena: (byte / 255) x 3, 0 per pixel
};

// heights (float) -> normals; staged box (TW + 8) x (TH + 2) from (tx0-4, ty0-1)
__global__ void __launch_bounds__(kThreads)
normals_kernel(const __grid_constant__ CUtensorMap tmap, bool use_tma, NormArgs a, Geoms gs) {
  __shared__ __align__(128) float tile[(TH + 2) * (TW + 8)];
  __shared__ __align__(8) uint64_t bar;
  const TileRef t = tile_ref(gs, blockIdx.x);
  constexpr int SW = TW + 8, SH = TH + 2;
  const CUtensorMap* map = pick_map(gs, t, use_tma ? &tmap : nullptr, kTmaLabels);
  if (!stage<float>(tile, map, a.heights + t.off, t.W, t.H, t.tx0 - 4, t.ty0 - 1, SW, SH, &bar,
                    a.status))
    return;
  // shift the view so that column index 0 is x = tx0 - 1
  sobel_tile(tile + 3, SW, t.tx0, t.ty0, t.W, t.H, a.zinv, a.out + 3 * t.off);
}

// RGB8 -> luminance tile -> normals; staged bytes (3 TW + 32) x (TH + 2)
// from byte column 3 tx0 - 16.  With a.features set, the tile's pixels also
// get the float4 features pack_kernel writes (same table, same values), so a
// pipeline that needs both reads the bytes once.
__global__ void __launch_bounds__(kThreads)
normals_rgb8_kernel(const __grid_constant__ CUtensorMap tmap, bool use_tma, NormArgs a,
                    Geoms gs) {
  pdl_wait();
  constexpr int SWB = 3 * TW + 32, SH = TH + 2, HP = TW + 2;
  __shared__ __align__(128) unsigned char bytes[SWB * SH];
  __shared__ float lum[SH * HP];
  __shared__ float lin[256];
  __shared__ float u8[256];
  __shared__ __align__(8) uint64_t bar;
  const TileRef t = tile_ref(gs, blockIdx.x);
  for (int i = threadIdx.x; i < 256; i += blockDim.x) {
    lin[i] = lin100(i);
    u8[i] = (float)i / 255.0f;
  }
  const CUtensorMap* map = pick_map(gs, t, use_tma ? &tmap : nullptr, kTmaRgb);
  if (!stage<unsigned char>(bytes, map, a.rgb + 3 * t.off, 3 * t.W, t.H, 3 * t.tx0 - 16,
                            t.ty0 - 1, SWB, SH, &bar, a.status))
    return;
  for (int i = threadIdx.x; i < SH * HP; i += blockDim.x) {
    const int r = i / HP, c = i % HP;  // pixel x = tx0 - 1 + c
    const unsigned char* p = bytes + r * SWB + 3 * c + 13;
    lum[i] = lum_from_lin(lin[p[0]], lin[p[1]], lin[p[2]]);
  }
  if (a.features) {
    float4* f4 = a.features + t.off;
    for (int i = threadIdx.x; i < TH * TW; i += blockDim.x) {
      const int r = i / TW, c = i % TW;
      const int x = t.tx0 + c, y = t.ty0 + r;
      if (x >= t.W || y >= t.H) continue;
      const unsigned char* p = bytes + (r + 1) * SWB + 3 * c + 16;   // pixel x
      f4[(size_t)y * t.W + x] = make_float4(u8[p[0]], u8[p[1]], u8[p[2]], 0.0f);
    }
  }
  __syncthreads();
  sobel_tile(lum, HP, t.tx0, t.ty0, t.W, t.H, a.zinv, a.out + 3 * t.off);
}

// ---- feature packing ------------------------------------------------------------
__global__ void pack_kernel(const uint8_t* __restrict__ rgb, int64_t n, float4* __restrict__ f4,
                            float* __restrict__ lumo) {
  __shared__ float u8[256];
  __shared__ float lin[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) {
    u8[i] = (float)i / 255.0f;
    lin[i] = lin100(i);
  }
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int r = rgb[3 * i], g = rgb[3 * i + 1], b = rgb[3 * i + 2];
    if (f4) f4[i] = make_float4(u8[r], u8[g], u8[b], 0.0f);
    if (lumo) lumo[i] = lum_from_lin(lin[r], lin[g], lin[b]);
  }
}

// ---- intensity / chroma -----------------------------------------------------------
// The sample's (intensity, r / intensity, g / intensity) planes: channels
// byte / 255 clamped to >= 1/255 (main.cu:169-173), intensity = (r + g + b)
// * (1/3), one reciprocal, two products (conversion.inl:99-108), FP32 in the
// reference's order.  Planar 3 x n output.
__global__ void ic_kernel(const uint8_t* __restrict__ rgb, int64_t n, float* __restrict__ out) {
  __shared__ float v8[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x)
    v8[i] = fmaxf(__fdiv_rn((float)i, 255.0f), __fdiv_rn(1.0f, 255.0f));
  __syncthreads();
  const float third = __fdiv_rn(1.0f, 3.0f);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float r = v8[rgb[3 * i]], g = v8[rgb[3 * i + 1]], b = v8[rgb[3 * i + 2]];
    const float in = __fmul_rn(__fadd_rn(__fadd_rn(r, g), b), third);
    const float ri = __fdiv_rn(1.0f, in);
    out[i] = in;
    out[n + i] = __fmul_rn(r, ri);
    out[2 * n + i] = __fmul_rn(g, ri);
  }
}

// ---- L*a*b* and the beta feature ------------------------------------------------
// L*a*b* of an sRGB byte triple after the sample's clamp (conversion.inl:8-25
// rgb_to_xyz, :46-64 xyz_to_lab; operations in the reference's order, FP32).
struct Lab {
  float L, a, b;
};
__device__ __forceinline__ float lab_f(float t) {
  return t > 0.008856f ? cbrtf(t) : __fadd_rn(__fmul_rn(7.787f, t), 16.0f / 116.0f);
}
__device__ __forceinline__ Lab lab_from_lin(float r, float g, float b) {
  const float X = __fadd_rn(__fadd_rn(__fmul_rn(r, 0.4124564f), __fmul_rn(g, 0.3575761f)),
                            __fmul_rn(b, 0.1804375f));
  const float Y = __fadd_rn(__fadd_rn(__fmul_rn(r, 0.2126729f), __fmul_rn(g, 0.7151522f)),
                            __fmul_rn(b, 0.0721750f));
  const float Z = __fadd_rn(__fadd_rn(__fmul_rn(r, 0.0193339f), __fmul_rn(g, 0.1191920f)),
                            __fmul_rn(b, 0.9503041f));
  const float fx = lab_f(__fmul_rn(X, 1.0f / 95.047f));
  const float fy = lab_f(__fmul_rn(Y, 0.01f));
  const float fz = lab_f(__fmul_rn(Z, 1.0f / 108.883f));
  Lab o;
  o.L = __fsub_rn(__fmul_rn(116.0f, fy), 16.0f);
  o.a = __fmul_rn(500.0f, __fsub_rn(fx, fy));
  o.b = __fmul_rn(200.0f, __fsub_rn(fy, fz));
  return o;
}

// order-preserving integer key of a float (for atomicMax over any sign)
__device__ __forceinline__ unsigned okey(float v) {
  const unsigned u = __float_as_uint(v);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float okey_inv(unsigned k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// pass 1: the largest L* and the largest |a*| of the image (beta_feature.cu:52-64)
__global__ void lab_max_kernel(const uint8_t* __restrict__ rgb, int64_t n, unsigned* maxima) {
  __shared__ float lin[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) lin[i] = lin100(i);
  __syncthreads();
  unsigned kl = 0, ka = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const Lab c = lab_from_lin(lin[rgb[3 * i]], lin[rgb[3 * i + 1]], lin[rgb[3 * i + 2]]);
    kl = max(kl, okey(c.L));
    ka = max(ka, okey(fabsf(c.a)));
  }
  kl = __reduce_max_sync(0xffffffffu, kl);
  ka = __reduce_max_sync(0xffffffffu, ka);
  if ((threadIdx.x & 31) == 0) {
    atomicMax(maxima, kl);
    atomicMax(maxima + 1, ka);
  }
}

// pass 2: (beta, a*, b*) features and L* (beta_feature.cu:26-45: beta = -mu
// below 0.2 L*max, +mu above 0.95 L*max, for pixels with |a*| and |b*| below
// 0.2 max |a*|; 0 otherwise)
__global__ void lab_beta_kernel(const uint8_t* __restrict__ rgb, int64_t n, const unsigned* maxima,
                                float mu, float* __restrict__ out, int float4_out,
                                float* __restrict__ lumo) {
  __shared__ float lin[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) lin[i] = lin100(i);
  __syncthreads();
  const float lmax = okey_inv(maxima[0]);
  const float lambda = __fmul_rn(0.2f, okey_inv(maxima[1]));
  const float lo = __fmul_rn(lmax, 0.20f), hi = __fmul_rn(lmax, 0.95f);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const Lab c = lab_from_lin(lin[rgb[3 * i]], lin[rgb[3 * i + 1]], lin[rgb[3 * i + 2]]);
    float beta = 0.0f;
    if (fabsf(c.a) < lambda && fabsf(c.b) < lambda) {
      if (c.L < lo) beta = -mu;
      else if (c.L > hi) beta = mu;
    }
    if (float4_out) {
      reinterpret_cast<float4*>(out)[i] = make_float4(beta, c.a, c.b, 0.0f);
    } else {
      out[i] = beta;
      out[n + i] = c.a;
      out[2 * n + i] = c.b;
    }
    if (lumo) lumo[i] = c.L;
  }
}

// Batches: the same two passes over the tile grid of many images, with
// per-image maxima (2 words per image: L*max and |a*|max keys).  A block is
// one 32 x 64 tile of one image, so no pixel searches for its image.
__global__ void __launch_bounds__(kThreads)
lab_max_geoms_kernel(const uint8_t* __restrict__ rgb, Geoms gs, unsigned* maxima) {
  __shared__ float lin[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) lin[i] = lin100(i);
  __syncthreads();
  const TileRef t = tile_ref(gs, blockIdx.x);
  unsigned kl = 0, ka = 0;
  for (int i = threadIdx.x; i < TH * TW; i += blockDim.x) {
    const int x = t.tx0 + (i % TW), y = t.ty0 + i / TW;
    if (x >= t.W || y >= t.H) continue;
    const uint8_t* p = rgb + 3 * (t.off + (long long)y * t.W + x);
    const Lab c = lab_from_lin(lin[p[0]], lin[p[1]], lin[p[2]]);
    kl = max(kl, okey(c.L));
    ka = max(ka, okey(fabsf(c.a)));
  }
  kl = __reduce_max_sync(0xffffffffu, kl);
  ka = __reduce_max_sync(0xffffffffu, ka);
  if ((threadIdx.x & 31) == 0 && kl) {
    atomicMax(maxima + 2 * t.img, kl);
    atomicMax(maxima + 2 * t.img + 1, ka);
  }
}

__global__ void __launch_bounds__(kThreads)
lab_beta_geoms_kernel(const uint8_t* __restrict__ rgb, Geoms gs, const unsigned* maxima, float mu,
                      float4* __restrict__ out) {
  __shared__ float lin[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) lin[i] = lin100(i);
  __syncthreads();
  const TileRef t = tile_ref(gs, blockIdx.x);
  const float lmax = okey_inv(maxima[2 * t.img]);
  const float lambda = __fmul_rn(0.2f, okey_inv(maxima[2 * t.img + 1]));
  const float lo = __fmul_rn(lmax, 0.20f), hi = __fmul_rn(lmax, 0.95f);
  for (int i = threadIdx.x; i < TH * TW; i += blockDim.x) {
    const int x = t.tx0 + (i % TW), y = t.ty0 + i / TW;
    if (x >= t.W || y >= t.H) continue;
    const long long g = t.off + (long long)y * t.W + x;
    const uint8_t* p = rgb + 3 * g;
    const Lab c = lab_from_lin(lin[p[0]], lin[p[1]], lin[p[2]]);
    float beta = 0.0f;
    if (fabsf(c.a) < lambda && fabsf(c.b) < lambda) {
      if (c.L < lo) beta = -mu;
      else if (c.L > hi) beta = mu;
    }
    out[g] = make_float4(beta, c.a, c.b, 0.0f);
  }
}

}  // namespace stn

// The sample's Lab + beta features of every image of a batch into its float4
// arena (maxima: 2 words per image, cleared here).
int lab_beta_geoms(const uint8_t* rgb, const Geoms& gs, float mu, float* features4,
                   unsigned* maxima, cudaStream_t st) {
  SG_CUDA_TRY(cudaMemsetAsync(maxima, 0, sizeof(unsigned) * 2 * (size_t)gs.n, st));
  stn::lab_max_geoms_kernel<<<gs.total_tiles, stn::kThreads, 0, st>>>(rgb, gs, maxima);
  SG_TRY(launch_status());
  stn::lab_beta_geoms_kernel<<<gs.total_tiles, stn::kThreads, 0, st>>>(
      rgb, gs, maxima, mu, reinterpret_cast<float4*>(features4));
  return launch_status();
}
}  // namespace sg

using namespace sg;

extern "C" int split_erode(const int32_t* labels_in, int32_t* labels_out, int width, int height,
                           int radius, void* stream) {
  if (!labels_in || !labels_out || width < 1 || height < 1 || radius < 1 || radius > 16)
    return SPLIT_ERR_INVALID;
  if ((int64_t)width * height > 0x7fffffffLL) return SPLIT_ERR_INVALID;
  const size_t n = (size_t)width * height;
  const char* a = reinterpret_cast<const char*>(labels_in);
  const char* b = reinterpret_cast<const char*>(labels_out);
  if (a < b + n * 4 && b < a + n * 4) return SPLIT_ERR_INVALID;
  return stn::erode_launch(labels_in, labels_out, width, height, radius, nullptr, nullptr,
                           nullptr, as_stream(stream));
}

extern "C" int split_erode_mapped(const int32_t* labels_in, int32_t* labels_out, int width,
                                  int height, int radius, const void* merge_workspace,
                                  void* stream) {
  if (!labels_in || !labels_out || !merge_workspace || width < 1 || height < 1 || radius < 1 ||
      radius > 16)
    return SPLIT_ERR_INVALID;
  if ((int64_t)width * height > 0x7fffffffLL) return SPLIT_ERR_INVALID;
  const size_t n = (size_t)width * height;
  const char* a = reinterpret_cast<const char*>(labels_in);
  const char* b = reinterpret_cast<const char*>(labels_out);
  if (a < b + n * 4 && b < a + n * 4) return SPLIT_ERR_INVALID;
  MergeView mv;
  SG_TRY(merge_view(merge_workspace, width, height, &mv));
  return stn::erode_launch(labels_in, labels_out, width, height, radius, mv.state, mv.fin,
                           nullptr, as_stream(stream));
}

extern "C" int split_sobel_normals(const float* heights, int width, int height, float depth,
                                   float* normals, void* stream) {
  if (!heights || !normals || width < 1 || height < 1) return SPLIT_ERR_INVALID;
  if ((int64_t)width * height > 0x7fffffffLL) return SPLIT_ERR_INVALID;
  CUtensorMap map;
  memset(&map, 0, sizeof(map));
  const bool use_tma =
      make_tmap_2d(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, heights, (uint64_t)width,
                   (uint64_t)height, (uint64_t)width * 4, stn::TW + 8, stn::TH + 2) == SPLIT_OK;
  stn::NormArgs a{heights, nullptr, normals, 1.0f / fmaxf(0.001f, depth), nullptr};
  const Geoms gs = single_geom(width, height);
  stn::normals_kernel<<<gs.total_tiles, stn::kThreads, 0, as_stream(stream)>>>(map, use_tma, a,
                                                                                gs);
  return launch_status();
}

namespace sg {
int normals_rgb8_geoms(const uint8_t* rgb, const Geoms& gs, float depth, float* normals,
                       float* features4, cudaStream_t st) {
  CUtensorMap map;
  memset(&map, 0, sizeof(map));
  bool use_tma = false;
  if (gs.n == 1)
    use_tma = make_tmap_2d(&map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, rgb, (uint64_t)gs.one.W * 3,
                           (uint64_t)gs.one.H, (uint64_t)gs.one.W * 3, 3 * stn::TW + 32,
                           stn::TH + 2) == SPLIT_OK;
  stn::NormArgs a{nullptr, rgb, normals, 1.0f / fmaxf(0.001f, depth),
                  nullptr, reinterpret_cast<float4*>(features4)};
  launch_pdl(stn::normals_rgb8_kernel, dim3(gs.total_tiles), dim3(stn::kThreads), 0, st, map,
             use_tma, a, gs);
  return launch_status();
}

int erode_geoms(const int32_t* in, int32_t* out, const Geoms& gs, int radius, const void* mstate,
                const int32_t* mfin, int local_labels, cudaStream_t st) {
  return stn::erode_geoms_launch(in, out, gs, radius, static_cast<const mrg::State*>(mstate),
                                 mfin, local_labels, nullptr, st);
}

// Tensor maps of one batch image for the batch stencils (labels for the
// erosion, RGB8 bytes for the normals).  Returns the TMA bits that apply.
int batch_image_maps(const int32_t* labels, const uint8_t* rgb, int W, int H, int radius,
                     CUtensorMap* lab_map, CUtensorMap* rgb_map) {
  int bits = 0;
  const int XP = stn::erode_halo(radius);
  memset(lab_map, 0, sizeof(CUtensorMap));
  memset(rgb_map, 0, sizeof(CUtensorMap));
  if (labels && make_tmap_2d(lab_map, CU_TENSOR_MAP_DATA_TYPE_INT32, 4, labels, (uint64_t)W,
                             (uint64_t)H, (uint64_t)W * 4, (uint32_t)(stn::TW + 2 * XP),
                             (uint32_t)(stn::TH + 2 * radius)) == SPLIT_OK)
    bits |= stn::kTmaLabels;
  if (rgb && make_tmap_2d(rgb_map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, rgb, (uint64_t)W * 3,
                          (uint64_t)H, (uint64_t)W * 3, 3 * stn::TW + 32,
                          stn::TH + 2) == SPLIT_OK)
    bits |= stn::kTmaRgb;
  return bits;
}
}  // namespace sg

extern "C" int split_sobel_normals_rgb8(const uint8_t* rgb, int width, int height, float depth,
                                        float* normals, void* stream) {
  if (!rgb || !normals || width < 1 || height < 1) return SPLIT_ERR_INVALID;
  if ((int64_t)width * height * 3 > 0x7fffffffLL) return SPLIT_ERR_INVALID;
  return normals_rgb8_geoms(rgb, single_geom(width, height), depth, normals, nullptr,
                            as_stream(stream));
}

extern "C" int split_rgb8_to_ic(const uint8_t* rgb, int64_t npixels, float* ic, void* stream) {
  if (!rgb || !ic || npixels <= 0) return SPLIT_ERR_INVALID;
  DeviceInfo di;
  SG_TRY(device_info(&di));
  int64_t blocks = (npixels + 255) / 256;
  if (blocks > (int64_t)di.sm_count * 8) blocks = (int64_t)di.sm_count * 8;
  stn::ic_kernel<<<(int)blocks, 256, 0, as_stream(stream)>>>(rgb, npixels, ic);
  return launch_status();
}

extern "C" int split_pack_rgb8(const uint8_t* rgb, int64_t npixels, float* features4,
                               float* luminance, void* stream) {
  if (!rgb || npixels <= 0 || (!features4 && !luminance)) return SPLIT_ERR_INVALID;
  if (features4 && (reinterpret_cast<uintptr_t>(features4) & 15)) return SPLIT_ERR_INVALID;
  DeviceInfo di;
  SG_TRY(device_info(&di));
  int64_t blocks = (npixels + 255) / 256;
  if (blocks > (int64_t)di.sm_count * 8) blocks = (int64_t)di.sm_count * 8;
  stn::pack_kernel<<<(int)blocks, 256, 0, as_stream(stream)>>>(
      rgb, npixels, reinterpret_cast<float4*>(features4), luminance);
  return launch_status();
}

// Lab + beta features of the sample (samples/src/main.cu:169-173, :215-225):
// two passes over the RGB8 image, nothing else read or written.
extern "C" size_t split_pack_lab_beta_workspace_size(int64_t npixels) {
  (void)npixels;
  return 512;
}

extern "C" int split_pack_lab_beta(const uint8_t* rgb, int64_t npixels, float mu, int layout,
                                   float* features, float* luminance, void* workspace,
                                   size_t workspace_bytes, void* stream) {
  if (!rgb || !features || npixels <= 0 || !(mu >= 0.0f)) return SPLIT_ERR_INVALID;
  if (layout != SPLIT_LAYOUT_PLANAR && layout != SPLIT_LAYOUT_FLOAT4) return SPLIT_ERR_INVALID;
  if (layout == SPLIT_LAYOUT_FLOAT4 && (reinterpret_cast<uintptr_t>(features) & 15))
    return SPLIT_ERR_INVALID;
  if (!workspace || workspace_bytes < 512 || (reinterpret_cast<uintptr_t>(workspace) & 255))
    return SPLIT_ERR_WORKSPACE;
  cudaStream_t st = as_stream(stream);
  unsigned* maxima = reinterpret_cast<unsigned*>(static_cast<char*>(workspace) + 256);
  SG_CUDA_TRY(cudaMemsetAsync(maxima, 0, 2 * sizeof(unsigned), st));
  DeviceInfo di;
  SG_TRY(device_info(&di));
  int64_t blocks = (npixels + 255) / 256;
  if (blocks > (int64_t)di.sm_count * 8) blocks = (int64_t)di.sm_count * 8;
  stn::lab_max_kernel<<<(int)blocks, 256, 0, st>>>(rgb, npixels, maxima);
  SG_TRY(launch_status());
  stn::lab_beta_kernel<<<(int)blocks, 256, 0, st>>>(rgb, npixels, maxima, mu, features,
                                                     layout == SPLIT_LAYOUT_FLOAT4, luminance);
  return launch_status();
}
