// Shape-from-shading normals from a shading image and a light direction.
//
// Restates split/src/split/device/sfs/estimate_normals.cu:251-308: the
// normals x (planar 3 x N) solve A x = b with
//   A = (L L^T) (x) I_N + 2 lambda B (x) I_3        (:260-278, build_M :85-121)
//   B = 5-point Poisson matrix of the H x W grid, off-diagonals -1 for the
//       in-grid 4-neighbours, diagonal 4 - [row on the border] - [column on
//       the border] (build_B :124-171, the reference's valence rule)
//   b = intensity * L  (build_L :232-248),  L normalised (:258-265)
// from x0 = (0, 0, 1) (:283-287) by relaxation until |b - A x| <=
// tol |b| or max_iter sweeps (apply_sor.cu:9-38: omega 1, tol 1e-5, 1500
// iterations), then normalised with z >= 0 (normalize_vectors.cu:15-41).
//
// The reference assembles A with cuSPARSE calls CUDA 12 no longer has
// (:174-230); here A is never stored.  Each sweep is a red-black block
// Gauss-Seidel pass: a pixel's three unknowns are solved together, the 3 x 3
// block c I + L L^T (c = 2 lambda * valence) inverted in closed form,
//   x_i = (r - L (L . r) / (c + L . L)) / c,  r = s_i L + 2 lambda * sum_j x_j,
// with pixels of one colour independent of each other.  B as the reference
// builds it is the grid's graph Laplacian (every row sums to zero), so A is
// only positive semi-definite: a constant field perpendicular to L is in its
// null space, and the relaxation order decides that component of the
// converged normals.  The order here (red, then black, within a sweep) is the
// one the FP64 restatement in the oracle follows.  The residual test runs
// before every sweep as in the reference's monitor; its sums are FP64
// per-block partials added in block order by every block, so every block
// takes the same decision and the result does not depend on timing.
#include <cmath>

#include "common.cuh"

namespace sg {
namespace sor {

constexpr int kThreads = 256;
constexpr int kMaxBlocks = 4096;

struct Args {
  const float* s;      // shading intensity, H x W
  float* x;            // normals, planar 3 x N (in/out)
  int W, H;
  float L0, L1, L2;    // normalised light direction
  float lam2;          // 2 * smoothness weight
  int max_iter;
  float tol;
  double* partial;     // [2][kMaxBlocks]
  int32_t* d_iters;
  WsHeader* hdr;
};

__device__ __forceinline__ int valence(int r, int c, int H, int W) {
  return 4 - ((r == 0 || r == H - 1) ? 1 : 0) - ((c == 0 || c == W - 1) ? 1 : 0);
}

// sum of the in-grid 4-neighbours' unknowns
__device__ __forceinline__ void neighbour_sum(const float* x, long long n, int r, int c, int H,
                                              int W, float (&S)[3]) {
  S[0] = S[1] = S[2] = 0.0f;
  const long long i = (long long)r * W + c;
  const long long nb[4] = {i - W, i - 1, i + 1, i + W};
  const bool in[4] = {r > 0, c > 0, c + 1 < W, r + 1 < H};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (!in[k]) continue;
#pragma unroll
    for (int d = 0; d < 3; ++d) S[d] = __fadd_rn(S[d], __ldcg(x + d * n + nb[k]));
  }
}

// FP64 block sum in a fixed order (warp trees, then warps in order)
__device__ double block_sum(double v) {
  __shared__ double w[kThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int k = 0; k < kThreads / 32; ++k) t += w[k];
  __syncthreads();
  return t;   // valid in thread 0
}

// every block adds the partials of all blocks in block order
__device__ double grid_total(const double* partial) {
  __shared__ double tot;
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (unsigned b = 0; b < gridDim.x; ++b) t += __ldcg(partial + b);
    tot = t;
  }
  __syncthreads();
  return tot;
}

__global__ void __launch_bounds__(kThreads) sor_kernel(Args a) {
  const long long n = (long long)a.W * a.H;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const float L[3] = {a.L0, a.L1, a.L2};
  const float LL = __fadd_rn(__fadd_rn(__fmul_rn(L[0], L[0]), __fmul_rn(L[1], L[1])),
                             __fmul_rn(L[2], L[2]));
  // x0 = (0, 0, 1) and |b|^2 = sum s_i^2 |L|^2
  double acc = 0.0;
  for (long long i = tid; i < n; i += stride) {
    __stcg(a.x + i, 0.0f);
    __stcg(a.x + n + i, 0.0f);
    __stcg(a.x + 2 * n + i, 1.0f);
    const double si = (double)__ldg(a.s + i);
    acc += si * si;
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) __stcg(a.partial + blockIdx.x, acc);
  if (!grid_barrier(a.hdr)) return;
  const double bnorm2 = grid_total(a.partial) * (double)LL;
  const double limit2 = (double)a.tol * (double)a.tol * bnorm2;
  const int Wh = (a.W + 1) / 2;
  const long long nh = (long long)a.H * Wh;
  int it = 0;
  for (;; ++it) {
    // residual of the current iterate
    double* part = a.partial + (size_t)((it + 1) & 1) * kMaxBlocks;
    double r2 = 0.0;
    for (long long i = tid; i < n; i += stride) {
      const int r = (int)(i / a.W), c = (int)(i - (long long)r * a.W);
      float S[3];
      neighbour_sum(a.x, n, r, c, a.H, a.W, S);
      const float xi[3] = {__ldcg(a.x + i), __ldcg(a.x + n + i), __ldcg(a.x + 2 * n + i)};
      const float lx = __fadd_rn(__fadd_rn(__fmul_rn(L[0], xi[0]), __fmul_rn(L[1], xi[1])),
                                 __fmul_rn(L[2], xi[2]));
      const float v = (float)valence(r, c, a.H, a.W);
      const float si = __ldg(a.s + i);
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float lap = __fsub_rn(__fmul_rn(v, xi[d]), S[d]);
        const float ax = __fadd_rn(__fmul_rn(L[d], lx), __fmul_rn(a.lam2, lap));
        const double e = (double)__fsub_rn(__fmul_rn(si, L[d]), ax);
        r2 += e * e;
      }
    }
    r2 = block_sum(r2);
    if (threadIdx.x == 0) __stcg(part + blockIdx.x, r2);
    if (!grid_barrier(a.hdr)) return;
    if (grid_total(part) <= limit2 || it >= a.max_iter) break;
    // one red-black sweep
    for (int colour = 0; colour < 2; ++colour) {
      for (long long k = tid; k < nh; k += stride) {
        const int r = (int)(k / Wh);
        const int c = 2 * (int)(k - (long long)r * Wh) + ((r + colour) & 1);
        if (c >= a.W) continue;
        const long long i = (long long)r * a.W + c;
        float S[3];
        neighbour_sum(a.x, n, r, c, a.H, a.W, S);
        const float si = __ldg(a.s + i);
        float rv[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) rv[d] = __fadd_rn(__fmul_rn(si, L[d]), __fmul_rn(a.lam2, S[d]));
        const float cc = __fmul_rn(a.lam2, (float)valence(r, c, a.H, a.W));
        const float lr = __fadd_rn(__fadd_rn(__fmul_rn(L[0], rv[0]), __fmul_rn(L[1], rv[1])),
                                   __fmul_rn(L[2], rv[2]));
        const float q = __fdiv_rn(lr, __fadd_rn(cc, LL));
#pragma unroll
        for (int d = 0; d < 3; ++d)
          __stcg(a.x + d * n + i, __fdiv_rn(__fsub_rn(rv[d], __fmul_rn(L[d], q)), cc));
      }
      if (!grid_barrier(a.hdr)) return;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && a.d_iters) *a.d_iters = it;
  // unit normals with z >= 0
  for (long long i = tid; i < n; i += stride) {
    const float x0 = __ldcg(a.x + i), x1 = __ldcg(a.x + n + i), x2 = __ldcg(a.x + 2 * n + i);
    const float m = __fadd_rn(__fadd_rn(__fmul_rn(x0, x0), __fmul_rn(x1, x1)), __fmul_rn(x2, x2));
    const float rmag = __fdiv_rn(1.0f, __fsqrt_rn(m));
    a.x[i] = __fmul_rn(x0, rmag);
    a.x[n + i] = __fmul_rn(x1, rmag);
    a.x[2 * n + i] = __fmul_rn(fabsf(x2), rmag);
  }
}

struct Layout {
  WsHeader* hdr;
  double* partial;
  size_t bytes;
};

inline Layout carve(void* ws) {
  Carver c(ws);
  Layout l;
  l.hdr = c.take<WsHeader>(1);
  l.partial = c.take<double>((size_t)2 * kMaxBlocks);
  l.bytes = c.size();
  return l;
}

}  // namespace sor
}  // namespace sg

using namespace sg;

extern "C" size_t split_estimate_normals_workspace_size(int width, int height) {
  if (width < 1 || height < 1) return 0;
  return sor::carve(nullptr).bytes;
}

extern "C" int split_estimate_normals(const float* intensity, int width, int height, float lx,
                                      float ly, float lz, float smoothness, int max_iter,
                                      float tol, float* normals, int32_t* d_iterations,
                                      void* workspace, size_t workspace_bytes, void* stream) {
  using namespace sg::sor;
  if (!intensity || !normals || width < 1 || height < 1 || max_iter < 0 || !(tol >= 0.0f) ||
      !(smoothness > 0.0f))
    return SPLIT_ERR_INVALID;
  if ((int64_t)width * height > 0x7fffffffLL / 3) return SPLIT_ERR_INVALID;
  const float mag2 = lx * lx + ly * ly + lz * lz;
  if (!(mag2 > 0.0f)) return SPLIT_ERR_INVALID;
  Layout l = carve(nullptr);
  if (!workspace || workspace_bytes < l.bytes || (reinterpret_cast<uintptr_t>(workspace) & 255))
    return SPLIT_ERR_WORKSPACE;
  l = carve(workspace);
  cudaStream_t st = as_stream(stream);
  SG_CUDA_TRY(cudaMemsetAsync(l.hdr, 0, sizeof(WsHeader), st));
  DeviceInfo di;
  SG_TRY(device_info(&di));
  int per_sm = 0;
  SG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sor_kernel, kThreads, 0));
  if (per_sm < 1) return SPLIT_ERR_UNSUPPORTED;
  int grid = di.sm_count * per_sm;
  if (grid > kMaxBlocks) grid = kMaxBlocks;
  const int64_t need = ((int64_t)width * height + kThreads - 1) / kThreads;
  if (grid > need) grid = (int)need;
  // the light direction normalised as the reference does (estimate_normals.cu:258-265)
  const float rmag = 1.0f / std::sqrt(mag2);
  Args a{intensity, normals, width, height, lx * rmag, ly * rmag, lz * rmag, 2.0f * smoothness,
         max_iter, tol, l.partial, d_iterations, l.hdr};
  void* args[] = {&a};
  SG_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)sor_kernel, dim3(grid), dim3(kThreads),
                                          args, 0, st));
  return launch_status();
}
