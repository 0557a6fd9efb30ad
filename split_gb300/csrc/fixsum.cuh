// Order-independent per-cluster sums of pixel features: each feature value is
// rounded to a multiple of 2^-24 and added as a 96-bit fixed-point number
// (the low 32 bits and the signed rest in two 64-bit words, each added with
// 64-bit atomics), so totals do not depend on the order pixels arrive in.
// Used by the many-cluster update and by the many-cluster k-means.
#pragma once

#include "common.cuh"

namespace sg {
namespace fix {

constexpr float kScale = 16777216.0f;        // 2^24
constexpr float kLimit = 274877906944.0f;    // 2^38: |feature| bound of the format

__device__ __forceinline__ unsigned long long shfl_xor_u64(unsigned long long v, int o) {
  const unsigned a = __shfl_xor_sync(0xffffffffu, (unsigned)v, o);
  const unsigned b = __shfl_xor_sync(0xffffffffu, (unsigned)(v >> 32), o);
  return ((unsigned long long)b << 32) | a;
}
__device__ __forceinline__ unsigned long long shfl_down_u64(unsigned long long v, int o) {
  const unsigned a = __shfl_down_sync(0xffffffffu, (unsigned)v, o);
  const unsigned b = __shfl_down_sync(0xffffffffu, (unsigned)(v >> 32), o);
  return ((unsigned long long)b << 32) | a;
}

// Fixed-point words of the features of a pixel with label l (l < 0: zeros).
// A value outside the format's range records SPLIT_ERR_OVERFLOW.
template <int DIM>
__device__ __forceinline__ void quantize(const float (&f)[DIM], int l, int* status,
                                         unsigned long long (&qlo)[DIM],
                                         unsigned long long (&qhi)[DIM]) {
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    if (l >= 0 && !(fabsf(f[d]) < kLimit)) set_status(status, SPLIT_ERR_OVERFLOW);
    const long long q = l >= 0 ? __float2ll_rn(__fmul_rn(f[d], kScale)) : 0ll;
    qlo[d] = (unsigned long long)q & 0xffffffffull;
    qhi[d] = (unsigned long long)(q >> 32);
  }
}

// Adds every lane's words (and a count of one) to the sums of its label l
// (l < 0: nothing), lo / hi at [l * DIM + d], cnt at [l].  All 32 lanes call it.  Lanes hold consecutive
// pixels, so labels come in runs: a warp with one label adds one butterfly
// sum; otherwise a segmented reduction leaves each run's sums in its first
// lane (each lane adds from lane + o while that lane is still in its run) and
// only run heads issue atomics.  Integer sums: the same totals as per-pixel
// adds.
template <int DIM>
__device__ __forceinline__ void warp_add(int l, unsigned long long (&qlo)[DIM],
                                         unsigned long long (&qhi)[DIM],
                                         unsigned long long* __restrict__ lo,
                                         unsigned long long* __restrict__ hi,
                                         unsigned* __restrict__ cnt) {
  const int lane = threadIdx.x & 31;
  const int l0 = __shfl_sync(0xffffffffu, l, 0);
  if (__all_sync(0xffffffffu, l == l0)) {
    if (l0 < 0) return;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        qlo[d] += shfl_xor_u64(qlo[d], o);
        qhi[d] += shfl_xor_u64(qhi[d], o);
      }
    }
    if (lane == 0) {
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        atomicAdd(lo + (size_t)l0 * DIM + d, qlo[d]);
        atomicAdd(hi + (size_t)l0 * DIM + d, qhi[d]);
      }
      atomicAdd(cnt + l0, 32u);
    }
    return;
  }
  const int lprev = __shfl_up_sync(0xffffffffu, l, 1);
  const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || l != lprev);
  const unsigned after = heads & ~(0xffffffffu >> (31 - lane));   // heads right of this lane
  const int run_end = after ? __ffs(after) - 1 : 32;
  unsigned c = l >= 0 ? 1u : 0u;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const bool in_run = lane + o < run_end;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const unsigned long long a = shfl_down_u64(qlo[d], o);
      const unsigned long long b = shfl_down_u64(qhi[d], o);
      if (in_run) {
        qlo[d] += a;
        qhi[d] += b;
      }
    }
    const unsigned cc = __shfl_down_sync(0xffffffffu, c, o);
    if (in_run) c += cc;
  }
  if (l >= 0 && ((heads >> lane) & 1u)) {
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      atomicAdd(lo + (size_t)l * DIM + d, qlo[d]);
      atomicAdd(hi + (size_t)l * DIM + d, qhi[d]);
    }
    atomicAdd(cnt + l, c);
  }
}

// Narrow form of warp_add, for words from features below 2^32 in magnitude
// (|q| < 2^56): a lane's sum of up to 4 pixels' words and any warp sum of
// those stay below 2^63, so each dimension is reduced as one 64-bit word and
// split into the low 32 bits and the signed rest only for the atomics.  The
// totals equal those of warp_add on the same pixels.  `per_lane` pixels
// (1 to 4, the same in every lane) are counted for each lane with l >= 0.
template <int DIM>
__device__ __forceinline__ void warp_add_narrow(int l, long long (&q)[DIM], unsigned per_lane,
                                                unsigned long long* __restrict__ lo,
                                                unsigned long long* __restrict__ hi,
                                                unsigned* __restrict__ cnt) {
  const int lane = threadIdx.x & 31;
  const int l0 = __shfl_sync(0xffffffffu, l, 0);
  int head = l;
  unsigned c = l >= 0 ? per_lane : 0u;
  if (__all_sync(0xffffffffu, l == l0)) {
    if (l0 < 0) return;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
        q[d] += (long long)shfl_xor_u64((unsigned long long)q[d], o);
    }
    c = 32u * per_lane;
    head = lane == 0 ? l0 : -1;
  } else {
    const int lprev = __shfl_up_sync(0xffffffffu, l, 1);
    const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || l != lprev);
    const unsigned after = heads & ~(0xffffffffu >> (31 - lane));
    const int run_end = after ? __ffs(after) - 1 : 32;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const bool in_run = lane + o < run_end;
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        const long long b = (long long)shfl_down_u64((unsigned long long)q[d], o);
        if (in_run) q[d] += b;
      }
      const unsigned cc = __shfl_down_sync(0xffffffffu, c, o);
      if (in_run) c += cc;
    }
    if (!((heads >> lane) & 1u)) head = -1;
  }
  if (head >= 0) {
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      atomicAdd(lo + (size_t)head * DIM + d, (unsigned long long)q[d] & 0xffffffffull);
      atomicAdd(hi + (size_t)head * DIM + d, (unsigned long long)(q[d] >> 32));
    }
    atomicAdd(cnt + head, c);
  }
}

// The exact sum (hi * 2^32 + lo) * 2^-24 divided by n, in FP64, rounded once
// to FP32.  lo's bits above 32 are carried into hi first, so the FP64 sum is
// the correctly rounded value of the integer (for |hi| < 2^53) however the
// adds split it between the two words.
__device__ __forceinline__ float mean(unsigned long long lo, unsigned long long hi, unsigned n) {
  const long long h = (long long)hi + (long long)(lo >> 32);
  const double l = (double)(lo & 0xffffffffull);
  const double S = __dmul_rn(__dadd_rn(__dmul_rn((double)h, 4294967296.0), l), 1.0 / 16777216.0);
  return __double2float_rn(__ddiv_rn(S, (double)n));
}

}  // namespace fix
}  // namespace sg
