// Packed FP32x2 arithmetic (sm_100 and later: add / sub / mul / fma on two
// single-precision lanes in one instruction).  Each lane is rounded to
// nearest like the scalar __fadd_rn / __fsub_rn / __fmul_rn / __fmaf_rn, so
// results are bit-identical to the scalar forms.
#pragma once

#include <cuda_runtime.h>

namespace sg {

__device__ __forceinline__ float2 fsub2(float2 a, float2 b) {
  float2 r;
  asm("{.reg .b64 a_, b_, r_;\n\t"
      "mov.b64 a_, {%2, %3};\n\tmov.b64 b_, {%4, %5};\n\t"
      "sub.rn.f32x2 r_, a_, b_;\n\tmov.b64 {%0, %1}, r_;}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
__device__ __forceinline__ float2 fadd2(float2 a, float2 b) {
  float2 r;
  asm("{.reg .b64 a_, b_, r_;\n\t"
      "mov.b64 a_, {%2, %3};\n\tmov.b64 b_, {%4, %5};\n\t"
      "add.rn.f32x2 r_, a_, b_;\n\tmov.b64 {%0, %1}, r_;}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
__device__ __forceinline__ float2 fmul2(float2 a, float2 b) {
  float2 r;
  asm("{.reg .b64 a_, b_, r_;\n\t"
      "mov.b64 a_, {%2, %3};\n\tmov.b64 b_, {%4, %5};\n\t"
      "mul.rn.f32x2 r_, a_, b_;\n\tmov.b64 {%0, %1}, r_;}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) {
  float2 r;
  asm("{.reg .b64 a_, b_, c_, r_;\n\t"
      "mov.b64 a_, {%2, %3};\n\tmov.b64 b_, {%4, %5};\n\tmov.b64 c_, {%6, %7};\n\t"
      "fma.rn.f32x2 r_, a_, b_, c_;\n\tmov.b64 {%0, %1}, r_;}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return r;
}

}  // namespace sg
