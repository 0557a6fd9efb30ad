// Forced include for the CPU (Thrust OMP) build of the reference's
// segmentation sources (oracle/refbuild.py).  Test infrastructure only.
//  - host min/max for the unqualified calls in the sources;
//  - stand-ins that let g++ parse the one CUDA kernel those sources define
//    (it is never launched).
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <ctime>
#include <iostream>
using std::max;
using std::min;

#ifndef __global__
#define __global__
#endif
#ifndef __shared__
#define __shared__
#endif
struct sg_ref_uint3 {
  unsigned x, y, z;
};
static sg_ref_uint3 threadIdx, blockIdx, blockDim;
inline void __syncthreads() {}
