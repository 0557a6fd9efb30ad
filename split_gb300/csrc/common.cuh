// Shared helpers of the sm_103a kernels: status handling, workspace carving,
// the bounded device-wide barrier and small device utilities.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include <utility>

#include <cuda/atomic>

#include "../../include/split_gb300.h"

namespace sg {

// ---------------------------------------------------------------------------
// host-side status helpers
// ---------------------------------------------------------------------------
#define SG_CUDA_TRY(expr)                          \
  do {                                             \
    cudaError_t e_ = (expr);                       \
    if (e_ != cudaSuccess) return SPLIT_ERR_CUDA;  \
  } while (0)

#define SG_TRY(expr)              \
  do {                            \
    int s_ = (expr);              \
    if (s_ != SPLIT_OK) return s_; \
  } while (0)

// Kernels launched by the library since load (every launch site reports
// through launch_status()).
void count_launch();

// Programmatic dependent launch: the kernel may be scheduled while the
// previous kernel on the stream finishes; it must execute pdl_wait() before
// touching anything that kernel writes (and before any write of its own that
// the previous kernel reads).
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                              cudaStream_t st, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

inline int launch_status() {
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e == cudaErrorNoKernelImageForDevice || e == cudaErrorInvalidDeviceFunction)
    return SPLIT_ERR_UNSUPPORTED;
  return e == cudaSuccess ? SPLIT_OK : SPLIT_ERR_CUDA;
}

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Per-device properties cached after the first query.
struct DeviceInfo {
  int device;
  int sm_count;
  int max_smem_optin;
};
int device_info(DeviceInfo* out);

// ---------------------------------------------------------------------------
// workspace layout
// ---------------------------------------------------------------------------
// Every workspace starts with this header.  `status` holds the first error a
// device detected (0 = none).  The barrier words back the device-wide barrier
// of persistent kernels; `count` returns to zero after every barrier.
struct WsHeader {
  int status;
  unsigned barrier_count;
  unsigned barrier_gen;
  unsigned work_counter[2];
  int pad0;
  // layout the workspace's persistent state was last cleared for (0: never)
  unsigned long long stamp;
  int pad[56];
};
static_assert(sizeof(WsHeader) == 256, "header is one 256-byte line");

// Bump allocator over a caller workspace; with base == nullptr it only
// measures, so size queries and carving share one code path.
struct Carver {
  char* base;
  size_t off;
  explicit Carver(void* b) : base(static_cast<char*>(b)), off(0) {}
  template <class T>
  T* take(size_t count) {
    off = (off + 255) & ~size_t(255);
    T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
    off += count * sizeof(T);
    return p;
  }
  size_t size() const { return (off + 255) & ~size_t(255); }
};

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ void set_status(int* st, int code) {
  atomicCAS(st, 0, code);
}

// Status words of the sub-workspaces a composite call (pipeline, batch)
// carves from its own: fold_status moves the first error among them into the
// composite workspace's own status word (read by split_workspace_status) and
// clears them, so that a sub-stage error is never lost and never reported
// twice.
struct StatusSources {
  int* p[8];
  int n;
};
__global__ void fold_status_kernel(int* dst, StatusSources s);
int fold_status(int* dst, const StatusSources& s, cudaStream_t st);
// Clears the sources' status words before the stages run: a reused
// workspace may hold anything where this call's sub-workspace headers lie.
int clear_status(const StatusSources& s, cudaStream_t st);
// Whether `workspace` was last used with layout `key` (a small direct-mapped
// memo; records the key).  After the first run of a layout the fold leaves
// the stage status words at zero, so the clear is needed only on a change
// (a miss only costs a clear).
bool layout_unchanged(const void* workspace, unsigned long long key);

// Iteration limit of every spin wait (about a second with the back-off below).
constexpr unsigned kSpinLimit = 1u << 24;

// Device-wide barrier for a cooperative (co-resident) grid.  Sense is carried
// by a generation counter.  A wait that exceeds `limit` polls (kSpinLimit by
// default) records SPLIT_ERR_TIMEOUT and returns false; callers then leave
// the kernel.  Block `skip` (a test setting; -1: none) returns false at once
// without arriving, so that the others' wait runs out.
__device__ __forceinline__ bool grid_barrier(WsHeader* h, unsigned limit = kSpinLimit,
                                             int skip = -1) {
  __syncthreads();
  __shared__ int ok;
  if (threadIdx.x == 0) {
    cuda::atomic_ref<unsigned, cuda::thread_scope_device> gen(h->barrier_gen);
    cuda::atomic_ref<unsigned, cuda::thread_scope_device> cnt(h->barrier_count);
    const unsigned nblocks = gridDim.x * gridDim.y * gridDim.z;
    const unsigned g = gen.load(cuda::memory_order_relaxed);
    const unsigned lim = limit;
    ok = 1;
    // acq_rel: publish this block's writes, observe the others' on release
    const unsigned arrived = skip == (int)blockIdx.x
                                 ? ~0u
                                 : cnt.fetch_add(1, cuda::memory_order_acq_rel);
    if (arrived == ~0u) {
      ok = 0;
    } else if (arrived == nblocks - 1) {
      cnt.store(0, cuda::memory_order_relaxed);
      gen.fetch_add(1, cuda::memory_order_release);
    } else {
      unsigned spins = 0;
      while (gen.load(cuda::memory_order_acquire) == g) {
        if (++spins > lim) {
          set_status(&h->status, SPLIT_ERR_TIMEOUT);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    if (cuda::atomic_ref<int, cuda::thread_scope_device>(h->status).load(
            cuda::memory_order_relaxed) == SPLIT_ERR_TIMEOUT)
      ok = 0;
  }
  __syncthreads();
  return ok != 0;
}

// Device-wide barrier on a counter that only grows within a launch (the
// launch's setup zeroes it): the k-th barrier (k from 1) is passed when the
// counter reaches k * nblocks, and waiters poll the counter itself, so the
// last arrival releases everyone without a second word to publish.  Limits,
// the skipping block and the timeout status as in grid_barrier.
__device__ __forceinline__ bool grid_barrier_counted(WsHeader* h, unsigned k,
                                                     unsigned limit = kSpinLimit,
                                                     int skip = -1) {
  __syncthreads();
  __shared__ int ok;
  if (threadIdx.x == 0) {
    cuda::atomic_ref<unsigned, cuda::thread_scope_device> cnt(h->barrier_count);
    const unsigned target = k * (gridDim.x * gridDim.y * gridDim.z);
    ok = 1;
    if (skip == (int)blockIdx.x) {
      ok = 0;
    } else {
      // acq_rel: publish this block's writes, observe the others' on release
      unsigned v = cnt.fetch_add(1, cuda::memory_order_acq_rel) + 1u;
      unsigned spins = 0;
      while ((int)(v - target) < 0) {
        if (++spins > limit) {
          set_status(&h->status, SPLIT_ERR_TIMEOUT);
          ok = 0;
          break;
        }
        __nanosleep(64);
        v = cnt.load(cuda::memory_order_acquire);
      }
    }
    if (cuda::atomic_ref<int, cuda::thread_scope_device>(h->status).load(
            cuda::memory_order_relaxed) == SPLIT_ERR_TIMEOUT)
      ok = 0;
  }
  __syncthreads();
  return ok != 0;
}

__device__ __forceinline__ int warp_lane() { return threadIdx.x & 31; }

}  // namespace sg
