// Library-level entry points: version, status strings, device queries and the
// workspace status word.
#include <atomic>
#include <mutex>

#include "common.cuh"

namespace sg {

static std::atomic<unsigned long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int device_info(DeviceInfo* out) {
  static std::mutex mu;
  static DeviceInfo cache[64];
  static bool valid[64] = {false};
  int dev = 0;
  SG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return SPLIT_ERR_CUDA;
  std::lock_guard<std::mutex> lock(mu);
  if (!valid[dev]) {
    DeviceInfo d;
    d.device = dev;
    SG_CUDA_TRY(cudaDeviceGetAttribute(&d.sm_count, cudaDevAttrMultiProcessorCount, dev));
    SG_CUDA_TRY(cudaDeviceGetAttribute(&d.max_smem_optin,
                                       cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    int major = 0;
    SG_CUDA_TRY(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    if (major < 10) return SPLIT_ERR_UNSUPPORTED;
    cache[dev] = d;
    valid[dev] = true;
  }
  *out = cache[dev];
  return SPLIT_OK;
}

}  // namespace sg

using namespace sg;

extern "C" unsigned long long split_launch_count(void) {
  return g_launches.load(std::memory_order_relaxed);
}

extern "C" const char* split_version(void) { return "split_gb300 0.1.0 (sm_103a)"; }

extern "C" const char* split_status_string(int status) {
  switch (status) {
    case SPLIT_OK: return "ok";
    case SPLIT_ERR_INVALID: return "invalid argument";
    case SPLIT_ERR_WORKSPACE: return "workspace too small or misaligned";
    case SPLIT_ERR_NOT_CONVERGED: return "device loop reached its iteration cap";
    case SPLIT_ERR_CUDA: return "CUDA runtime error";
    case SPLIT_ERR_OVERFLOW: return "device table capacity exceeded";
    case SPLIT_ERR_TIMEOUT: return "device-wide barrier wait timed out";
    case SPLIT_ERR_UNSUPPORTED: return "unsupported device";
    default: return "unknown status";
  }
}

namespace sg {
// first error in source order wins, as with set_status
__global__ void fold_status_kernel(int* dst, StatusSources s) {
  pdl_wait();
  if (threadIdx.x != 0) return;
  for (int i = 0; i < s.n; ++i) {
    volatile int* q = s.p[i];
    const int v = *q;
    if (v) {
      set_status(dst, v);
      *q = 0;
    }
  }
}

int fold_status(int* dst, const StatusSources& s, cudaStream_t st) {
  launch_pdl(fold_status_kernel, dim3(1), dim3(32), 0, st, dst, s);
  return launch_status();
}

bool layout_unchanged(const void* workspace, unsigned long long key) {
  struct Entry {
    const void* ws;
    unsigned long long key;
  };
  static std::mutex mu;
  static Entry memo[256] = {};
  const size_t i = (reinterpret_cast<uintptr_t>(workspace) >> 8) & 255;
  std::lock_guard<std::mutex> lock(mu);
  const bool same = memo[i].ws == workspace && memo[i].key == key;
  memo[i] = Entry{workspace, key};
  return same;
}

__global__ void clear_status_kernel(StatusSources s) {
  pdl_wait();
  if ((int)threadIdx.x < s.n) *s.p[threadIdx.x] = 0;
}

int clear_status(const StatusSources& s, cudaStream_t st) {
  launch_pdl(clear_status_kernel, dim3(1), dim3(32), 0, st, s);
  return launch_status();
}
}  // namespace sg

extern "C" int split_workspace_status(void* workspace, void* stream, int* out_status) {
  if (!workspace || !out_status) return SPLIT_ERR_INVALID;
  cudaStream_t st = as_stream(stream);
  int h = 0;
  SG_CUDA_TRY(cudaMemcpyAsync(&h, workspace, sizeof(int), cudaMemcpyDeviceToHost, st));
  SG_CUDA_TRY(cudaStreamSynchronize(st));
  SG_CUDA_TRY(cudaMemsetAsync(workspace, 0, sizeof(int), st));
  *out_status = h;
  return SPLIT_OK;
}
