// Device-side record of the last small-segment merge, shared by the merge
// passes and by the fused relabel + erosion stencil.
#pragma once

#include "common.cuh"

namespace sg {
namespace mrg {

struct State {
  const int32_t* sizes;  // per-segment sizes used by the decision
  int P;
  int policy;
  int unsorted;          // REF_CHROMA: labels were not already sorted
  unsigned list_count;   // occupied table slots
  int cap_log2;
  int n;                 // pixels (segment ids lie in [0, n))
  int overflow;          // the pair pass found the table full (see split_round)
  unsigned dec_count;    // decided segments of the rounds (overflow path)
  int pad[6];
};

// Final label of a pixel whose pre-merge label is v.  Small segments take the
// end of their map chain (fin); with the reference rule, already-sorted labels
// are left unchanged (map_until_converged.cuh:25-30 compares against the
// sorted label copy and stops at once).
__device__ __forceinline__ int relabel(const State& st, const int32_t* fin, int v) {
  if (st.policy == SPLIT_MERGE_REF_CHROMA && !st.unsorted) return v;
  if (v < 0 || v >= st.n) return v;
  return __ldg(st.sizes + v) < st.P ? __ldg(fin + v) : v;
}

}  // namespace mrg

// Pointers into a merge workspace for the fused relabel + erosion.
struct MergeView {
  const mrg::State* state;
  const int32_t* fin;
};
int merge_view(const void* ws, int width, int height, MergeView* out);
int merge_view_n(const void* ws, int64_t n, MergeView* out);
struct Geoms;
// Merge decision over a geometry table (relabel left to the fused erosion).
int merge_geoms(const int32_t* labels, const Geoms& gs, int P, int policy, const int32_t* d_sizes,
                void* workspace, size_t workspace_bytes, cudaStream_t st);
size_t merge_workspace_bytes(int64_t n);
int merge_decide_only(const int32_t* labels, int width, int height, int P, int policy,
                      const float* chroma, const int32_t* d_sizes, void* workspace,
                      size_t workspace_bytes, cudaStream_t st);

}  // namespace sg
