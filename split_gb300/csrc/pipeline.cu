// The segmentation path as one plain launch sequence for one image: feature
// packing, k-means, connected components, small-segment merge decision,
// fused relabel + erosion, and Sobel normals of the luminance plane.
// Mirrors the stage order of samples/src/main.cu:154-314.
#include "geom.cuh"
#include "merge_state.cuh"

namespace sg {
namespace pipe {

// The sample's Lab + beta features (float4 per pixel) instead of RGB / 255.
constexpr int kFeaturesLabBeta = SPLIT_PIPELINE_FEATURES_LAB_BETA;

inline bool packs(const split_pipeline_params& p) {
  return p.features == SPLIT_LAYOUT_FLOAT4 || p.features == kFeaturesLabBeta;
}

struct Layout {
  WsHeader* hdr;
  void* pack_ws;   // maxima of the Lab + beta pass
  float* features4;
  int32_t* seg;
  int32_t* sizes;
  void* km_ws;
  size_t km_bytes;
  void* ccl_ws;
  size_t ccl_bytes;
  void* mrg_ws;
  size_t mrg_bytes;
  float* ic;   // intensity / chroma planes for the reference chroma merge rule
  size_t bytes;
};

static Layout carve(void* ws, int W, int H, const split_pipeline_params& p) {
  const int64_t n = (int64_t)W * H;
  Carver c(ws);
  Layout l;
  l.hdr = c.take<WsHeader>(1);
  l.pack_ws = p.features == kFeaturesLabBeta ? c.take<char>(512) : nullptr;
  l.features4 = packs(p) ? c.take<float>((size_t)n * 4) : nullptr;
  l.seg = c.take<int32_t>((size_t)n);
  l.sizes = c.take<int32_t>((size_t)n);
  l.km_bytes = split_kmeans_cluster_workspace_size_2d(n, W, p.nclusters, p.dim);
  l.km_ws = c.take<char>(l.km_bytes);
  l.ccl_bytes = split_ccl_workspace_size(W, H);
  l.ccl_ws = c.take<char>(l.ccl_bytes);
  l.mrg_bytes = p.merge_P > 0 ? split_merge_small_workspace_size(W, H) : 0;
  l.mrg_ws = p.merge_P > 0 ? c.take<char>(l.mrg_bytes) : nullptr;
  l.ic = p.merge_P > 0 && p.merge_policy == SPLIT_MERGE_REF_CHROMA
             ? c.take<float>((size_t)3 * n)
             : nullptr;
  l.bytes = c.size();
  return l;
}

static bool valid(const split_pipeline_params* p) {
  // K above 64 runs the many-cluster k-means (split_kmeans_cluster picks it)
  return p && p->nclusters >= 1 && p->nclusters <= (1 << 20) && (p->dim == 3 || p->dim == 5) &&
         p->kmeans_iters >= 0 &&
         (p->features == SPLIT_LAYOUT_FLOAT4 || p->features == SPLIT_LAYOUT_RGB8 ||
          p->features == kFeaturesLabBeta) &&
         (p->connectivity == 4 || p->connectivity == 8) &&
         (p->convention == SPLIT_LABEL_MIN_INDEX || p->convention == SPLIT_LABEL_MAX_INDEX) &&
         p->merge_P >= 0 &&
         (p->merge_policy == SPLIT_MERGE_MOST_BOUNDARY ||
          p->merge_policy == SPLIT_MERGE_REF_CHROMA) &&
         p->erode_radius >= 0 &&
         p->erode_radius <= 16;
}

}  // namespace pipe
}  // namespace sg

using namespace sg;

extern "C" size_t split_pipeline_workspace_size(int width, int height,
                                                const split_pipeline_params* params) {
  if (width < 1 || height < 1 || !pipe::valid(params)) return 0;
  return pipe::carve(nullptr, width, height, *params).bytes;
}

extern "C" int split_pipeline_run(const uint8_t* rgb, int width, int height,
                                  const split_pipeline_params* params, float* centroids,
                                  int32_t* cluster_labels, int32_t* segment_labels,
                                  float* normals, void* workspace, size_t workspace_bytes,
                                  void* const* stage_events, void* stream) {
  if (!rgb || !centroids || !cluster_labels || !segment_labels || width < 1 || height < 1 ||
      !pipe::valid(params))
    return SPLIT_ERR_INVALID;
  if ((int64_t)width * height * 3 > 0x7fffffffLL) return SPLIT_ERR_INVALID;
  const split_pipeline_params& p = *params;
  if (p.compute_normals && !normals) return SPLIT_ERR_INVALID;
  pipe::Layout l = pipe::carve(nullptr, width, height, p);
  if (!workspace || workspace_bytes < l.bytes || (reinterpret_cast<uintptr_t>(workspace) & 255))
    return SPLIT_ERR_WORKSPACE;
  l = pipe::carve(workspace, width, height, p);
  cudaStream_t st = as_stream(stream);
  const int64_t n = (int64_t)width * height;
  // the stages' own status words (sub-workspace headers), cleared first and
  // folded into the pipeline's status word at the end
  StatusSources ss{};
  ss.p[ss.n++] = &static_cast<WsHeader*>(l.km_ws)->status;
  ss.p[ss.n++] = &static_cast<WsHeader*>(l.ccl_ws)->status;
  if (l.mrg_ws) ss.p[ss.n++] = &static_cast<WsHeader*>(l.mrg_ws)->status;
  auto mark = [&](int i) -> int {
    if (stage_events)
      SG_CUDA_TRY(cudaEventRecord(reinterpret_cast<cudaEvent_t>(stage_events[i]), st));
    return SPLIT_OK;
  };
  // 0: features
  SG_TRY(mark(0));
  const unsigned long long layout_key =
      ((unsigned long long)(unsigned)width << 32 | (unsigned)height) ^
      ((unsigned long long)l.bytes << 7) ^ ((unsigned long long)p.features << 3) ^
      (unsigned long long)(p.merge_P > 0) ^ ((unsigned long long)p.merge_policy << 1);
  if (!layout_unchanged(workspace, layout_key)) SG_TRY(clear_status(ss, st));
  // byte / 255 features with the normals, from one read of the bytes (the
  // normals stage below is then empty)
  const bool fused = p.features == SPLIT_LAYOUT_FLOAT4 && p.compute_normals;
  if (fused)
    SG_TRY(normals_rgb8_geoms(rgb, single_geom(width, height), p.depth, normals, l.features4,
                              st));
  else if (p.features == SPLIT_LAYOUT_FLOAT4)
    SG_TRY(split_pack_rgb8(rgb, n, l.features4, nullptr, stream));
  else if (p.features == pipe::kFeaturesLabBeta)
    SG_TRY(split_pack_lab_beta(rgb, n, p.beta_mu, SPLIT_LAYOUT_FLOAT4, l.features4, nullptr,
                               l.pack_ws, 512, stream));
  SG_TRY(mark(1));
  // 1: k-means
  SG_TRY(mark(2));
  const void* pts = pipe::packs(p) ? static_cast<const void*>(l.features4)
                             : static_cast<const void*>(rgb);
  // byte / 255 features lie in the unit cube; Lab + beta ones do not
  const int layout = p.features == SPLIT_LAYOUT_FLOAT4
                         ? (SPLIT_LAYOUT_FLOAT4 | SPLIT_FEATURES_UNIT_RANGE)
                         : pipe::packs(p) ? SPLIT_LAYOUT_FLOAT4 : p.features;
  SG_TRY(split_kmeans_cluster(pts, layout, p.dim, n, width, p.xy_scale, centroids,
                              p.nclusters, cluster_labels, l.km_ws, l.km_bytes, p.kmeans_iters,
                              p.kmeans_threshold, nullptr, stream));
  SG_TRY(mark(3));
  // 2: connected components (+ component sizes for the merge)
  SG_TRY(mark(4));
  SG_TRY(split_ccl(cluster_labels, width, height, p.connectivity, p.convention, l.seg,
                   p.merge_P > 0 ? l.sizes : nullptr, l.ccl_ws, l.ccl_bytes, stream));
  SG_TRY(mark(5));
  // 3: merge decision (the relabel is fused into the erosion below)
  SG_TRY(mark(6));
  // the reference rule compares mean chroma: the sample's r / intensity
  // plane (row 1 of rgb_to_ic, main.cu:176-193)
  const float* chroma = l.ic ? l.ic + n : nullptr;
  if (l.ic) SG_TRY(split_rgb8_to_ic(rgb, n, l.ic, stream));
  if (p.merge_P > 0)
    SG_TRY(merge_decide_only(l.seg, width, height, p.merge_P, p.merge_policy, chroma, l.sizes,
                             l.mrg_ws, l.mrg_bytes, st));
  SG_TRY(mark(7));
  // 4: relabel + erosion
  SG_TRY(mark(8));
  if (p.erode_radius > 0) {
    if (p.merge_P > 0)
      SG_TRY(split_erode_mapped(l.seg, segment_labels, width, height, p.erode_radius, l.mrg_ws,
                                stream));
    else
      SG_TRY(split_erode(l.seg, segment_labels, width, height, p.erode_radius, stream));
  } else {
    SG_CUDA_TRY(cudaMemcpyAsync(segment_labels, l.seg, sizeof(int32_t) * (size_t)n,
                                cudaMemcpyDeviceToDevice, st));
    if (p.merge_P > 0)
      SG_TRY(split_merge_small(segment_labels, width, height, p.merge_P, p.merge_policy, chroma,
                               l.sizes, l.mrg_ws, l.mrg_bytes, stream));
  }
  SG_TRY(mark(9));
  // 5: normals of the luminance plane, straight from the bytes
  SG_TRY(mark(10));
  if (p.compute_normals && !fused)
    SG_TRY(split_sobel_normals_rgb8(rgb, width, height, p.depth, normals, stream));
  // errors the stages recorded in their own workspace headers, into the
  // pipeline's status word
  SG_TRY(fold_status(&l.hdr->status, ss, st));
  SG_TRY(mark(11));
  return SPLIT_OK;
}
