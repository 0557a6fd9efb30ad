// Batches of uneven images through the segmentation path in one fixed launch
// sequence.  The plan lays the images out in pixel arenas (64-pixel aligned
// starts), uploads per-image descriptors and tensor maps once (bind), and
// then every run is a short, graph-capturable sequence of launches:
//   pack -> one cooperative k-means launch over every image's tiles ->
//   labelling over the tile grid of all images -> merge decision ->
//   fused relabel + erosion -> normals.
// Labels are arena-global linear indices until the erosion writes them back
// image-local, so no pass ever mixes pixels of two images.
#include <string.h>

#include <new>
#include <vector>

#include "geom.cuh"
#include "kmeans_batch.h"
#include "merge_state.cuh"

namespace sg {
int ccl_geoms(const int32_t* in, const Geoms& gs, int connectivity, int convention, int32_t* out,
              int32_t* sizes, WsHeader* hdr, cudaStream_t st);
size_t ccl_workspace_bytes(int tiles);
int erode_geoms(const int32_t* in, int32_t* out, const Geoms& gs, int radius, const void* mstate,
                const int32_t* mfin, int local_labels, cudaStream_t st);
int batch_image_maps(const int32_t* labels, const uint8_t* rgb, int W, int H, int radius,
                     CUtensorMap* lab_map, CUtensorMap* rgb_map);
int lab_beta_geoms(const uint8_t* rgb, const Geoms& gs, float mu, float* features4,
                   unsigned* maxima, cudaStream_t st);
// split_pipeline_params.features value of the sample's Lab + beta features
constexpr int kFeaturesLabBeta = SPLIT_PIPELINE_FEATURES_LAB_BETA;
// the batch packs float4 features (RGB / 255, or Lab + beta) before k-means
inline bool packs_float4(const split_pipeline_params& p) {
  return p.features == SPLIT_LAYOUT_FLOAT4 || p.features == kFeaturesLabBeta;
}
}  // namespace sg

using namespace sg;

struct split_batch {
  std::vector<split_batch_image> images;
  std::vector<int64_t> pix_off;
  std::vector<int64_t> cen_off;
  std::vector<int> tile_begin;
  split_pipeline_params params;
  int64_t arena_px = 0;
  int64_t cen_floats = 0;
  int total_tiles = 0;
  size_t km_bytes = 0, ccl_bytes = 0, mrg_bytes = 0;
  // bound state
  bool bound = false;
  const uint8_t* rgb = nullptr;
  float* centroids = nullptr;
  int32_t* cluster_labels = nullptr;
  int32_t* segment_labels = nullptr;
  float* normals = nullptr;
  void* ws = nullptr;
  KmBatchPlan km{};
};

namespace {

struct Layout {
  WsHeader* hdr;
  float* features4;
  unsigned* maxima;   // Lab + beta: L*max and |a*|max keys per image
  int32_t* seg;
  int32_t* sizes;
  void* km_ws;
  void* ccl_ws;
  void* mrg_ws;
  ImgGeom* geoms;
  CUtensorMap* lab_maps;
  CUtensorMap* rgb_maps;
  size_t bytes;
};

Layout carve(void* ws, const split_batch& b) {
  Carver c(ws);
  Layout l;
  const size_t n = (size_t)b.arena_px;
  const size_t ni = b.images.size();
  l.hdr = c.take<WsHeader>(1);
  l.features4 = packs_float4(b.params) ? c.take<float>(n * 4) : nullptr;
  l.maxima = b.params.features == kFeaturesLabBeta ? c.take<unsigned>(2 * ni) : nullptr;
  l.seg = c.take<int32_t>(n);
  l.sizes = c.take<int32_t>(n);
  l.km_ws = c.take<char>(b.km_bytes);
  l.ccl_ws = c.take<char>(b.ccl_bytes);
  l.mrg_ws = b.params.merge_P > 0 ? c.take<char>(b.mrg_bytes) : nullptr;
  l.geoms = c.take<ImgGeom>(ni);
  l.lab_maps = c.take<CUtensorMap>(ni);
  l.rgb_maps = c.take<CUtensorMap>(ni);
  l.bytes = c.size();
  return l;
}

std::vector<KmBatchImage> km_images(const split_batch& b, const Layout& l) {
  std::vector<KmBatchImage> v(b.images.size());
  for (size_t i = 0; i < b.images.size(); ++i) {
    const split_batch_image& im = b.images[i];
    KmBatchImage& k = v[i];
    k.points = packs_float4(b.params)
                   ? static_cast<const void*>(l.features4 ? l.features4 + 4 * b.pix_off[i] : nullptr)
                   : static_cast<const void*>(b.rgb ? b.rgb + 3 * b.pix_off[i] : nullptr);
    k.npoints = (int64_t)im.width * im.height;
    k.width = im.width;
    k.nclusters = im.nclusters;
    k.iters = im.kmeans_iters;
    k.threshold = b.params.kmeans_threshold;
    k.centroids = b.centroids ? b.centroids + b.cen_off[i] : nullptr;
    k.labels = b.cluster_labels ? b.cluster_labels + b.pix_off[i] : nullptr;
  }
  return v;
}

Geoms device_geoms(const split_batch& b, const Layout& l, const CUtensorMap* maps) {
  Geoms g{};
  g.table = l.geoms;
  g.maps = maps;
  g.n = (int)b.images.size();
  g.total_tiles = b.total_tiles;
  g.total_px = b.arena_px;
  if (g.n == 1) {
    // a one-image batch also goes through the table (n == 1 would use `one`)
    g.one.W = b.images[0].width;
    g.one.H = b.images[0].height;
    g.one.off = 0;
    g.one.tile_begin = 0;
    g.one.tiles_x = (b.images[0].width + kTileW - 1) / kTileW;
    g.one.tma_ok = 0;
  }
  return g;
}

}  // namespace

extern "C" int split_batch_create(const split_batch_image* images, int nimages,
                                  const split_pipeline_params* params, split_batch** out) {
  if (!images || nimages < 1 || !params || !out) return SPLIT_ERR_INVALID;
  const split_pipeline_params& p = *params;
  if ((p.dim != 3 && p.dim != 5) || (p.connectivity != 4 && p.connectivity != 8) ||
      (p.features != SPLIT_LAYOUT_FLOAT4 && p.features != SPLIT_LAYOUT_RGB8 &&
       p.features != kFeaturesLabBeta) ||
      p.erode_radius < 1 || p.erode_radius > 16 || p.merge_P < 0 ||
      p.merge_policy != SPLIT_MERGE_MOST_BOUNDARY)
    return SPLIT_ERR_INVALID;
  split_batch* b = new (std::nothrow) split_batch();
  if (!b) return SPLIT_ERR_INVALID;
  b->params = p;
  b->images.assign(images, images + nimages);
  int64_t off = 0, coff = 0;
  int tiles = 0;
  for (int i = 0; i < nimages; ++i) {
    const split_batch_image& im = images[i];
    if (im.width < 1 || im.height < 1 || im.nclusters < 1 || im.nclusters > 64 ||
        im.kmeans_iters < 0) {
      delete b;
      return SPLIT_ERR_INVALID;
    }
    b->pix_off.push_back(off);
    b->cen_off.push_back(coff);
    b->tile_begin.push_back(tiles);
    off += ((int64_t)im.width * im.height + 63) / 64 * 64;
    coff += (int64_t)p.dim * im.nclusters;
    tiles += tiles_of(im.width, im.height);
  }
  if (off > 0x7fffffffLL) {
    delete b;
    return SPLIT_ERR_INVALID;
  }
  b->arena_px = off;
  b->cen_floats = coff;
  b->total_tiles = tiles;
  std::vector<KmBatchImage> kmi = km_images(*b, Layout{});
  b->km_bytes = kmeans_batch_workspace(kmi.data(), nimages);
  b->ccl_bytes = ccl_workspace_bytes(tiles);
  b->mrg_bytes = p.merge_P > 0 ? merge_workspace_bytes(off) : 0;
  *out = b;
  return SPLIT_OK;
}

extern "C" void split_batch_destroy(split_batch* b) { delete b; }

extern "C" size_t split_batch_workspace_size(const split_batch* b) {
  return b ? carve(nullptr, *b).bytes : 0;
}
extern "C" int64_t split_batch_arena_pixels(const split_batch* b) { return b ? b->arena_px : 0; }
extern "C" int64_t split_batch_pixel_offset(const split_batch* b, int i) {
  return (b && i >= 0 && i < (int)b->images.size()) ? b->pix_off[i] : -1;
}
extern "C" int64_t split_batch_centroid_floats(const split_batch* b) {
  return b ? b->cen_floats : 0;
}
extern "C" int64_t split_batch_centroid_offset(const split_batch* b, int i) {
  return (b && i >= 0 && i < (int)b->images.size()) ? b->cen_off[i] : -1;
}

extern "C" int split_batch_bind(split_batch* b, const uint8_t* rgb, float* centroids,
                                int32_t* cluster_labels, int32_t* segment_labels, float* normals,
                                void* workspace, size_t workspace_bytes, void* stream) {
  if (!b || !rgb || !centroids || !cluster_labels || !segment_labels) return SPLIT_ERR_INVALID;
  if (b->params.compute_normals && !normals) return SPLIT_ERR_INVALID;
  Layout l = carve(nullptr, *b);
  if (!workspace || workspace_bytes < l.bytes || (reinterpret_cast<uintptr_t>(workspace) & 255))
    return SPLIT_ERR_WORKSPACE;
  l = carve(workspace, *b);
  cudaStream_t st = as_stream(stream);
  b->rgb = rgb;
  b->centroids = centroids;
  b->cluster_labels = cluster_labels;
  b->segment_labels = segment_labels;
  b->normals = normals;
  b->ws = workspace;
  std::vector<KmBatchImage> kmi = km_images(*b, l);
  // byte / 255 features lie in the unit cube; Lab + beta ones do not
  const int layout = b->params.features == SPLIT_LAYOUT_FLOAT4
                         ? (SPLIT_LAYOUT_FLOAT4 | SPLIT_FEATURES_UNIT_RANGE)
                         : b->params.features == kFeaturesLabBeta ? SPLIT_LAYOUT_FLOAT4
                                                                  : SPLIT_LAYOUT_RGB8;
  SG_TRY(kmeans_batch_prepare(kmi.data(), (int)kmi.size(), layout, b->params.dim,
                              b->params.xy_scale, l.km_ws, b->km_bytes, st, &b->km));
  const size_t ni = b->images.size();
  std::vector<ImgGeom> geoms(ni);
  std::vector<CUtensorMap> lab_maps(ni), rgb_maps(ni);
  for (size_t i = 0; i < ni; ++i) {
    const split_batch_image& im = b->images[i];
    ImgGeom& g = geoms[i];
    g.W = im.width;
    g.H = im.height;
    g.off = b->pix_off[i];
    g.tile_begin = b->tile_begin[i];
    g.tiles_x = (im.width + kTileW - 1) / kTileW;
    g.tma_ok = batch_image_maps(l.seg + g.off, rgb + 3 * g.off, im.width, im.height,
                                b->params.erode_radius, &lab_maps[i], &rgb_maps[i]);
  }
  SG_CUDA_TRY(cudaMemcpyAsync(l.geoms, geoms.data(), sizeof(ImgGeom) * ni,
                              cudaMemcpyHostToDevice, st));
  SG_CUDA_TRY(cudaMemcpyAsync(l.lab_maps, lab_maps.data(), sizeof(CUtensorMap) * ni,
                              cudaMemcpyHostToDevice, st));
  SG_CUDA_TRY(cudaMemcpyAsync(l.rgb_maps, rgb_maps.data(), sizeof(CUtensorMap) * ni,
                              cudaMemcpyHostToDevice, st));
  // a rebound arena may hold anything where this layout's stage headers lie
  {
    StatusSources ss{};
    ss.p[ss.n++] = &static_cast<WsHeader*>(l.km_ws)->status;
    ss.p[ss.n++] = &static_cast<WsHeader*>(l.ccl_ws)->status;
    if (l.mrg_ws) ss.p[ss.n++] = &static_cast<WsHeader*>(l.mrg_ws)->status;
    SG_TRY(clear_status(ss, st));
  }
  SG_CUDA_TRY(cudaStreamSynchronize(st));
  b->bound = true;
  return SPLIT_OK;
}

extern "C" int split_batch_run(split_batch* b, void* stream) {
  return split_batch_run_events(b, nullptr, stream);
}

extern "C" int split_batch_run_events(split_batch* b, void* const* stage_events, void* stream) {
  if (!b || !b->bound) return SPLIT_ERR_INVALID;
  const split_pipeline_params& p = b->params;
  Layout l = carve(b->ws, *b);
  cudaStream_t st = as_stream(stream);
  auto mark = [&](int i) -> int {
    if (stage_events)
      SG_CUDA_TRY(cudaEventRecord(reinterpret_cast<cudaEvent_t>(stage_events[i]), st));
    return SPLIT_OK;
  };
  // the stages' own status words (sub-workspace headers, cleared at bind),
  // folded into the batch's at the end
  StatusSources ss{};
  ss.p[ss.n++] = &static_cast<WsHeader*>(l.km_ws)->status;
  ss.p[ss.n++] = &static_cast<WsHeader*>(l.ccl_ws)->status;
  if (l.mrg_ws) ss.p[ss.n++] = &static_cast<WsHeader*>(l.mrg_ws)->status;
  // 0: byte / 255 features with the normals, from one read of the bytes
  SG_TRY(mark(0));
  const bool fused = p.features == SPLIT_LAYOUT_FLOAT4 && p.compute_normals;
  if (fused)
    SG_TRY(normals_rgb8_geoms(b->rgb, device_geoms(*b, l, l.rgb_maps), p.depth, b->normals,
                              l.features4, st));
  else if (p.features == SPLIT_LAYOUT_FLOAT4)
    SG_TRY(split_pack_rgb8(b->rgb, b->arena_px, l.features4, nullptr, stream));
  else if (p.features == kFeaturesLabBeta)
    SG_TRY(lab_beta_geoms(b->rgb, device_geoms(*b, l, nullptr), p.beta_mu, l.features4, l.maxima,
                          st));
  SG_TRY(mark(1));
  // 1: k-means over every image
  SG_TRY(mark(2));
  SG_TRY(kmeans_batch_run(b->km, l.km_ws, st));
  SG_TRY(mark(3));
  // 2: connected components
  SG_TRY(mark(4));
  const Geoms gs = device_geoms(*b, l, nullptr);
  SG_TRY(ccl_geoms(b->cluster_labels, gs, p.connectivity, SPLIT_LABEL_MIN_INDEX, l.seg,
                   p.merge_P > 0 ? l.sizes : nullptr, reinterpret_cast<WsHeader*>(l.ccl_ws), st));
  SG_TRY(mark(5));
  // 3: merge decision
  SG_TRY(mark(6));
  const void* mstate = nullptr;
  const int32_t* mfin = nullptr;
  if (p.merge_P > 0) {
    SG_TRY(merge_geoms(l.seg, gs, p.merge_P, p.merge_policy, l.sizes, l.mrg_ws, b->mrg_bytes, st));
    MergeView mv;
    SG_TRY(merge_view_n(l.mrg_ws, b->arena_px, &mv));
    mstate = mv.state;
    mfin = mv.fin;
  }
  SG_TRY(mark(7));
  // 4: relabel + erosion
  SG_TRY(mark(8));
  SG_TRY(erode_geoms(l.seg, b->segment_labels, device_geoms(*b, l, l.lab_maps), p.erode_radius,
                     mstate, mfin, 1, st));
  SG_TRY(mark(9));
  // 5: normals (empty when the features pass wrote them)
  SG_TRY(mark(10));
  if (p.compute_normals && !fused)
    SG_TRY(normals_rgb8_geoms(b->rgb, device_geoms(*b, l, l.rgb_maps), p.depth, b->normals,
                              nullptr, st));
  // errors the stages recorded in their own workspace headers, into the
  // batch's status word
  SG_TRY(fold_status(&l.hdr->status, ss, st));
  return mark(11);
}
