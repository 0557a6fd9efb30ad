/*
 * split_gb300.h - C ABI of the GB300-native segmentation hot path.
 *
 * Drop-in boundary for nitronoid/split's device entry points (k-means,
 * connected components, label compression, small-segment merge, erosion,
 * Sobel normals).  Every entry point:
 *   - takes plain device pointers, sizes and a cudaStream_t (passed as void*);
 *   - allocates nothing: all scratch comes from a caller-provided workspace
 *     sized by the matching *_workspace_size query;
 *   - is asynchronous on `stream` and never synchronises the host;
 *   - returns a split_status for argument/launch errors.  Errors that only
 *     the device can detect (a capacity overflow, an iteration cap) are
 *     recorded in the workspace's status word and read back with
 *     split_workspace_status();
 *   - never throws, exits or spins without a bound.
 *
 * Layouts follow the reference (split/include/split/detail/internal.h:35-39,
 * samples/src/main.cu:164-168): planar float features dim x n (row d holds
 * dimension d of every pixel), row-major int32 label images, planar 3 x n
 * float normals.  The packed layouts (RGB8 interleaved, float4 per pixel) are
 * native extensions.
 *
 * A workspace must be zero-filled once before its first use (cudaMemset);
 * every call leaves it ready for the next call.  Calls that share a
 * workspace must be ordered on one stream.
 */
#ifndef SPLIT_GB300_H
#define SPLIT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
typedef enum split_status {
  SPLIT_OK = 0,
  SPLIT_ERR_INVALID = 1,       /* bad argument (null pointer, size, flag)   */
  SPLIT_ERR_WORKSPACE = 2,     /* workspace too small or misaligned         */
  SPLIT_ERR_NOT_CONVERGED = 3, /* a device loop reached its iteration cap   */
  SPLIT_ERR_CUDA = 4,          /* a CUDA runtime call or launch failed      */
  SPLIT_ERR_OVERFLOW = 5,      /* a device table ran out of capacity        */
  SPLIT_ERR_TIMEOUT = 6,       /* a device-wide barrier wait hit its limit  */
  SPLIT_ERR_UNSUPPORTED = 7    /* no GB300-class device / kernel image      */
} split_status;

/* ---- feature layouts --------------------------------------------------- */
enum {
  SPLIT_LAYOUT_PLANAR = 0, /* float, dim x n, row d = dimension d            */
  SPLIT_LAYOUT_FLOAT4 = 1, /* float4 per pixel (r, g, b, unused)             */
  SPLIT_LAYOUT_RGB8 = 2    /* uint8 r, g, b interleaved; value = byte / 255  */
};
/* For FLOAT4 and RGB8 layouts, dim is 3 (colour) or 5 (colour plus
 * xy_scale * column and xy_scale * row, synthesised from the pixel index). */
/* Flag or-ed into a FLOAT4 layout: the caller guarantees every colour feature
 * lies in [0, 1] (true of split_pack_rgb8 output; always true of RGB8).  The
 * assignment then bounds colour distances by the unit cube instead of
 * measuring each batch.  Features outside [0, 1] under this flag may be
 * mislabelled. */
#define SPLIT_FEATURES_UNIT_RANGE 0x100
/* Flag or-ed into the layout of split_kmeans_cluster: measure the centroid
 * shift of the convergence test the way the reference's cluster() does
 * (cluster.cu:40-50, :73-87).  It keeps the previous centroids in workspace
 * words that label_points and calculate_centroids overwrite within the same
 * iteration (label.cu:80-88, centroids.cu:40-63), so its "shift" compares the
 * new centroids with 1 / (cluster sizes) and with the distances of two or
 * three pixels near index 2N / K to the iteration's input centroids.  With
 * this flag a threshold >= 0 stops at the reference's iteration (3-D
 * features, K >= 3 only; anything else is SPLIT_ERR_INVALID).  Without it the
 * shift is the L2 change of the centroid matrix, as cluster.cu's comments
 * describe. */
#define SPLIT_KMEANS_REFERENCE_SHIFT 0x200

/* ---- label conventions / policies -------------------------------------- */
enum {
  SPLIT_LABEL_MIN_INDEX = 0, /* component label = its minimum linear index  */
  SPLIT_LABEL_MAX_INDEX = 1  /* component label = its maximum linear index,
                                the reference's fixed point                  */
};
enum {
  SPLIT_MERGE_MOST_BOUNDARY = 0, /* join the neighbour sharing most edges   */
  SPLIT_MERGE_REF_CHROMA = 1     /* the reference's nearest-chroma rule      */
};

const char* split_version(void);
const char* split_status_string(int status);

/* Reads (and clears) the device-side status word of a workspace after the
 * work queued on `stream` completes.  Synchronises `stream`. */
int split_workspace_status(void* workspace, void* stream, int* out_status);


/* ======================================================================== */
/* k-means                                                                  */
/* ======================================================================== */

/* Replaces split::device::kmeans::cluster_workspace
 * (split/include/split/device/kmeans/cluster.cuh:46-47).  The workspace holds
 * the clustering state (about 21 KB) and, for images at least 64 pixels wide,
 * the exact feature sums of 64-column spans kept from the first iteration
 * (64 bytes per span, about 0.5 byte per pixel), which let later iterations
 * skip the pixels of spans with a single candidate cluster.  Without the
 * width the bound covers any width.  A smaller workspace (at least the state)
 * is accepted: the call then reads every pixel in every iteration, with the
 * same results. */
size_t split_kmeans_cluster_workspace_size(int64_t npoints, int nclusters,
                                           int dim);
/* The same for a known image width (what the call's `width` will be). */
size_t split_kmeans_cluster_workspace_size_2d(int64_t npoints, int width,
                                              int nclusters, int dim);

/* Replaces split::device::kmeans::cluster (cluster.cuh:31-37,
 * split/src/split/device/kmeans/cluster.cu:27-93).
 * points: layout-dependent, see above; width: image width (pixels per row,
 * used for the synthesised xy features; any value >= 1 otherwise).
 * centroids: dim x nclusters planar, in/out.  labels: int32[npoints] out.
 * Runs until max_iter iterations, or until |delta - old_delta| <= threshold
 * where delta is the L2 shift of the centroid matrix (threshold < 0: exactly
 * max_iter iterations).  The convergence test runs on the device; the number
 * of iterations performed is written to *d_iterations (device int) if not
 * null.  The returned labels are the assignment computed from the centroids
 * of the final iteration's input, the returned centroids the update computed
 * from those labels, as in the reference.  nclusters: 1 to 64 in one
 * persistent launch; 65 to 2^20 (the reference sets no limit) in the
 * many-cluster path, which queues one assignment and one forming launch per
 * iteration (max_iter pairs; those after the device-side stop return at
 * once) and needs the workspace size for that K. */
int split_kmeans_cluster(const void* points, int layout, int dim,
                         int64_t npoints, int width, float xy_scale,
                         float* centroids, int nclusters, int32_t* labels,
                         void* workspace, size_t workspace_bytes, int max_iter,
                         float threshold, int32_t* d_iterations, void* stream);

/* Allocation-free variant of split_kmeans_cluster (same arguments and
 * results, no workspace).  It has no counterpart in the reference.  It is for
 * callers that cannot allocate device memory where they cluster: a
 * latency-critical serving loop (cudaMalloc / cudaFree synchronise the
 * device) and host plugins whose device memory belongs to a pool they may
 * not touch.  Its scratch is one fixed-size device array in the library
 * (20736 bytes), held by every GPU that loads the library until the process
 * exits.
 *   - Limit: the array holds one image's clustering state for up to 64
 *     clusters of 3 or 5 dimensions, whatever the image size.  Larger K (or
 *     another D) returns SPLIT_ERR_INVALID before any work is queued.
 *   - The first call on each device looks up the array's device address
 *     (cudaGetSymbolAddress) with that device current; make that first call
 *     before any stream capture.  A cudaDeviceReset may move the array:
 *     after resetting a device, do not call this entry point on it again.
 *   - All calls share the array and overwrite it: calls whose work overlaps
 *     on the GPU race.  Order them on one stream.
 *   - d_status (device int, optional) receives the device-side status word
 *     (0, or e.g. SPLIT_ERR_TIMEOUT) when the work completes. */
int split_kmeans_cluster_noalloc(const void* points, int layout, int dim,
                                 int64_t npoints, int width, float xy_scale,
                                 float* centroids, int nclusters,
                                 int32_t* labels, int max_iter,
                                 float threshold, int32_t* d_iterations,
                                 int32_t* d_status, void* stream);

/* Test setting of the bounded waits (no counterpart in the reference, which
 * has no device-wide waits).  Process-wide; applies to the single-image
 * k-means launches queued after the call (not to batches).  A device-wide
 * barrier of those launches gives up after spin_limit polls (0: the default,
 * about a second), and block skip_block (>= 0; -1: none) leaves at its first
 * barrier without arriving, so that the other blocks' wait runs out: the call
 * then reports SPLIT_ERR_TIMEOUT through split_workspace_status, and every
 * block returns (nothing waits without a limit).  (0, -1) restores normal
 * operation. */
void split_kmeans_set_wait_test(unsigned spin_limit, int skip_block);

/* Replaces split::device::kmeans::label_points_workspace (label.cuh:39-40). */
size_t split_kmeans_assign_workspace_size(int64_t npoints, int nclusters);

/* Replaces split::device::kmeans::label_points (label.cuh:27-31,
 * label.cu:74-106): nearest centroid, squared distance accumulated in
 * dimension order, ties to the lowest cluster index.  nclusters 1 to 2^20
 * (above 64 through the many-cluster path). */
int split_kmeans_assign(const void* points, int layout, int dim,
                        int64_t npoints, int width, float xy_scale,
                        const float* centroids, int nclusters, int32_t* labels,
                        void* workspace, size_t workspace_bytes, void* stream);

/* Replaces split::device::kmeans::calculate_centroids_workspace
 * (centroids.cuh:39-40). */
size_t split_kmeans_update_workspace_size(int64_t npoints, int nclusters,
                                          int dim);

/* Replaces split::device::kmeans::calculate_centroids (centroids.cuh:26-30,
 * centroids.cu:22-101): per-cluster mean of the member points, accumulated
 * in FP32 in a fixed order (bit-reproducible).  A cluster with no members
 * keeps its previous centroid (the reference shifts later slots instead).
 * labels outside [0, nclusters) are ignored. */
int split_kmeans_update(const int32_t* labels, const void* points, int layout,
                        int dim, int64_t npoints, int width, float xy_scale,
                        float* centroids, int nclusters, void* workspace,
                        size_t workspace_bytes, void* stream);

/* Replaces split::device::kmeans::propagate_centroids (propagation.cuh:23-26,
 * propagation.cu:9-24): out[d * npoints + i] = centroids[d * nclusters +
 * labels[i]] for d < dim (planar output). */
int split_kmeans_propagate(const int32_t* labels, int64_t npoints,
                           const float* centroids, int nclusters, int dim,
                           float* out, void* stream);

/* ======================================================================== */
/* connected components / label compression                                 */
/* ======================================================================== */

/* Replaces the temp-size contract of split::device::ccl::connected_components
 * (connected_components.cuh:25-29), which allocates internally
 * (connected_components.cu:93-94, 140-142). */
size_t split_ccl_workspace_size(int width, int height);

/* Replaces split::device::ccl::connected_components (connected_components.cuh:
 * 25-29, connected_components.cu:80-181).  labels_in: row-major int32 image
 * (any values; equality defines the regions); labels_out: int32[w*h].
 * connectivity: 4 (reference) or 8.  convention: SPLIT_LABEL_MIN_INDEX or
 * SPLIT_LABEL_MAX_INDEX (the reference's converged labels).
 * d_sizes: optional int32[w*h]; if not null, d_sizes[root] receives the pixel
 * count of the component labelled `root` (entries at non-label indices are
 * left unspecified).  Always converges (union-find); the reference's
 * i_max_iterations cap has no counterpart. */
int split_ccl(const int32_t* labels_in, int width, int height,
              int connectivity, int convention, int32_t* labels_out,
              int32_t* d_sizes, void* workspace, size_t workspace_bytes,
              void* stream);

/* Replaces split::device::ccl::compress_labels (compress_labels.cuh:21-23,
 * compress_labels.cu:10-35): labels (in place) become their rank among the
 * distinct values.  Values must lie in [-1, n).  The number of distinct
 * labels is written to *d_count (device int). */
size_t split_compress_labels_workspace_size(int64_t n);
int split_compress_labels(int32_t* labels, int64_t n, int32_t* d_count,
                          void* workspace, size_t workspace_bytes,
                          void* stream);

/* Replaces split::device::ccl::segment_adjacency_edges
 * (segment_adjacency.cuh:14-16, segment_adjacency.cu:170-254): for every
 * pixel i in index order and every in-image neighbour j in the order NW, N,
 * NE, W, E, SW, S, SE whose label differs, one edge (i, j).  The m sources
 * are written to edges[0, m) and the targets to edges[m, 2m); `edges` must
 * hold 16 * width * height ints (as the reference's).  m is written to
 * *d_count (device int).  width * height must be below 2^27. */
size_t split_segment_adjacency_edges_workspace_size(int width, int height);
int split_segment_adjacency_edges(const int32_t* labels, int width, int height,
                                  int32_t* edges, int32_t* d_count, void* workspace,
                                  size_t workspace_bytes, void* stream);

/* Replaces split::device::ccl::segment_adjacency (segment_adjacency.cuh:
 * 21-24, segment_adjacency.cu:256-289): the distinct (label, neighbouring
 * label) pairs of those edges, sorted by key then by value, into keys[k] /
 * adjacency[k] (each must hold 8 * width * height ints, as the reference's
 * edge-count bound); their number is written to *d_count (device int).  Any
 * int labels.  The workspace holds two sort buffers of 8 * width * height
 * 64-bit keys. */
size_t split_segment_adjacency_workspace_size(int width, int height);
int split_segment_adjacency(const int32_t* labels, int width, int height, int32_t* keys,
                            int32_t* adjacency, int32_t* d_count, void* workspace,
                            size_t workspace_bytes, void* stream);

/* ======================================================================== */
/* small-segment merge                                                      */
/* ======================================================================== */

/* Replaces split::device::ccl::merge_small_segments_workspace
 * (merge_small_segments.cuh:21-22). */
size_t split_merge_small_workspace_size(int width, int height);

/* Replaces split::device::ccl::merge_small_segments (merge_small_segments.cuh:
 * 15-19, merge_small_segments.cu:92-196).  labels (in/out): segment ids in
 * [0, w*h).  Segments smaller than P join one 8-adjacent neighbour chosen by
 * `policy` (SPLIT_MERGE_MOST_BOUNDARY: most shared 8-neighbour edges, ties to
 * the lowest id; SPLIT_MERGE_REF_CHROMA: the reference's nearest mean-chroma
 * rule, chroma = planar 2 x n float, only row 0 read as in the reference).
 * Mutual pairs keep the larger id; chains resolve to their end.  Output ids
 * are input ids (not compressed).  d_sizes: optional per-segment pixel counts
 * indexed by segment id (as produced by split_ccl); null = computed here. */
int split_merge_small(int32_t* labels, int width, int height, int P,
                      int policy, const float* chroma, const int32_t* d_sizes,
                      void* workspace, size_t workspace_bytes, void* stream);

/* Replaces split::device::ccl::merge_smooth_boundaries_workspace
 * (merge_smooth_boundaries.cuh:29-31). */
size_t split_merge_smooth_workspace_size(int width, int height);

/* Replaces split::device::ccl::merge_smooth_boundaries
 * (merge_smooth_boundaries.cuh:20-25, merge_smooth_boundaries.cu:134-243).
 * labels (in/out): segment ids in [0, w*h).  points: planar float features,
 * at least 3 rows of w*h (rows 0..2 are read).  Every segment joins the
 * 8-adjacent segment with the smallest mean |x_p - x_q| over their directed
 * boundary edges (ties to the lowest id), among pairs with more than 15
 * edges and mean below threshold * max_i |x_i|.  Mutual pairs keep the
 * larger id; chains resolve to their end.  The reference file does not
 * compile as written (its reduce_by_key takes a predicate as the
 * reduction); this follows its documented intent.  The segment count the
 * reference takes is not needed. */
int split_merge_smooth(int32_t* labels, int width, int height, const float* points,
                       float threshold, void* workspace, size_t workspace_bytes,
                       void* stream);

/* ======================================================================== */
/* erosion / normals / feature preparation                                  */
/* ======================================================================== */

/* Replaces split::device::morph::erode (erode.cuh:16-18, erode.cu:139-159):
 * square (2r+1)^2 erosion of every label's mask, image border = background,
 * eroded pixels = -1.  in and out must not overlap; r in [1, 16]. */
int split_erode(const int32_t* labels_in, int32_t* labels_out, int width,
                int height, int radius, void* stream);

/* Erosion of merged labels: out = erode(map[labels_in]) where map is the
 * segment map left in `merge_workspace` by the last split_merge_small call on
 * the same labels (fused relabel + erosion; labels_in is then the pre-merge
 * image). */
int split_erode_mapped(const int32_t* labels_in, int32_t* labels_out,
                       int width, int height, int radius,
                       const void* merge_workspace, void* stream);

/* Replaces split::device::sfs::sobel_normals (sobel_normals.cuh:17-20,
 * sobel_normals.cu:86-119): heights row-major float[h*w] -> planar 3 x n
 * float normals, n = normalize(Gx, Gy, 1 / max(0.001, depth)), z >= 0. */
int split_sobel_normals(const float* heights, int width, int height,
                        float depth, float* normals, void* stream);

/* Replaces split::device::sfs::estimate_normals (estimate_normals.cuh:14-18,
 * estimate_normals.cu:251-308): normals (planar 3 x n) of a shading image
 * lit from (lx, ly, lz), solving (L L^T (x) I + 2 smoothness * B (x) I3) x =
 * intensity * L (B: the grid's 5-point Poisson matrix with the reference's
 * border valence) from x = (0, 0, 1) by red-black block relaxation until
 * |b - A x| <= tol |b| or max_iter sweeps (the reference: 1e-5, 1500), then
 * normalised with z >= 0.  smoothness > 0.  *d_iterations (device int,
 * optional) receives the sweeps performed.  The reference's cuSPARSE
 * assembly no longer builds with CUDA 12; the system is applied matrix-free
 * here. */
size_t split_estimate_normals_workspace_size(int width, int height);
int split_estimate_normals(const float* intensity, int width, int height, float lx,
                           float ly, float lz, float smoothness, int max_iter,
                           float tol, float* normals, int32_t* d_iterations,
                           void* workspace, size_t workspace_bytes, void* stream);

/* Normals from an RGB8 image: heights = luminance L* / 100 (fused, the
 * luminance plane is never written). */
int split_sobel_normals_rgb8(const uint8_t* rgb, int width, int height,
                             float depth, float* normals, void* stream);

/* Feature preparation (samples/src/main.cu:164-223): RGB8 interleaved ->
 * float4 (r, g, b, 0) / 255 (optional) and luminance L* / 100 of the
 * channels clamped to >= 1/255 (optional, split/include/split/device/color/
 * detail/conversion.inl:8-64). */
int split_pack_rgb8(const uint8_t* rgb, int64_t npixels, float* features4,
                    float* luminance, void* stream);

/* The sample's intensity and chroma planes (samples/src/main.cu:169-179;
 * replaces color::convert_color_space(rgb, ic, rgb_to_ic<>()),
 * split/include/split/device/color/conversion.cuh:58 and
 * detail/conversion.inl:99-108): RGB8 -> channels byte / 255 clamped to
 * >= 1/255 -> ic planar 3 x n: intensity (r + g + b) / 3, then r / intensity
 * and g / intensity (the chroma rows the reference's merge_small_segments
 * reads).  FP32 in the reference's order of operations. */
int split_rgb8_to_ic(const uint8_t* rgb, int64_t npixels, float* ic, void* stream);

/* The sample's k-means features (samples/src/main.cu:169-173, :215-225;
 * replaces color::convert_color_space(rgb_to_lab) followed by
 * color::beta_feature, beta_feature.cuh:12-15): RGB8 -> channels clamped to
 * >= 1/255 -> L*a*b* (conversion.inl:8-64) -> (beta, a*, b*) with beta = -mu
 * for achromatic pixels (|a*|, |b*| < 0.2 max |a*|) darker than 0.2 L*max,
 * +mu for achromatic pixels brighter than 0.95 L*max, 0 otherwise
 * (beta_feature.cu:26-78).  layout: SPLIT_LAYOUT_FLOAT4 ((beta, a*, b*, 0)
 * per pixel, 16-byte aligned) or SPLIT_LAYOUT_PLANAR (3 x n).  luminance:
 * optional n floats of L*.  Two passes over the RGB8 input. */
size_t split_pack_lab_beta_workspace_size(int64_t npixels);
int split_pack_lab_beta(const uint8_t* rgb, int64_t npixels, float mu, int layout,
                        float* features, float* luminance, void* workspace,
                        size_t workspace_bytes, void* stream);

/* ======================================================================== */
/* pipeline                                                                  */
/* ======================================================================== */

/* The sample's segmentation path as one call (samples/src/main.cu:154-314:
 * features -> kmeans::cluster -> ccl::connected_components -> small-segment
 * merge -> morph::erode) plus Sobel normals of the luminance plane. */
typedef struct split_pipeline_params {
  int nclusters;          /* 1 to 2^20 (above 64: the many-cluster k-means) */
  int dim;                /* 3 (RGB) or 5 (RGB + xy_scale * (column, row))   */
  float xy_scale;
  int kmeans_iters;
  float kmeans_threshold; /* < 0: exactly kmeans_iters iterations            */
  int features;           /* SPLIT_LAYOUT_FLOAT4: pack float4 features first;
                             SPLIT_LAYOUT_RGB8: read the bytes directly;
                             SPLIT_PIPELINE_FEATURES_LAB_BETA: the sample's
                             (beta, a*, b*) features (split_pack_lab_beta;
                             in a batch with per-image maxima)             */
  int connectivity;       /* 4 or 8                                          */
  int convention;         /* SPLIT_LABEL_MIN_INDEX / SPLIT_LABEL_MAX_INDEX   */
  int merge_P;            /* merge segments smaller than P; 0 = no merge     */
  int merge_policy;       /* SPLIT_MERGE_MOST_BOUNDARY, or SPLIT_MERGE_REF_CHROMA
                             on the sample's r / intensity plane
                             (split_rgb8_to_ic, computed in the pipeline;
                             single images only, not batches)              */
  int erode_radius;       /* 0 = no erosion                                  */
  int compute_normals;    /* nonzero: normals of L* / 100                    */
  float depth;
  float beta_mu;          /* mu of the beta feature (the reference: 1e5)     */
} split_pipeline_params;

/* Errors recorded on the device by any stage of split_pipeline_run or
 * split_batch_run are reported through the status word of the call's own
 * workspace (split_workspace_status), each once. */

/* split_pipeline_params.features value for the sample's Lab + beta features. */
#define SPLIT_PIPELINE_FEATURES_LAB_BETA 3

enum { SPLIT_PIPELINE_STAGES = 6 }; /* pack, kmeans, ccl, merge, erode, normals */

size_t split_pipeline_workspace_size(int width, int height,
                                     const split_pipeline_params* params);

/* rgb: device RGB8 interleaved image.  centroids: dim x K planar, in/out
 * (initial centroids in).  cluster_labels, segment_labels: int32[w*h] out
 * (segment_labels = merged, eroded labels; -1 = eroded).  normals: planar
 * 3 x w*h float out (may be null when compute_normals == 0).
 * stage_events: null, or 2 * SPLIT_PIPELINE_STAGES cudaEvent_t recorded
 * before/after each stage (a skipped stage records both back to back).  With
 * SPLIT_LAYOUT_FLOAT4 features and compute_normals set, one pass over the
 * bytes writes both the features and the normals: the first stage times it
 * and the normals stage is empty. */
int split_pipeline_run(const uint8_t* rgb, int width, int height,
                       const split_pipeline_params* params, float* centroids,
                       int32_t* cluster_labels, int32_t* segment_labels,
                       float* normals, void* workspace, size_t workspace_bytes,
                       void* const* stage_events, void* stream);

/* ======================================================================== */
/* batches                                                                   */
/* ======================================================================== */

/* Many images of uneven size and per-image K / iteration count through the
 * segmentation path in one fixed launch sequence (about 12 launches whatever
 * the image count; the k-means stage is one cooperative launch over every
 * image's tiles).  Each image's results are identical to running it alone. */
typedef struct split_batch_image {
  int width, height;
  int nclusters;    /* K <= 64 */
  int kmeans_iters;
} split_batch_image;

typedef struct split_batch split_batch; /* opaque host-side plan */

/* params: as for split_pipeline_run; nclusters and kmeans_iters come from the
 * images instead; erode_radius must be >= 1. */
int split_batch_create(const split_batch_image* images, int nimages,
                       const split_pipeline_params* params, split_batch** out);
void split_batch_destroy(split_batch* batch);
size_t split_batch_workspace_size(const split_batch* batch);
/* Arena layout: image i's pixels start at pixel_offset(i) (a multiple of 64);
 * the RGB8 arena holds 3 bytes, the label arenas one int32 and the normals
 * arena 3 planes of floats (image i's planes start at 3 * pixel_offset(i))
 * per arena pixel.  Centroids: image i's dim x K planar block starts at
 * centroid_offset(i) (in floats). */
int64_t split_batch_arena_pixels(const split_batch* batch);
int64_t split_batch_pixel_offset(const split_batch* batch, int image);
int64_t split_batch_centroid_floats(const split_batch* batch);
int64_t split_batch_centroid_offset(const split_batch* batch, int image);
/* Binds device buffers and a zero-filled workspace: uploads the image
 * descriptors and tensor maps (synchronises `stream`; not capturable). */
int split_batch_bind(split_batch* batch, const uint8_t* rgb, float* centroids,
                     int32_t* cluster_labels, int32_t* segment_labels,
                     float* normals, void* workspace, size_t workspace_bytes,
                     void* stream);
/* Runs the bound batch: kernel launches and memsets only, so the call can be
 * captured into a CUDA graph.  `centroids` must hold the initial centroids;
 * segment labels come out image-local (minimum linear index within the
 * image, -1 = eroded). */
int split_batch_run(split_batch* batch, void* stream);
/* split_batch_run with per-stage timing: stage_events is null, or
 * 2 * SPLIT_PIPELINE_STAGES cudaEvent_t recorded on `stream` around the
 * batch's stages in the order of split_pipeline_run's (features, k-means,
 * labelling, merge decision, relabel + erosion, normals). */
int split_batch_run_events(split_batch* batch, void* const* stage_events,
                           void* stream);

/* Kernels launched by this library since it was loaded (all entry points). */
unsigned long long split_launch_count(void);

/* ======================================================================== */
/* serving (no counterpart in the reference, whose only caller segments one  */
/* image per run: samples/src/main.cu:154-372)                               */
/* ======================================================================== */

/* A continuous-batching server on one GPU.  Requests are admitted in arrival
 * order while their device footprint fits the HBM budget, packed into
 * batches (split_batch_*) while fewer than max_inflight batches are on the
 * device, and run with uploads, compute and downloads on three streams.  A
 * worker thread owned by the server does all of this; submit and poll may be
 * called from any thread.  Every request's results equal the same request
 * served alone (and the single-image pipeline's). */
typedef struct split_server split_server; /* opaque */

typedef struct split_server_config {
  split_pipeline_params params; /* as for split_batch_create (per-request K
                                   and iteration count replace nclusters and
                                   kmeans_iters) */
  size_t hbm_budget_bytes;      /* admission budget; 0: 40 GiB */
  int64_t max_batch_pixels;     /* pixel cap of a batch; 0: 64 Mi pixels (a
                                   larger image still forms a batch alone) */
  int max_inflight;             /* batches on the device at once; 0: 2 (<= 8) */
  int device;                   /* CUDA device ordinal */
} split_server_config;

/* One request.  All pointers are host memory that must stay valid until the
 * request's completion has been returned by split_server_poll; page-locked
 * buffers (cudaHostAlloc / cudaHostRegister) let the copies overlap. */
typedef struct split_request {
  const uint8_t* rgb;       /* height * width * 3 bytes, interleaved RGB8 */
  int width, height;
  int nclusters;            /* K <= 64 */
  int kmeans_iters;
  const float* centroids;   /* initial centroids, dim x K planar */
  int32_t* segment_labels;  /* out: height * width (image-local minimum
                               index of each segment, -1 = eroded) */
  float* centroids_out;     /* out (optional): dim x K */
  float* normals;           /* out (optional): 3 x height * width planar */
  int32_t* cluster_labels;  /* out (optional): height * width */
  void* user;               /* returned with the completion */
} split_request;

typedef struct split_completion {
  uint64_t ticket;    /* from split_server_submit */
  void* user;
  int status;         /* SPLIT_OK, or the error of the request's batch */
  int64_t pixels;
  double latency_ms;  /* submit -> results in the host buffers */
} split_completion;

typedef struct split_server_counters {
  uint64_t submitted, completed, batches;
  size_t in_use_bytes;       /* footprint of admitted, unfinished requests */
  size_t peak_in_use_bytes;
  size_t bytes_per_pixel;    /* the footprint of a pixel of a request */
  size_t budget_bytes;
} split_server_counters;

int split_server_create(const split_server_config* config, split_server** out);
/* The device footprint of one pixel of a request under these parameters
 * (arenas plus workspace; a request of w x h pixels holds
 * ceil(w * h / 64) * 64 times this while admitted).  0: invalid parameters. */
size_t split_server_bytes_per_pixel(const split_pipeline_params* params);
/* Grows every slot's resident arena to hold a batch of `pixels` pixels in up
 * to `max_requests` images (so that serving allocates nothing later).  Only
 * while the server is idle. */
int split_server_reserve(split_server* server, int64_t pixels, int max_requests);
/* Queues a request (never blocks on the GPU).  SPLIT_ERR_WORKSPACE: its
 * footprint exceeds the whole budget. */
int split_server_submit(split_server* server, const split_request* request,
                        uint64_t* ticket);
/* Returns up to `max` completions (*n of them), waiting up to timeout_ms for
 * the first (0: do not wait; < 0: until one arrives or nothing is pending). */
int split_server_poll(split_server* server, split_completion* out, int max,
                      int timeout_ms, int* n);
int split_server_stats(split_server* server, split_server_counters* out);
/* Finishes every submitted request, then frees the server. */
int split_server_destroy(split_server* server);
/* The admission and batch-formation policy on the host alone (for tests):
 * n requests of the given footprints and pixel counts arrive at once;
 * batch_of[i] receives request i's batch.  Returns the number of batches or
 * a negative status. */
int split_server_admission_test(const int64_t* footprints, const int64_t* pixels,
                                int n, int64_t budget, int64_t max_batch_pixels,
                                int max_inflight, int32_t* batch_of,
                                int64_t* peak_in_use);

/* ======================================================================== */
/* tuning table (no counterpart in the reference)                           */
/* ======================================================================== */

/* Launch choices per image size class, filled by an autotuner
 * (split_gb300/tune.py measures the candidates on the current GPU and caches
 * the winners).  An image uses the first entry whose max_pixels is at least
 * its pixel count; with no such entry (or an empty table) the defaults
 * apply: 64-row k-means units, as many resident blocks per SM as fit.
 * The unit height is chosen from each image's own size, so an image gets the
 * same reduction tree (and bit-identical results) alone, in a pipeline and
 * in a batch.  Results differ between unit heights only by FP32 rounding of
 * the centroid sums.  Changing the table between sizing a batch and binding
 * it is allowed (workspaces are sized for the smallest unit height). */
#define SPLIT_TUNE_MAX_ENTRIES 64
typedef struct {
  int64_t max_pixels;        /* upper bound of the class (entries ascending) */
  int kmeans_unit_rows;      /* 16, 32, 64 or 128: rows of a k-means unit    */
  int kmeans_blocks_per_sm;  /* 0 = as many as fit, else 1..8 (capped);
                                single-image clustering only (batches run
                                as many as fit)                           */
} split_tune_entry;

/* Replaces the table (n = 0 restores the defaults).  Rejects unsorted
 * classes and values outside the ranges above. */
int split_tune_set(const split_tune_entry* entries, int n);
/* Copies up to `capacity` entries; returns the table's length. */
int split_tune_get(split_tune_entry* out, int capacity);

#ifdef __cplusplus
}
#endif

#endif /* SPLIT_GB300_H */
