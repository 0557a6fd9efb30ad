/*
 * split_gb300.hpp -- header-only C++ layer over the C ABI (split_gb300.h)
 * that restores the names, namespaces and argument order of split's device
 * entry points, so call sites written against
 * split/include/split/device/{kmeans,ccl,morph,sfs}/ keep compiling after a
 * namespace change.
 *
 * The reference's cusp::array1d/array2d views become the non-owning view1d /
 * view2d below (pointer + sizes, row-major, planar for multi-channel data);
 * its thrust::device_ptr<void> temp becomes Temp, a caller-owned, zero-filled
 * device block sized by the *_workspace functions.  Failures throw
 * split::device::error (the reference's Thrust calls throw
 * thrust::system_error); device-side failures are read from the workspace
 * after the stream synchronises (Temp::check).
 */
#pragma once

#include <cuda_runtime_api.h>

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>

#include "split_gb300.h"

namespace split {
namespace device {

class error : public std::runtime_error {
 public:
  error(int status, const std::string& where)
      : std::runtime_error(where + ": " + split_status_string(status)), status_(status) {}
  int status() const noexcept { return status_; }

 private:
  int status_;
};

inline void check(int status, const char* where) {
  if (status != SPLIT_OK) throw error(status, where);
}

inline void check_cuda(cudaError_t e, const char* where) {
  if (e != cudaSuccess) throw error(SPLIT_ERR_CUDA, std::string(where) + " (" + cudaGetErrorString(e) + ")");
}

/* Non-owning 1-D view (cusp::array1d<T, device_memory>::view). */
template <class T>
struct view1d {
  T* ptr = nullptr;
  int64_t n = 0;
  view1d() = default;
  view1d(T* p, int64_t size) : ptr(p), n(size) {}
  int64_t size() const { return n; }
  T* data() const { return ptr; }
};

/* Non-owning row-major 2-D view (cusp::array2d_view<..., row_major>):
 * rows x cols, pitch == cols.  Features are planar D x N (one row per
 * channel), label images H x W, normals 3 x N. */
template <class T>
struct view2d {
  T* ptr = nullptr;
  int64_t rows = 0, cols = 0;
  view2d() = default;
  view2d(T* p, int64_t r, int64_t c) : ptr(p), rows(r), cols(c) {}
  int64_t num_rows() const { return rows; }
  int64_t num_cols() const { return cols; }
  int64_t num_entries() const { return rows * cols; }
  T* data() const { return ptr; }
  view1d<T> values() const { return view1d<T>(ptr, rows * cols); }
  view1d<T> row(int64_t i) const { return view1d<T>(ptr + i * cols, cols); }
};

template <class T>
using const_view2d = view2d<const T>;
template <class T>
using const_view1d = view1d<const T>;

/* Caller-owned device workspace.  Allocated 256-byte aligned and zero-filled
 * once; the entry points leave it ready for the next call.  A small tail
 * holds device scalars (iteration counts, segment counts) that the calls
 * returning host values read back. */
class Temp {
 public:
  Temp() = default;
  explicit Temp(size_t bytes) { reserve(bytes); }
  Temp(const Temp&) = delete;
  Temp& operator=(const Temp&) = delete;
  Temp(Temp&& o) noexcept : p_(o.p_), bytes_(o.bytes_) { o.p_ = nullptr; o.bytes_ = 0; }
  ~Temp() { if (p_) cudaFree(p_); }

  /* Grow to at least `bytes` (contents are not kept). */
  void reserve(size_t bytes) {
    bytes = (bytes + 255) & ~size_t(255);
    if (p_ && bytes <= bytes_) return;
    if (p_) cudaFree(p_);
    p_ = nullptr;
    check_cuda(cudaMalloc(&p_, bytes + kTail), "Temp: cudaMalloc");
    check_cuda(cudaMemset(p_, 0, bytes + kTail), "Temp: cudaMemset");
    bytes_ = bytes;
  }
  void* get() const { return p_; }
  size_t size() const { return bytes_; }
  int32_t* scalar(int i) const {
    return reinterpret_cast<int32_t*>(static_cast<char*>(p_) + bytes_) + i;
  }
  /* Throws if a call that used this workspace recorded a device-side error. */
  void check(cudaStream_t stream = nullptr) const {
    int st = SPLIT_OK;
    split::device::check(split_workspace_status(p_, stream, &st), "split_workspace_status");
    split::device::check(st, "device");
  }

 private:
  static constexpr size_t kTail = 256;
  void* p_ = nullptr;
  size_t bytes_ = 0;
};

namespace detail {
/* A feature list without an image behind it is tiled as rows of this width. */
inline int default_width(int64_t n) { return n < 4096 ? (int)(n > 0 ? n : 1) : 4096; }
}  // namespace detail

/* ------------------------------------------------------------------ kmeans */
namespace kmeans {

/* kmeans/cluster.cuh:46-47.  `width` is the image width when the points are
 * pixels (0: the points are tiled as rows of up to 4096). */
inline std::size_t cluster_workspace(int npoints, int nclusters, int dim, int width = 0) {
  return split_kmeans_cluster_workspace_size_2d(
      npoints, width > 0 ? width : detail::default_width(npoints), nclusters, dim);
}

/* How cluster() measures the centroid shift of its convergence test.
 * reference: as the reference's own code does (SPLIT_KMEANS_REFERENCE_SHIFT),
 *   so a threshold >= 0 stops at the reference's iteration; used where that
 *   rule is defined (threshold >= 0, 3-D points, K >= 3), the L2 change
 *   elsewhere (a threshold < 0 runs exactly max_iter iterations either way).
 * l2_change: the L2 change of the centroid matrix. */
enum class Convergence { reference, l2_change };

/* kmeans/cluster.cuh:31-37.  Planar D x N points (D = 3 or 5, all rows read
 * from memory), D x K centroids in/out, any K up to 2^20 (K <= 64 in the
 * persistent kernel, larger K in the many-cluster path).  Returns the
 * iterations performed (the reference returns nothing; reading the count
 * synchronises `stream`). */
inline int cluster(const_view2d<float> points, view2d<float> centroids, view1d<int> labels,
                   Temp& temp, int max_iter, float threshold = 1.f, int width = 0,
                   cudaStream_t stream = nullptr,
                   Convergence convergence = Convergence::reference) {
  const int64_t n = points.num_cols();
  const int w = width > 0 ? width : detail::default_width(n);
  const int k = (int)centroids.num_cols();
  const bool ref_rule = convergence == Convergence::reference && threshold >= 0.f &&
                        points.num_rows() == 3 && k >= 3 && n * (k - 2) >= 3 * (int64_t)k;
  temp.reserve(split_kmeans_cluster_workspace_size_2d(n, w, (int)centroids.num_cols(),
                                                      (int)points.num_rows()));
  check(split_kmeans_cluster(points.data(),
                             SPLIT_LAYOUT_PLANAR | (ref_rule ? SPLIT_KMEANS_REFERENCE_SHIFT : 0),
                             (int)points.num_rows(), n, w,
                             0.f, centroids.data(), (int)centroids.num_cols(), labels.data(),
                             temp.get(), temp.size(), max_iter, threshold, temp.scalar(0),
                             stream),
        "kmeans::cluster");
  int iters = 0;
  check_cuda(cudaMemcpyAsync(&iters, temp.scalar(0), sizeof(int), cudaMemcpyDeviceToHost, stream),
             "kmeans::cluster: iterations");
  check_cuda(cudaStreamSynchronize(stream), "kmeans::cluster: sync");
  temp.check(stream);
  return iters;
}

/* kmeans/label.cuh:39-40 */
inline std::size_t label_points_workspace(int npoints, int nclusters) {
  return split_kmeans_assign_workspace_size(npoints, nclusters);
}

/* kmeans/label.cuh:27-31 (centroids first, as in the reference). */
inline void label_points(const_view2d<float> centroids, const_view2d<float> points,
                         view1d<int> labels, Temp& temp, cudaStream_t stream = nullptr) {
  const int64_t n = points.num_cols();
  temp.reserve(split_kmeans_assign_workspace_size(n, (int)centroids.num_cols()));
  check(split_kmeans_assign(points.data(), SPLIT_LAYOUT_PLANAR, (int)points.num_rows(), n,
                            detail::default_width(n), 0.f, centroids.data(),
                            (int)centroids.num_cols(), labels.data(), temp.get(), temp.size(),
                            stream),
        "kmeans::label_points");
}

/* kmeans/centroids.cuh:39-40.  The reference's size takes no dimension; 5
 * (the largest supported) covers every call. */
inline std::size_t calculate_centroids_workspace(int npoints, int ncentroids) {
  return split_kmeans_update_workspace_size(npoints, ncentroids, 5);
}

/* kmeans/centroids.cuh:26-30.  A cluster without members keeps its input
 * centroid.  Labels outside [0, K) are ignored (eroded pixels, -1). */
inline void calculate_centroids(const_view1d<int> labels, const_view2d<float> points,
                                view2d<float> centroids, Temp& temp,
                                cudaStream_t stream = nullptr) {
  const int64_t n = points.num_cols();
  const int dim = (int)points.num_rows();
  temp.reserve(split_kmeans_update_workspace_size(n, (int)centroids.num_cols(), dim));
  check(split_kmeans_update(labels.data(), points.data(), SPLIT_LAYOUT_PLANAR, dim, n,
                            detail::default_width(n), 0.f, centroids.data(),
                            (int)centroids.num_cols(), temp.get(), temp.size(), stream),
        "kmeans::calculate_centroids");
}

/* kmeans/propagation.cuh:23-26 */
inline void propagate_centroids(const_view1d<int> labels, const_view2d<float> centroids,
                                view2d<float> points, cudaStream_t stream = nullptr) {
  check(split_kmeans_propagate(labels.data(), labels.size(), centroids.data(),
                               (int)centroids.num_cols(), (int)centroids.num_rows(),
                               points.data(), stream),
        "kmeans::propagate_centroids");
}

}  // namespace kmeans

/* --------------------------------------------------------------------- ccl */
namespace ccl {

/* ccl/connected_components.cuh:25-29.  Labels are the maximum linear index of
 * each 4-connected component (the reference's converged result) unless
 * another connectivity / convention is given; `max_iterations` is accepted
 * and ignored (union-find always converges). */
inline void connected_components(const_view2d<int> labels, Temp& temp, view1d<int> out,
                                 int max_iterations = 10, int connectivity = 4,
                                 int convention = SPLIT_LABEL_MAX_INDEX,
                                 int32_t* d_sizes = nullptr, cudaStream_t stream = nullptr) {
  (void)max_iterations;
  const int w = (int)labels.num_cols(), h = (int)labels.num_rows();
  temp.reserve(split_ccl_workspace_size(w, h));
  check(split_ccl(labels.data(), w, h, connectivity, convention, out.data(), d_sizes,
                  temp.get(), temp.size(), stream),
        "ccl::connected_components");
}

/* ccl/compress_labels.cuh:21-23.  Returns the number of distinct labels
 * (synchronises `stream`, as the reference's host-side return does). */
inline int compress_labels(view1d<int> labels, Temp& temp, cudaStream_t stream = nullptr) {
  temp.reserve(split_compress_labels_workspace_size(labels.size()));
  check(split_compress_labels(labels.data(), labels.size(), temp.scalar(1), temp.get(),
                              temp.size(), stream),
        "ccl::compress_labels");
  int count = 0;
  check_cuda(cudaMemcpyAsync(&count, temp.scalar(1), sizeof(int), cudaMemcpyDeviceToHost, stream),
             "ccl::compress_labels: count");
  check_cuda(cudaStreamSynchronize(stream), "ccl::compress_labels: sync");
  temp.check(stream);
  return count;
}

/* ccl/segment_adjacency.cuh:14-16.  `edges` holds 16 entries per pixel;
 * returns the edge count m (sources in edges[0, m), targets in edges[m, 2m);
 * synchronises `stream`, as the reference's host-side return does). */
inline int segment_adjacency_edges(const_view2d<int> labels, view1d<int> edges, Temp& temp,
                                   cudaStream_t stream = nullptr) {
  const int w = (int)labels.num_cols(), h = (int)labels.num_rows();
  temp.reserve(split_segment_adjacency_edges_workspace_size(w, h));
  check(split_segment_adjacency_edges(labels.data(), w, h, edges.data(), temp.scalar(1),
                                      temp.get(), temp.size(), stream),
        "ccl::segment_adjacency_edges");
  int count = 0;
  check_cuda(cudaMemcpyAsync(&count, temp.scalar(1), sizeof(int), cudaMemcpyDeviceToHost, stream),
             "ccl::segment_adjacency_edges: count");
  check_cuda(cudaStreamSynchronize(stream), "ccl::segment_adjacency_edges: sync");
  temp.check(stream);
  return count;
}

/* ccl/segment_adjacency.cuh:21-24.  `keys` and `adjacency` hold 8 entries
 * per pixel; returns the number of distinct sorted pairs (synchronises). */
inline int segment_adjacency(const_view2d<int> labels, view1d<int> keys, view1d<int> adjacency,
                             Temp& temp, cudaStream_t stream = nullptr) {
  const int w = (int)labels.num_cols(), h = (int)labels.num_rows();
  temp.reserve(split_segment_adjacency_workspace_size(w, h));
  check(split_segment_adjacency(labels.data(), w, h, keys.data(), adjacency.data(),
                                temp.scalar(1), temp.get(), temp.size(), stream),
        "ccl::segment_adjacency");
  int count = 0;
  check_cuda(cudaMemcpyAsync(&count, temp.scalar(1), sizeof(int), cudaMemcpyDeviceToHost, stream),
             "ccl::segment_adjacency: count");
  check_cuda(cudaStreamSynchronize(stream), "ccl::segment_adjacency: sync");
  temp.check(stream);
  return count;
}

/* ccl/merge_small_segments.cuh:21-22 (the segment count is not needed). */
inline std::size_t merge_small_segments_workspace(int npoints, int nsegments, int width) {
  (void)nsegments;
  return split_merge_small_workspace_size(width, (npoints + width - 1) / width);
}

/* ccl/merge_small_segments.cuh:15-19.  The reference's rule by default
 * (nearest mean chroma, its channel-0 reading included); pass
 * SPLIT_MERGE_MOST_BOUNDARY for the boundary-count rule.  Labels need not be
 * compressed. */
inline void merge_small_segments(const_view2d<float> chrominance, view2d<int> labels, Temp& temp,
                                 int P = 10, int policy = SPLIT_MERGE_REF_CHROMA,
                                 cudaStream_t stream = nullptr) {
  const int w = (int)labels.num_cols(), h = (int)labels.num_rows();
  temp.reserve(split_merge_small_workspace_size(w, h));
  check(split_merge_small(labels.data(), w, h, P, policy, chrominance.data(), nullptr,
                          temp.get(), temp.size(), stream),
        "ccl::merge_small_segments");
}

/* ccl/merge_smooth_boundaries.cuh:29-31 (segment and edge counts not needed). */
inline std::size_t merge_smooth_boundaries_workspace(int npoints, int nsegments, int nedges,
                                                     int width) {
  (void)nsegments;
  (void)nedges;
  return split_merge_smooth_workspace_size(width, (npoints + width - 1) / width);
}

/* ccl/merge_smooth_boundaries.cuh:20-25.  points: planar (>= 3) x N. */
inline void merge_smooth_boundaries(const_view2d<float> points, int nsegments,
                                    view2d<int> labels, Temp& temp, float threshold = 0.01f,
                                    cudaStream_t stream = nullptr) {
  (void)nsegments;
  const int w = (int)labels.num_cols(), h = (int)labels.num_rows();
  temp.reserve(split_merge_smooth_workspace_size(w, h));
  check(split_merge_smooth(labels.data(), w, h, points.data(), threshold, temp.get(),
                           temp.size(), stream),
        "ccl::merge_smooth_boundaries");
}

}  // namespace ccl

/* ------------------------------------------------------------------- morph */
namespace morph {

/* morph/erode.cuh:16-18: in-place square erosion of every label's mask
 * (eroded pixels = -1), any niterations >= 0.  The kernel writes to a
 * separate buffer: pass one (`scratch`, at least as large as `labels`) or let
 * the call take stream-ordered memory (cudaMallocAsync) for it, as the
 * reference allocates internally.  One kernel pass erodes by up to 16; a
 * larger radius runs in passes (square erosions compose: radius a then b is
 * radius a + b, with the image border and -1 pixels as background). */
inline void erode(view2d<int> labels, int niterations = 1, int32_t* scratch = nullptr,
                  cudaStream_t stream = nullptr) {
  if (niterations < 0) check(SPLIT_ERR_INVALID, "morph::erode");
  if (niterations == 0) return;
  const int w = (int)labels.num_cols(), h = (int)labels.num_rows();
  const size_t bytes = sizeof(int32_t) * (size_t)w * h;
  int32_t* tmp = scratch;
  if (!tmp) check_cuda(cudaMallocAsync((void**)&tmp, bytes, stream), "morph::erode: alloc");
  int32_t* src = labels.data();
  int32_t* dst = tmp;
  int st = SPLIT_OK;
  for (int left = niterations; left > 0 && st == SPLIT_OK;) {
    const int r = left < 16 ? left : 16;
    st = split_erode(src, dst, w, h, r, stream);
    left -= r;
    int32_t* t = src;
    src = dst;
    dst = t;
  }
  if (st == SPLIT_OK && src != labels.data())
    st = cudaMemcpyAsync(labels.data(), src, bytes, cudaMemcpyDeviceToDevice, stream) ==
                 cudaSuccess ? SPLIT_OK : SPLIT_ERR_CUDA;
  if (!scratch) cudaFreeAsync(tmp, stream);
  check(st, "morph::erode");
}

}  // namespace morph

/* --------------------------------------------------------------------- sfs */
namespace sfs {

/* sfs/sobel_normals.cuh:17-20: H x W heights -> 3 x N planar normals. */
inline void sobel_normals(const_view2d<float> heights, view2d<float> normals, float depth,
                          cudaStream_t stream = nullptr) {
  check(split_sobel_normals(heights.data(), (int)heights.num_cols(), (int)heights.num_rows(),
                            depth, normals.data(), stream),
        "sfs::sobel_normals");
}

/* sfs/estimate_normals.cuh:14-18: H x W shading intensity lit from L ->
 * 3 x N planar normals; relaxation to |b - A x| <= tol |b| (the reference:
 * 1e-5, 1500 sweeps).  Returns the sweeps performed (synchronises). */
inline int estimate_normals(const_view2d<float> shading_intensity, float3 light_vector,
                            view2d<float> normals, float smoothness_weight, Temp& temp,
                            int max_iter = 1500, float tol = 1e-5f,
                            cudaStream_t stream = nullptr) {
  const int w = (int)shading_intensity.num_cols(), h = (int)shading_intensity.num_rows();
  temp.reserve(split_estimate_normals_workspace_size(w, h));
  check(split_estimate_normals(shading_intensity.data(), w, h, light_vector.x, light_vector.y,
                               light_vector.z, smoothness_weight, max_iter, tol, normals.data(),
                               temp.scalar(2), temp.get(), temp.size(), stream),
        "sfs::estimate_normals");
  int iters = 0;
  check_cuda(cudaMemcpyAsync(&iters, temp.scalar(2), sizeof(int), cudaMemcpyDeviceToHost, stream),
             "sfs::estimate_normals: sweeps");
  check_cuda(cudaStreamSynchronize(stream), "sfs::estimate_normals: sync");
  temp.check(stream);
  return iters;
}

}  // namespace sfs

// ---- color -----------------------------------------------------------------
namespace color {

/* The sample's feature preparation from RGB8 bytes (the reference converts
 * float images with convert_color_space, conversion.cuh:21-58; main.cu:
 * 169-225).  Inputs are interleaved RGB8, n = the columns of the output. */

/* rgb_to_ic: ic (3 x n) = intensity, r / intensity, g / intensity of the
 * channels clamped to >= 1/255 (conversion.inl:99-108). */
inline void rgb8_to_ic(const unsigned char* rgb, view2d<float> ic, cudaStream_t stream = nullptr) {
  check(split_rgb8_to_ic(rgb, (int64_t)ic.num_cols(), ic.data(), stream), "color::rgb8_to_ic");
}

/* rgb_to_lab + beta_feature: features (3 x n) = beta, a*, b*; luminance
 * (optional, n) = L* (beta_feature.cuh:12-15). */
inline void rgb8_to_lab_beta(const unsigned char* rgb, view2d<float> features, Temp& temp,
                             float mu = 1e5f, float* luminance = nullptr,
                             cudaStream_t stream = nullptr) {
  const int64_t n = (int64_t)features.num_cols();
  temp.reserve(split_pack_lab_beta_workspace_size(n));
  check(split_pack_lab_beta(rgb, n, mu, SPLIT_LAYOUT_PLANAR, features.data(), luminance,
                            temp.get(), temp.size(), stream),
        "color::rgb8_to_lab_beta");
}

}  // namespace color

}  // namespace device
}  // namespace split
