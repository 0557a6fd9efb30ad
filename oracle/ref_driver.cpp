// extern "C" driver over the reference's own segmentation entry points,
// compiled for the CPU with Thrust's OMP device system (oracle/refbuild.py).
// Test infrastructure only: used to generate golden fixtures, to pin the
// oracle restatement, and as the timed CPU reference.  Host arrays in, host
// arrays out; all layouts follow the reference (planar D x N features,
// row-major H x W labels, planar 3 x N normals).
#include <cstdint>
#include <cstring>
#include <vector>

#include <thrust/copy.h>
#include <thrust/device_malloc.h>
#include <thrust/device_free.h>

#include "split/device/ccl/compress_labels.cuh"
#include "split/device/color/beta_feature.cuh"
#include "split/device/color/conversion.cuh"
#include "split/device/detail/unary_functional.cuh"
#include "split/device/ccl/connected_components.cuh"
#include "split/device/ccl/merge_small_segments.cuh"
#include "split/device/ccl/merge_smooth_boundaries.cuh"
#include "split/device/ccl/segment_adjacency.cuh"
#include "split/device/kmeans/centroids.cuh"
#include "split/device/kmeans/cluster.cuh"
#include "split/device/kmeans/label.cuh"
#include "split/device/kmeans/propagation.cuh"
#include "split/device/morph/erode.cuh"
#include "split/device/sfs/sobel_normals.cuh"

// The one CUDA kernel in these sources (segment_adjacency.cu, never launched)
// declares an extern shared array; under the host build it needs a symbol.
namespace split {
namespace device {
namespace ccl {
int s_labels[1];
}
}  // namespace device
}  // namespace split

using split::real;
using Mat = cusp::array2d<real, cusp::device_memory>;
using IMat = cusp::array2d<int, cusp::device_memory>;
using IVec = cusp::array1d<int, cusp::device_memory>;

namespace {
struct Temp {
  explicit Temp(std::size_t n) : p(thrust::device_malloc(n > 0 ? n : 1)) {}
  ~Temp() { thrust::device_free(p); }
  thrust::device_ptr<void> p;
};
template <class A, class T>
void to_dev(A& a, const T* h, std::size_t n) {
  thrust::copy(h, h + n, a.values.begin());
}
template <class A, class T>
void to_host(const A& a, T* h, std::size_t n) {
  thrust::copy(a.values.begin(), a.values.begin() + n, h);
}
}  // namespace

extern "C" {

int ref_kmeans_cluster(const float* pts, int dim, int n, float* cent, int k, int32_t* labels,
                       int iters) {
  Mat P(dim, n), Cc(dim, k);
  IVec L(n);
  to_dev(P, pts, (std::size_t)dim * n);
  to_dev(Cc, cent, (std::size_t)dim * k);
  Temp t(split::device::kmeans::cluster_workspace(n, k, dim));
  split::device::kmeans::cluster(P, Cc, L, t.p, iters, -1.0f);
  to_host(Cc, cent, (std::size_t)dim * k);
  thrust::copy(L.begin(), L.end(), labels);
  return 0;
}

// cluster() with a convergence threshold (cluster.cu:71: it stops once the
// change of the centroid shift between iterations is at most i_threshold).
// The reference reports its iteration count and every shift on stdout only;
// oracle/ref.py reads them from there.
int ref_kmeans_cluster_threshold(const float* pts, int dim, int n, float* cent, int k,
                                 int32_t* labels, int max_iter, float threshold) {
  Mat P(dim, n), Cc(dim, k);
  IVec L(n);
  to_dev(P, pts, (std::size_t)dim * n);
  to_dev(Cc, cent, (std::size_t)dim * k);
  Temp t(split::device::kmeans::cluster_workspace(n, k, dim));
  split::device::kmeans::cluster(P, Cc, L, t.p, max_iter, threshold);
  to_host(Cc, cent, (std::size_t)dim * k);
  thrust::copy(L.begin(), L.end(), labels);
  return 0;
}

int ref_label_points(const float* pts, int dim, int n, const float* cent, int k,
                     int32_t* labels) {
  Mat P(dim, n), Cc(dim, k);
  IVec L(n);
  to_dev(P, pts, (std::size_t)dim * n);
  to_dev(Cc, cent, (std::size_t)dim * k);
  Temp t(split::device::kmeans::label_points_workspace(n, k));
  split::device::kmeans::label_points(Cc, P, L, t.p);
  thrust::copy(L.begin(), L.end(), labels);
  return 0;
}

int ref_calculate_centroids(const int32_t* labels, const float* pts, int dim, int n, float* cent,
                            int k) {
  Mat P(dim, n), Cc(dim, k);
  IVec L(n);
  to_dev(P, pts, (std::size_t)dim * n);
  thrust::copy(labels, labels + n, L.begin());
  Temp t(split::device::kmeans::calculate_centroids_workspace(n, k));
  split::device::kmeans::calculate_centroids(L, P, Cc, t.p);
  to_host(Cc, cent, (std::size_t)dim * k);
  return 0;
}

int ref_connected_components(const int32_t* in, int w, int h, int32_t* out, int max_iter) {
  IMat A(h, w);
  IVec O((std::size_t)w * h);
  to_dev(A, in, (std::size_t)w * h);
  Temp t(sizeof(int) * (std::size_t)w * h * 2);
  split::device::ccl::connected_components(A, t.p, O, max_iter);
  thrust::copy(O.begin(), O.end(), out);
  return 0;
}

int ref_compress_labels(int32_t* labels, int n) {
  IVec L(n);
  thrust::copy(labels, labels + n, L.begin());
  Temp t(sizeof(int) * (std::size_t)n);
  const int c = split::device::ccl::compress_labels(L, t.p);
  thrust::copy(L.begin(), L.end(), labels);
  return c;
}

int ref_merge_small_segments(const float* chroma, int32_t* labels, int w, int h, int P) {
  const std::size_t n = (std::size_t)w * h;
  Mat Ch(2, n);
  IMat L(h, w);
  to_dev(Ch, chroma, 2 * n);
  to_dev(L, labels, n);
  int mx = 0;
  for (std::size_t i = 0; i < n; ++i) mx = std::max(mx, (int)labels[i]);
  Temp t(split::device::ccl::merge_small_segments_workspace((int)n, mx + 1));
  split::device::ccl::merge_small_segments(Ch, L, t.p, P);
  to_host(L, labels, n);
  return 0;
}

// merge_smooth_boundaries (merge_smooth_boundaries.cu:134-243, staged with
// the one-token reduction fix recorded in refbuild.py).  labels: h x w,
// compressed to [0, nsegments); points: planar 3 x n features.  Its
// workspace query takes the edge count, which only the call itself learns:
// the bound 8 n (every pixel's eight neighbours) is passed.
int ref_merge_smooth_boundaries(const float* pts, int32_t* labels, int w, int h, int nsegments,
                                float threshold) {
  const std::size_t n = (std::size_t)w * h;
  Mat P(3, n);
  IMat L(h, w);
  to_dev(P, pts, 3 * n);
  to_dev(L, labels, n);
  Temp t(split::device::ccl::merge_smooth_boundaries_workspace((int)n, nsegments, (int)(8 * n)));
  split::device::ccl::merge_smooth_boundaries(P, nsegments, L, t.p, threshold);
  to_host(L, labels, n);
  return 0;
}

// segment_adjacency_edges (segment_adjacency.cu:170-254): the m sources then
// the m targets into `edges` (room for 2 m); returns m.
int ref_segment_adjacency_edges(const int32_t* labels, int w, int h, int32_t* edges) {
  const std::size_t n = (std::size_t)w * h;
  IMat L(h, w);
  to_dev(L, labels, n);
  IVec E(16 * n);
  const int m = split::device::ccl::segment_adjacency_edges(L, E);
  thrust::copy(E.begin(), E.begin() + 2 * (std::size_t)m, edges);
  return m;
}

// segment_adjacency (segment_adjacency.cu:256-289): the distinct sorted label
// pairs into keys / adj (room for their number); returns it.
int ref_segment_adjacency(const int32_t* labels, int w, int h, int32_t* keys, int32_t* adj) {
  const std::size_t n = (std::size_t)w * h;
  IMat L(h, w);
  to_dev(L, labels, n);
  IVec K(8 * n), A(8 * n);
  const int m = split::device::ccl::segment_adjacency(L, K, A);
  thrust::copy(K.begin(), K.begin() + m, keys);
  thrust::copy(A.begin(), A.begin() + m, adj);
  return m;
}

int ref_erode(int32_t* labels, int w, int h, int niter) {
  IMat L(h, w);
  to_dev(L, labels, (std::size_t)w * h);
  split::device::morph::erode(L, niter);
  to_host(L, labels, (std::size_t)w * h);
  return 0;
}

int ref_sobel_normals(const float* heights, int w, int h, float depth, float* normals) {
  const std::size_t n = (std::size_t)w * h;
  Mat H(h, w), Nn(3, n);
  to_dev(H, heights, n);
  split::device::sfs::sobel_normals(H, Nn, depth);
  to_host(Nn, normals, 3 * n);
  return 0;
}

int ref_rgb_to_lab(const float* rgb, int n, float* lab) {
  Mat A(3, n), B(3, n);
  to_dev(A, rgb, 3 * (std::size_t)n);
  split::device::color::convert_color_space(A, B, split::device::color::rgb_to_lab<>());
  to_host(B, lab, 3 * (std::size_t)n);
  return 0;
}

// The sample's intensity / chroma planes (samples/src/main.cu:169-179): RGB
// in [0, 1] clamped to >= 1/255, then color::rgb_to_ic.
int ref_rgb_to_ic(const float* rgb, int n, float* ic) {
  Mat A(3, n), B(3, n);
  to_dev(A, rgb, 3 * (std::size_t)n);
  thrust::transform(A.values.begin(), A.values.end(), A.values.begin(),
                    split::device::detail::unary_max<real>(1.f / 255.f));
  split::device::color::convert_color_space(A, B, split::device::color::rgb_to_ic<>());
  to_host(B, ic, 3 * (std::size_t)n);
  return 0;
}

// The sample's feature preparation (samples/src/main.cu:169-173, :215-225):
// RGB in [0, 1] clamped to >= 1/255, converted to L*a*b*, L* saved, then the
// beta feature written in place of L*.  features: planar 3 x n (beta, a, b);
// luminance: n (L*).
int ref_lab_beta(const float* rgb, int n, float mu, float* features, float* luminance) {
  Mat A(3, n), B(3, n);
  to_dev(A, rgb, 3 * (std::size_t)n);
  thrust::transform(A.values.begin(), A.values.end(), A.values.begin(),
                    split::device::detail::unary_max<real>(1.f / 255.f));
  split::device::color::convert_color_space(A, B, split::device::color::rgb_to_lab<>());
  thrust::copy(B.row(0).begin(), B.row(0).end(), luminance);
  split::device::color::beta_feature(B, B.row(0), mu);
  to_host(B, features, 3 * (std::size_t)n);
  return 0;
}

int ref_propagate_centroids(const int32_t* labels, int n, const float* cent, int dim, int k,
                            float* out) {
  IVec L(n);
  Mat Cc(dim, k), O(dim, n);
  thrust::copy(labels, labels + n, L.begin());
  to_dev(Cc, cent, (std::size_t)dim * k);
  split::device::kmeans::propagate_centroids(L, Cc, O);
  to_host(O, out, (std::size_t)dim * n);
  return 0;
}

}  // extern "C"
