// The sample's segmentation sequence (samples/src/main.cu:216-304 of split)
// written against the reference's names through include/split_gb300.hpp:
// k-means -> 4-connected components -> compress -> chroma merge -> erosion,
// plus Sobel normals.  Writes every stage's output as raw little-endian
// arrays into the directory given as argv[1] for the Python test to check.
//
//   sample_pipeline OUTDIR [width height K iterations seed]
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "split_gb300.hpp"
#include "split_synth.h"

namespace sd = split::device;

template <class T>
static void dump(const std::string& dir, const char* name, const T* d_ptr, size_t n) {
  std::vector<T> h(n);
  sd::check_cuda(cudaMemcpy(h.data(), d_ptr, n * sizeof(T), cudaMemcpyDeviceToHost), name);
  std::string path = dir + "/" + name;
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f || std::fwrite(h.data(), sizeof(T), n, f) != n) {
    std::fprintf(stderr, "cannot write %s\n", path.c_str());
    std::exit(2);
  }
  std::fclose(f);
}

template <class T>
static T* upload(const std::vector<T>& h) {
  T* d = nullptr;
  sd::check_cuda(cudaMalloc((void**)&d, h.size() * sizeof(T)), "cudaMalloc");
  sd::check_cuda(cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice), "upload");
  return d;
}

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s OUTDIR [width height K iterations seed]\n", argv[0]);
    return 2;
  }
  const std::string dir = argv[1];
  const int W = argc > 2 ? std::atoi(argv[2]) : 512;
  const int H = argc > 3 ? std::atoi(argv[3]) : 512;
  const int K = argc > 4 ? std::atoi(argv[4]) : 8;
  const int iters = argc > 5 ? std::atoi(argv[5]) : 10;
  const unsigned long long seed = argc > 6 ? std::strtoull(argv[6], nullptr, 0) : 1234;
  const int N = W * H;
  try {
    // synthetic RGB8 image (32 Voronoi cells, sigma 4) and planar RGB features
    std::vector<uint8_t> rgb((size_t)N * 3);
    if (split_synth_voronoi_rgb8(seed, W, H, 32, 0, 0, 4.0, rgb.data()) != 0) return 3;
    std::vector<float> feat((size_t)3 * N);
    for (int i = 0; i < N; ++i)
      for (int c = 0; c < 3; ++c) feat[(size_t)c * N + i] = rgb[(size_t)3 * i + c] / 255.0f;
    std::vector<float> cent((size_t)3 * K);
    if (split_synth_pick_centroids(seed, rgb.data(), W, H, K, 3, 0.1f, cent.data()) != 0) return 3;

    float* d_feat = upload(feat);
    float* d_cent = upload(cent);
    int32_t *d_km = nullptr, *d_seg = nullptr, *d_tmp = nullptr;
    float* d_nrm = nullptr;
    sd::check_cuda(cudaMalloc((void**)&d_km, sizeof(int32_t) * N), "alloc");
    sd::check_cuda(cudaMalloc((void**)&d_seg, sizeof(int32_t) * N), "alloc");
    sd::check_cuda(cudaMalloc((void**)&d_tmp, sizeof(int32_t) * N), "alloc");
    sd::check_cuda(cudaMalloc((void**)&d_nrm, sizeof(float) * 3 * N), "alloc");

    sd::Temp temp(sd::kmeans::cluster_workspace(N, K, 3, W));
    dump(dir, "centroids_in.f32", d_cent, (size_t)3 * K);
    const int done = sd::kmeans::cluster(sd::const_view2d<float>(d_feat, 3, N),
                                         sd::view2d<float>(d_cent, 3, K),
                                         sd::view1d<int>(d_km, N), temp, iters, -1.0f, W);
    dump(dir, "kmeans_labels.i32", d_km, N);
    dump(dir, "centroids.f32", d_cent, (size_t)3 * K);

    // the sample's own call (main.cu:244-245): up to 100 iterations with a
    // 1e-3 threshold, which stops where the reference's convergence test does
    float* d_cent2 = upload(cent);
    int32_t* d_km2 = nullptr;
    sd::check_cuda(cudaMalloc((void**)&d_km2, sizeof(int32_t) * N), "alloc");
    const int done_thr = sd::kmeans::cluster(sd::const_view2d<float>(d_feat, 3, N),
                                             sd::view2d<float>(d_cent2, 3, K),
                                             sd::view1d<int>(d_km2, N), temp, 100, 1e-3f, W);
    dump(dir, "kmeans_thr_labels.i32", d_km2, N);
    dump(dir, "centroids_thr.f32", d_cent2, (size_t)3 * K);
    cudaFree(d_cent2);
    cudaFree(d_km2);

    sd::ccl::connected_components(sd::const_view2d<int>(d_km, H, W), temp,
                                  sd::view1d<int>(d_seg, N), 100);
    dump(dir, "ccl.i32", d_seg, N);
    const int nseg = sd::ccl::compress_labels(sd::view1d<int>(d_seg, N), temp);
    dump(dir, "compressed.i32", d_seg, N);

    // chroma = feature rows 0 and 1 (the sample's commented-out merge reads
    // the a, b rows of its Lab image the same way)
    sd::ccl::merge_small_segments(sd::const_view2d<float>(d_feat, 2, N),
                                  sd::view2d<int>(d_seg, H, W), temp, 64);
    dump(dir, "merged.i32", d_seg, N);
    sd::morph::erode(sd::view2d<int>(d_seg, H, W), 1, d_tmp);
    dump(dir, "eroded.i32", d_seg, N);
    sd::sfs::sobel_normals(sd::const_view2d<float>(d_feat, H, W),
                           sd::view2d<float>(d_nrm, 3, N), 1.0f);
    dump(dir, "normals.f32", d_nrm, (size_t)3 * N);
    sd::check_cuda(cudaDeviceSynchronize(), "sync");
    temp.check();
    std::printf("{\"iterations\": %d, \"segments\": %d, \"iterations_thr\": %d}\n", done,
                nseg, done_thr);
    cudaFree(d_feat); cudaFree(d_cent); cudaFree(d_km); cudaFree(d_seg); cudaFree(d_tmp);
    cudaFree(d_nrm);
  } catch (const sd::error& e) {
    std::fprintf(stderr, "split error: %s\n", e.what());
    return 1;
  }
  return 0;
}
