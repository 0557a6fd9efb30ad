// Host interface of the multi-image k-means launch (used by the batch
// pipeline).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <vector>

namespace sg {

struct KmBatchImage {
  const void* points;   // this image's features (layout of the batch)
  int64_t npoints;
  int width;
  int nclusters;
  int iters;
  float threshold;
  float* centroids;     // dim x K planar, in/out
  int32_t* labels;      // npoints
};

struct KmBatchPlan {
  int nimages, units, max_iter, layout, dim;
  int blocks_per_sm;   // from the tuning table (0: as many as fit)
};

size_t kmeans_batch_workspace(const KmBatchImage* imgs, int nimages);
// Uploads the image descriptors (synchronises `st`; call outside capture).
int kmeans_batch_prepare(const KmBatchImage* imgs, int nimages, int layout, int dim,
                         float xy_scale, void* ws, size_t ws_bytes, cudaStream_t st,
                         KmBatchPlan* plan);
// Launches only (capturable into a CUDA graph).
int kmeans_batch_run(const KmBatchPlan& plan, void* ws, cudaStream_t st);

}  // namespace sg
