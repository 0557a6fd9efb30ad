/*
 * split_synth.h - seeded synthetic inputs for the segmentation path.
 *
 * The reference has no fixtures or datasets (its sample loads a user image,
 * samples/src/main.cu:157-158), so every workload of this library is generated
 * from a seed.  These host functions are exported by libsplit_synth.so
 * (split_synth/synth.c), a library of their own: the GPU path and the timed
 * CPU run of the reference's code see identical bytes, and a process that only
 * generates inputs loads nothing of the segmentation library.  All return 0 on
 * success, 1 on a bad argument, 2 on host OOM.
 */
#ifndef SPLIT_SYNTH_H
#define SPLIT_SYNTH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Voronoi partition of `ncells` seeded centres (integer squared distance, ties
 * to the lower centre index).  Cell colours are uniform random RGB8, or drawn
 * from `npalette` random palette entries when npalette > 0.  With
 * illum_gradient != 0 the colour is scaled by 0.6 + 0.4 * x / (width - 1).
 * Gaussian noise of standard deviation `sigma` is added per channel, then the
 * value is rounded and clipped to [0, 255].  Output: interleaved RGB8,
 * row-major, height * width * 3 bytes. */
int split_synth_voronoi_rgb8(uint64_t seed, int width, int height, int ncells,
                             int npalette, int illum_gradient, double sigma,
                             uint8_t* out_rgb);

/* `nclusters` distinct seeded pixel picks of an RGB8 image, written as
 * initial centroids in the planar dim x nclusters layout.  dim is 3 (RGB / 255)
 * or 5 (RGB / 255, xy_scale * column, xy_scale * row). */
int split_synth_pick_centroids(uint64_t seed, const uint8_t* rgb, int width,
                               int height, int nclusters, int dim,
                               float xy_scale, float* centroids);

/* The float feature value of an 8-bit channel: (float)v / 255.0f. */
float split_synth_feature_u8(uint8_t v);

/* Maze + blob label image (labelling stress case): one serpentine corridor
 * component with label 0 covering about half of the pixels, the remaining
 * wall pixels cut into small blobs with random nonzero 32-bit labels. */
int split_synth_maze_labels(uint64_t seed, int width, int height,
                            int32_t* out);

#ifdef __cplusplus
}
#endif

#endif /* SPLIT_SYNTH_H */
