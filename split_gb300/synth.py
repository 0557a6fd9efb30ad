"""Seeded synthetic inputs: the split_synth package, re-exported for the
package's own users (the autotuner's measuring images) and the tests."""
from split_synth import *  # noqa: F401,F403
from split_synth import features, maze_labels, pick_centroids, voronoi_rgb8  # noqa: F401
