"""Seeded synthetic inputs (include/split_synth.h) as numpy arrays."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N


def _p(a: np.ndarray):
    return C.c_void_p(a.ctypes.data)


def voronoi_rgb8(seed: int, width: int, height: int, ncells: int, npalette: int = 0,
                 illum_gradient: bool = False, sigma: float = 0.0) -> np.ndarray:
    out = np.empty((height, width, 3), dtype=np.uint8)
    N.check(N.load().split_synth_voronoi_rgb8(seed, width, height, ncells, npalette,
                                              int(illum_gradient), sigma, _p(out)),
            "synth.voronoi_rgb8")
    return out


def pick_centroids(seed: int, rgb: np.ndarray, k: int, dim: int = 3,
                   xy_scale: float = 0.1) -> np.ndarray:
    rgb = np.ascontiguousarray(rgb, dtype=np.uint8)
    h, w = rgb.shape[:2]
    out = np.empty((dim, k), dtype=np.float32)
    N.check(N.load().split_synth_pick_centroids(seed, _p(rgb), w, h, k, dim, xy_scale, _p(out)),
            "synth.pick_centroids")
    return out


def maze_labels(seed: int, width: int, height: int) -> np.ndarray:
    out = np.empty((height, width), dtype=np.int32)
    N.check(N.load().split_synth_maze_labels(seed, width, height, _p(out)), "synth.maze_labels")
    return out


def features(rgb: np.ndarray, dim: int = 3, xy_scale: float = 0.1) -> np.ndarray:
    """Planar (dim, N) float32 features of an RGB8 image: byte / 255 (float32
    division) and, for dim 5, xy_scale * (column, row) in float32."""
    h, w = rgb.shape[:2]
    f = (rgb.reshape(-1, 3).astype(np.float32) / np.float32(255.0)).T
    if dim == 3:
        return np.ascontiguousarray(f)
    yy, xx = np.divmod(np.arange(h * w, dtype=np.int64), w)
    s = np.float32(xy_scale)
    xy = np.stack([s * xx.astype(np.float32), s * yy.astype(np.float32)])
    return np.ascontiguousarray(np.concatenate([f, xy]).astype(np.float32))
