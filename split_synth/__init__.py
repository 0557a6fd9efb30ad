"""Seeded synthetic inputs (include/split_synth.h) as numpy arrays.

The reference ships no images or datasets, so every workload of the tests and
the benchmark is generated here from a seed: Voronoi images, initial centroid
picks and maze labels.  The generators are plain C (synth.c, SplitMix64 /
PCG32 / Box-Muller), built with gcc into libsplit_synth.so on first use; they
give the same bytes on x86-64 and AArch64.  This library is separate from the
segmentation library, so a process that only generates inputs (for example the
timed CPU run of the reference's code) loads nothing of the product.
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "synth.c")
HEADER = os.path.join(ROOT, "include", "split_synth.h")
LIB = os.path.join(HERE, "_build", platform.machine(), "libsplit_synth.so")

__all__ = ["voronoi_rgb8", "pick_centroids", "maze_labels", "features", "build", "load",
           "exported_symbols"]

_lib = None


def build(verbose: bool = False) -> str:
    """Compile synth.c into LIB (rebuilt when the source or header is newer)."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if not os.path.exists(LIB) or max(os.path.getmtime(SRC), os.path.getmtime(HEADER)) > \
            os.path.getmtime(LIB):
        cmd = ["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off", "-fopenmp",
               "-o", LIB, SRC, "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            raise RuntimeError("building libsplit_synth.so failed")
    if verbose:
        print(f"built {LIB}")
    return LIB


def load():
    global _lib
    if _lib is None:
        lib = C.CDLL(build())
        vp, i32, f32, u64 = C.c_void_p, C.c_int, C.c_float, C.c_uint64
        sigs = {
            "split_synth_voronoi_rgb8": (i32, [u64, i32, i32, i32, i32, i32, C.c_double, vp]),
            "split_synth_pick_centroids": (i32, [u64, vp, i32, i32, i32, i32, f32, vp]),
            "split_synth_feature_u8": (f32, [C.c_uint8]),
            "split_synth_maze_labels": (i32, [u64, i32, i32, vp]),
        }
        for name, (res, args) in sigs.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def exported_symbols() -> list[str]:
    return ["split_synth_voronoi_rgb8", "split_synth_pick_centroids", "split_synth_feature_u8",
            "split_synth_maze_labels"]


def _check(status: int, where: str) -> None:
    """0 success, 1 bad argument, 2 host out of memory (split_synth.h)."""
    if status:
        why = {1: "invalid argument", 2: "out of host memory"}.get(status, "error")
        raise ValueError(f"{where}: {why} (status {status})")


def _p(a: np.ndarray):
    return C.c_void_p(a.ctypes.data)


def voronoi_rgb8(seed: int, width: int, height: int, ncells: int, npalette: int = 0,
                 illum_gradient: bool = False, sigma: float = 0.0) -> np.ndarray:
    out = np.empty((height, width, 3), dtype=np.uint8)
    _check(load().split_synth_voronoi_rgb8(seed, width, height, ncells, npalette,
                                           int(illum_gradient), sigma, _p(out)),
           "synth.voronoi_rgb8")
    return out


def pick_centroids(seed: int, rgb: np.ndarray, k: int, dim: int = 3,
                   xy_scale: float = 0.1) -> np.ndarray:
    rgb = np.ascontiguousarray(rgb, dtype=np.uint8)
    h, w = rgb.shape[:2]
    out = np.empty((dim, k), dtype=np.float32)
    _check(load().split_synth_pick_centroids(seed, _p(rgb), w, h, k, dim, xy_scale, _p(out)),
           "synth.pick_centroids")
    return out


def maze_labels(seed: int, width: int, height: int) -> np.ndarray:
    out = np.empty((height, width), dtype=np.int32)
    _check(load().split_synth_maze_labels(seed, width, height, _p(out)), "synth.maze_labels")
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
