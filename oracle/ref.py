"""ctypes wrapper of the reference's own code built for the CPU (Thrust OMP),
see oracle/refbuild.py.  Test infrastructure only: golden-fixture generation,
pinning the oracle restatement, and the timed CPU reference."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_lib = None


def available() -> bool:
    from . import refbuild
    return os.path.exists(refbuild.LIB) or refbuild.build() is not None


def load():
    global _lib
    if _lib is None:
        from . import refbuild
        path = refbuild.build()
        if path is None:
            raise RuntimeError("reference sources unavailable")
        lib = C.CDLL(path)
        vp, i32, f32 = C.c_void_p, C.c_int, C.c_float
        sigs = {
            "ref_kmeans_cluster": [vp, i32, i32, vp, i32, vp, i32],
            "ref_label_points": [vp, i32, i32, vp, i32, vp],
            "ref_calculate_centroids": [vp, vp, i32, i32, vp, i32],
            "ref_connected_components": [vp, i32, i32, vp, i32],
            "ref_compress_labels": [vp, i32],
            "ref_merge_small_segments": [vp, vp, i32, i32, i32],
            "ref_erode": [vp, i32, i32, i32],
            "ref_segment_adjacency_edges": [vp, i32, i32, vp],
            "ref_segment_adjacency": [vp, i32, i32, vp, vp],
            "ref_sobel_normals": [vp, i32, i32, f32, vp],
            "ref_propagate_centroids": [vp, i32, vp, i32, i32, vp],
            "ref_rgb_to_lab": [vp, i32, vp],
        }
        for name, args in sigs.items():
            fn = getattr(lib, name)
            fn.restype = i32
            fn.argtypes = args
        _lib = lib
    return _lib


def _p(a):
    return C.c_void_p(a.ctypes.data)


def kmeans_cluster(points, centroids, iters):
    p = np.ascontiguousarray(points, np.float32)
    c = np.ascontiguousarray(centroids, np.float32).copy()
    lab = np.empty(p.shape[1], np.int32)
    load().ref_kmeans_cluster(_p(p), p.shape[0], p.shape[1], _p(c), c.shape[1], _p(lab), iters)
    return lab, c


def kmeans_cluster_threshold(points, centroids, max_iter, threshold):
    """cluster(..., max_iter, threshold) (cluster.cu:27-93).  Returns (labels,
    centroids, iterations, shifts): the reference prints each iteration's
    centroid shift and, at the end, its iteration count (cluster.cu:88-92);
    both are read back from its stdout."""
    import re
    import tempfile
    p = np.ascontiguousarray(points, np.float32)
    c = np.ascontiguousarray(centroids, np.float32).copy()
    lab = np.empty(p.shape[1], np.int32)
    lib = load()
    lib.ref_kmeans_cluster_threshold.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                                 C.c_int, C.c_void_p, C.c_int, C.c_float]
    lib.ref_kmeans_cluster_threshold.restype = C.c_int
    with tempfile.TemporaryFile(mode="w+") as f:
        with capture(f.fileno()):
            lib.ref_kmeans_cluster_threshold(_p(p), p.shape[0], p.shape[1], _p(c), c.shape[1],
                                             _p(lab), int(max_iter), float(threshold))
        f.seek(0)
        text = f.read()
    m = re.search(r"in (\d+) iterations", text)
    if not m:
        raise RuntimeError("the reference did not report its iteration count")
    shifts = [float(x) for x in re.findall(r"^([-+0-9.eE]+)$", text, re.M)]
    return lab, c, int(m.group(1)), shifts


def label_points(points, centroids):
    p = np.ascontiguousarray(points, np.float32)
    c = np.ascontiguousarray(centroids, np.float32)
    lab = np.empty(p.shape[1], np.int32)
    load().ref_label_points(_p(p), p.shape[0], p.shape[1], _p(c), c.shape[1], _p(lab))
    return lab


def calculate_centroids(labels, points, k):
    p = np.ascontiguousarray(points, np.float32)
    lab = np.ascontiguousarray(labels, np.int32)
    c = np.zeros((p.shape[0], k), np.float32)
    load().ref_calculate_centroids(_p(lab), _p(p), p.shape[0], p.shape[1], _p(c), k)
    return c


def connected_components(labels, max_iter=100000):
    a = np.ascontiguousarray(labels, np.int32)
    h, w = a.shape
    out = np.empty(a.size, np.int32)
    load().ref_connected_components(_p(a), w, h, _p(out), max_iter)
    return out.reshape(h, w)


def compress_labels(labels):
    a = np.ascontiguousarray(labels, np.int32).copy()
    n = load().ref_compress_labels(_p(a), a.size)
    return a, n


def merge_small_segments(chroma, labels, P):
    ch = np.ascontiguousarray(chroma, np.float32)
    a = np.ascontiguousarray(labels, np.int32).copy()
    h, w = a.shape
    load().ref_merge_small_segments(_p(ch), _p(a), w, h, P)
    return a


def merge_smooth_boundaries(points, labels, nsegments, threshold=0.01):
    """merge_smooth_boundaries (merge_smooth_boundaries.cu:134-243): points
    planar (3, N) float32, labels (H, W) compressed to [0, nsegments)."""
    p = np.ascontiguousarray(points, np.float32)
    a = np.ascontiguousarray(labels, np.int32).copy()
    h, w = a.shape
    lib = load()
    lib.ref_merge_smooth_boundaries.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                                C.c_int, C.c_float]
    lib.ref_merge_smooth_boundaries.restype = C.c_int
    with quiet():
        lib.ref_merge_smooth_boundaries(_p(p), _p(a), w, h, int(nsegments), float(threshold))
    return a


def segment_adjacency_edges(labels):
    """segment_adjacency_edges (segment_adjacency.cu:170-254): (sources,
    targets) of the reference's own edge list."""
    a = np.ascontiguousarray(labels, np.int32)
    h, w = a.shape
    out = np.zeros(16 * a.size, np.int32)
    m = load().ref_segment_adjacency_edges(_p(a), w, h, _p(out))
    return out[:m].copy(), out[m:2 * m].copy()


def segment_adjacency(labels):
    """segment_adjacency (segment_adjacency.cu:256-289): (keys, adjacency) of
    the reference's distinct sorted label pairs."""
    a = np.ascontiguousarray(labels, np.int32)
    h, w = a.shape
    k = np.zeros(8 * a.size, np.int32)
    v = np.zeros(8 * a.size, np.int32)
    m = load().ref_segment_adjacency(_p(a), w, h, _p(k), _p(v))
    return k[:m].copy(), v[:m].copy()


def erode(labels, niter=1):
    a = np.ascontiguousarray(labels, np.int32).copy()
    h, w = a.shape
    load().ref_erode(_p(a), w, h, niter)
    return a


def sobel_normals(heights, depth=1.0):
    hgt = np.ascontiguousarray(heights, np.float32)
    h, w = hgt.shape
    out = np.empty((3, h * w), np.float32)
    load().ref_sobel_normals(_p(hgt), w, h, depth, _p(out))
    return out


def propagate_centroids(labels, centroids):
    lab = np.ascontiguousarray(labels, np.int32)
    c = np.ascontiguousarray(centroids, np.float32)
    out = np.empty((c.shape[0], lab.size), np.float32)
    load().ref_propagate_centroids(_p(lab), lab.size, _p(c), c.shape[0], c.shape[1], _p(out))
    return out


def rgb_to_lab(rgb_planar):
    """(3, N) float RGB in [0, 1] -> (3, N) L*a*b* (conversion.inl:88-92)."""
    a = np.ascontiguousarray(rgb_planar, np.float32)
    out = np.empty_like(a)
    load().ref_rgb_to_lab(_p(a), a.shape[1], _p(out))
    return out


def rgb_to_ic(rgb_planar):
    """The sample's (intensity, r / i, g / i) planes: (3, N) RGB in [0, 1] ->
    (3, N) (main.cu:169-179; conversion.inl:99-108)."""
    a = np.ascontiguousarray(rgb_planar, np.float32)
    out = np.empty_like(a)
    lib = load()
    lib.ref_rgb_to_ic.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    lib.ref_rgb_to_ic.restype = C.c_int
    lib.ref_rgb_to_ic(_p(a), a.shape[1], _p(out))
    return out


def lab_beta(rgb_planar, mu=1e5):
    """The sample's features: (3, N) RGB in [0, 1] -> ((3, N) beta, a*, b*;
    (N,) L*)  (main.cu:169-173, :215-225; beta_feature.cu:47-78)."""
    a = np.ascontiguousarray(rgb_planar, np.float32)
    n = a.shape[1]
    feats = np.empty_like(a)
    lum = np.empty(n, np.float32)
    lib = load()
    lib.ref_lab_beta.argtypes = [C.c_void_p, C.c_int, C.c_float, C.c_void_p, C.c_void_p]
    lib.ref_lab_beta.restype = C.c_int
    lib.ref_lab_beta(_p(a), n, float(mu), _p(feats), _p(lum))
    return feats, lum


class capture:
    """Sends the process's stdout (file descriptor 1) to another descriptor
    for the duration of a block: the reference's progress prints."""

    def __init__(self, fd: int):
        self.fd = fd

    def __enter__(self):
        import sys
        sys.stdout.flush()
        self._saved = os.dup(1)
        os.dup2(self.fd, 1)
        return self

    def __exit__(self, *exc):
        libc = C.CDLL(None)
        libc.fflush(None)
        os.dup2(self._saved, 1)
        os.close(self._saved)


class quiet:
    """Silences the reference's progress prints (std::cout / printf) on the
    process's stdout for the duration of a block."""

    def __enter__(self):
        import sys
        sys.stdout.flush()
        self._fd = os.dup(1)
        self._null = os.open(os.devnull, os.O_WRONLY)
        os.dup2(self._null, 1)
        return self

    def __exit__(self, *exc):
        libc = C.CDLL(None)
        libc.fflush(None)
        os.dup2(self._fd, 1)
        os.close(self._fd)
        os.close(self._null)
