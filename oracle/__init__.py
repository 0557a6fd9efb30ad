"""ORACLE - test infrastructure only.

numpy wrappers over oracle/oracle.c, the CPU restatement of the reference's
segmentation hot path (see that file for the per-function reference
citations).  Imported by tests/, by __graft_entry__.smoke() and by bench.py's
cpu_baseline leg as the checker; the product library never uses it.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None


def _load():
    global _lib
    if _lib is None:
        import sys
        sys.path.insert(0, os.path.dirname(_HERE))
        from split_gb300 import build as b
        path = b.build_oracle()
        lib = C.CDLL(path)
        vp, i32, i64, f32 = C.c_void_p, C.c_int, C.c_int64, C.c_float
        sigs = {
            "orc_kmeans_assign_f32": (None, [vp, i32, i64, vp, i32, vp]),
            "orc_kmeans_assign_f64": (None, [vp, i32, i64, vp, i32, vp, vp, vp]),
            "orc_kmeans_update_f64": (None, [vp, vp, i32, i64, vp, i32, vp, vp]),
            "orc_ccl": (i32, [vp, i32, i32, i32, i32, vp]),
            "orc_compress_labels": (i64, [vp, i64]),
            "orc_merge_small": (i32, [vp, i32, i32, i32, i32, vp, vp]),
            "orc_erode": (i32, [vp, i32, i32, i32, vp]),
            "orc_sobel_normals_f64": (i32, [vp, i32, i32, f32, vp]),
            "orc_luminance_f64": (None, [vp, i64, vp]),
        }
        for name, (res, args) in sigs.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def kmeans_assign_f32(points: np.ndarray, centroids: np.ndarray) -> np.ndarray:
    """points (D, N), centroids (D, K) float32 -> labels (N,) int32."""
    p, c = _c(points, np.float32), _c(centroids, np.float32)
    out = np.empty(p.shape[1], dtype=np.int32)
    _load().orc_kmeans_assign_f32(_p(p), p.shape[0], p.shape[1], _p(c), c.shape[1], _p(out))
    return out


def kmeans_assign_f64(points: np.ndarray, centroids: np.ndarray):
    """-> (labels, best distance, second-best distance) in FP64."""
    p, c = _c(points, np.float32), _c(centroids, np.float32)
    n = p.shape[1]
    lab = np.empty(n, dtype=np.int32)
    d1 = np.empty(n, dtype=np.float64)
    d2 = np.empty(n, dtype=np.float64)
    _load().orc_kmeans_assign_f64(_p(p), p.shape[0], n, _p(c), c.shape[1], _p(lab), _p(d1),
                                  _p(d2))
    return lab, d1, d2


def kmeans_update_f64(labels: np.ndarray, points: np.ndarray, centroids_in: np.ndarray):
    """-> (centroids (D, K) float64, counts (K,) int64); empty clusters keep
    their input centroid."""
    lab, p, c = _c(labels, np.int32), _c(points, np.float32), _c(centroids_in, np.float32)
    d, k = c.shape
    out = np.empty((d, k), dtype=np.float64)
    cnt = np.empty(k, dtype=np.int64)
    _load().orc_kmeans_update_f64(_p(lab), _p(p), d, p.shape[1], _p(c), k, _p(out), _p(cnt))
    return out, cnt


def ccl(labels: np.ndarray, connectivity: int = 4, convention: int = 0) -> np.ndarray:
    """(H, W) int32 -> (H, W) int32 component labels (0: min index, 1: max)."""
    a = _c(labels, np.int32)
    h, w = a.shape
    out = np.empty_like(a)
    rc = _load().orc_ccl(_p(a), w, h, connectivity, convention, _p(out))
    if rc:
        raise RuntimeError(f"orc_ccl failed ({rc})")
    return out


def compress_labels(labels: np.ndarray):
    a = _c(labels, np.int32).copy()
    n = _load().orc_compress_labels(_p(a), a.size)
    return a, int(n)


def merge_small(labels: np.ndarray, P: int, policy: int = 0,
                chroma: np.ndarray | None = None) -> np.ndarray:
    """(H, W) segment ids in [0, H*W) -> merged ids (policy 0 most boundary,
    1 reference chroma on chroma row 0)."""
    a = _c(labels, np.int32)
    h, w = a.shape
    ch = None if chroma is None else _c(chroma, np.float32).reshape(-1)
    out = np.empty_like(a)
    rc = _load().orc_merge_small(_p(a), w, h, P, policy, _p(ch), _p(out))
    if rc:
        raise RuntimeError(f"orc_merge_small failed ({rc})")
    return out


def erode(labels: np.ndarray, radius: int = 1) -> np.ndarray:
    a = _c(labels, np.int32)
    h, w = a.shape
    out = np.empty_like(a)
    rc = _load().orc_erode(_p(a), w, h, radius, _p(out))
    if rc:
        raise RuntimeError(f"orc_erode failed ({rc})")
    return out


def sobel_normals_f64(heights: np.ndarray, depth: float = 1.0) -> np.ndarray:
    """(H, W) float32 -> (3, H*W) float64 normals."""
    a = _c(heights, np.float32)
    h, w = a.shape
    out = np.empty((3, h * w), dtype=np.float64)
    _load().orc_sobel_normals_f64(_p(a), w, h, depth, _p(out))
    return out


def luminance_f64(rgb: np.ndarray) -> np.ndarray:
    """RGB8 (..., 3) -> L*/100 (N,) float64."""
    a = _c(rgb, np.uint8)
    n = a.size // 3
    out = np.empty(n, dtype=np.float64)
    _load().orc_luminance_f64(_p(a), n, _p(out))
    return out


def canonical(labels: np.ndarray) -> np.ndarray:
    """Relabel a partition by the minimum linear index of each label class."""
    flat = np.asarray(labels).reshape(-1)
    _, first, inv = np.unique(flat, return_index=True, return_inverse=True)
    return first[inv].reshape(np.asarray(labels).shape).astype(np.int64)


def merge_smooth(labels: np.ndarray, points: np.ndarray, threshold: float = 0.01) -> np.ndarray:
    """(H, W) int32 segment ids in [0, H*W), planar (>= 3, H*W) float32
    features -> merged labels (smooth-boundary rule)."""
    a = _c(labels, np.int32).copy()
    p = _c(points, np.float32)
    h, w = a.shape
    lib = _load()
    lib.orc_merge_smooth.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_float]
    lib.orc_merge_smooth.restype = C.c_int
    rc = lib.orc_merge_smooth(_p(a), w, h, _p(p), float(threshold))
    if rc:
        raise RuntimeError(f"orc_merge_smooth failed ({rc})")
    return a


def rgb_to_ic_f32(rgb: np.ndarray) -> np.ndarray:
    """The sample's intensity / chroma planes in FP32, operation for operation
    (samples/src/main.cu:169-179; conversion.inl:99-108): RGB8 (..., 3) ->
    channels byte / 255 clamped to >= 1/255 -> intensity = (r + g + b) *
    (1/3), ri = 1 / intensity, (intensity, r * ri, g * ri).  Returns (3, N)
    float32; every step is one IEEE single operation, so the result is exact."""
    f32 = np.float32
    v = np.asarray(rgb, np.uint8).reshape(-1, 3).astype(f32) / f32(255.0)
    v = np.maximum(v, f32(1.0) / f32(255.0))
    r, g, b = v[:, 0], v[:, 1], v[:, 2]
    third = f32(1.0) / f32(3.0)
    inten = ((r + g) + b) * third
    ri = f32(1.0) / inten
    return np.stack([inten, r * ri, g * ri]).astype(f32)


def lab_beta_f64(rgb: np.ndarray, mu: float = 1e5):
    """The sample's features in FP64 (samples/src/main.cu:169-173, :215-225):
    RGB8 (..., 3) -> channels / 255 clamped to >= 1/255 -> sRGB linearised
    (conversion.inl:15-20) -> XYZ (:22-24) -> L*a*b* (:46-64) -> beta in
    place of L* (beta_feature.cu:26-78: lambda = 0.2 max |a*|, bounds 0.2
    and 0.95 of the largest L*).  Returns ((3, N) beta, a*, b*; (N,) L*)."""
    v = np.maximum(np.asarray(rgb, np.float64).reshape(-1, 3) / 255.0, 1.0 / 255.0)
    lin = np.where(v > 0.04045, ((v + 0.055) / 1.055) ** 2.4, v / 12.92) * 100.0
    m = np.array([[0.4124564, 0.3575761, 0.1804375],
                  [0.2126729, 0.7151522, 0.0721750],
                  [0.0193339, 0.1191920, 0.9503041]])
    xyz = lin @ m.T
    t = xyz / np.array([95.047, 100.0, 108.883])
    f = np.where(t > 0.008856, np.cbrt(t), 7.787 * t + 16.0 / 116.0)
    L = 116.0 * f[:, 1] - 16.0
    a = 500.0 * (f[:, 0] - f[:, 1])
    b = 200.0 * (f[:, 1] - f[:, 2])
    lam = 0.2 * np.abs(a).max()
    lo, hi = 0.2 * L.max(), 0.95 * L.max()
    achrom = (np.abs(a) < lam) & (np.abs(b) < lam)
    beta = np.where(achrom & (L < lo), -mu, np.where(achrom & (L > hi), mu, 0.0))
    return np.stack([beta, a, b]), L


def estimate_normals_rb(intensity: np.ndarray, light, smoothness: float, max_iter: int = 1500,
                        tol: float = 1e-5):
    """Shape-from-shading normals (split/src/split/device/sfs/estimate_normals.cu:251-308)
    in FP64: the system (L L^T (x) I + 2 smoothness * B (x) I3) x = intensity * L
    (B: 5-point Poisson matrix, diagonal 4 - [row on border] - [column on border],
    estimate_normals.cu:124-171) relaxed from x = (0, 0, 1) by red-black block
    Gauss-Seidel sweeps (each pixel's 3 x 3 block c I + L L^T solved exactly)
    until |b - A x| <= tol |b| or max_iter sweeps, then normalised with z >= 0.
    The system is singular (constant fields perpendicular to L are free), so
    the converged normals depend on the relaxation order: this restates the
    order the CUDA path uses.  Returns ((3, N) normals, sweeps)."""
    s = np.asarray(intensity, np.float64)
    h, w = s.shape
    L = np.asarray(light, np.float64)
    L = L / np.sqrt((L * L).sum())
    lam2 = 2.0 * smoothness
    rr, cc = np.mgrid[0:h, 0:w]
    val = 4.0 - ((rr == 0) | (rr == h - 1)) - ((cc == 0) | (cc == w - 1))
    x = np.zeros((3, h, w))
    x[2] = 1.0

    def nsum(x):
        S = np.zeros_like(x)
        S[:, 1:, :] += x[:, :-1, :]
        S[:, :-1, :] += x[:, 1:, :]
        S[:, :, 1:] += x[:, :, :-1]
        S[:, :, :-1] += x[:, :, 1:]
        return S

    b = L[:, None, None] * s[None]
    bn = np.sqrt((b * b).sum())
    colour = (rr + cc) & 1
    it = 0
    while True:
        S = nsum(x)
        lx = (L[:, None, None] * x).sum(0)
        ax = L[:, None, None] * lx[None] + lam2 * (val[None] * x - S)
        r = b - ax
        if np.sqrt((r * r).sum()) <= tol * bn or it >= max_iter:
            break
        for c in (0, 1):
            S = nsum(x)
            rv = b + lam2 * S
            cdiag = lam2 * val
            q = (L[:, None, None] * rv).sum(0) / (cdiag + 1.0)
            new = (rv - L[:, None, None] * q[None]) / cdiag[None]
            m = colour == c
            x[:, m] = new[:, m]
        it += 1
    n = np.sqrt((x * x).sum(0))
    out = np.stack([x[0] / n, x[1] / n, np.abs(x[2]) / n]).reshape(3, -1)
    return out, it


def reference_shift(points: np.ndarray, c_old: np.ndarray, c_new: np.ndarray,
                    counts: np.ndarray) -> float:
    """The centroid shift as the reference's cluster() measures it, in FP32
    (split/src/split/device/kmeans/cluster.cu:40-50, :73-87).  Its previous
    centroids sit at float offset 2N of the workspace, which label_points
    (label.cu:80-88: N x K distances, entry i * K + c) and calculate_centroids
    (centroids.cu:40-63: K reciprocal cluster sizes at offset 2N) overwrite in
    the same iteration.  The new centroids (planar 3 x K, entry j = d * K + k)
    are therefore compared with 1 / n_j for j < K and with the distance of
    point (2N + j) // K to input centroid (2N + j) % K (Norm2, label.cu:23-32)
    for j >= K; the squares are summed in j order."""
    f32 = np.float32
    p = np.asarray(points, f32)
    n = p.shape[1]
    k = c_new.shape[1]
    acc = f32(0.0)
    for j in range(3 * k):
        if j < k:
            word = f32(1.0) / f32(counts[j])
        else:
            e = 2 * n + j
            px, c = e // k, e % k
            a = [f32(p[d, px]) - f32(c_old[d, c]) for d in range(3)]
            word = (a[0] * a[0] + a[1] * a[1]) + a[2] * a[2]
        t = f32(c_new[j // k, j % k]) - f32(word)
        acc = f32(acc + t * t)
    return float(np.sqrt(acc, dtype=f32))


def kmeans_cluster_threshold(points: np.ndarray, c0: np.ndarray, max_iter: int,
                             threshold: float, reference_shift_rule: bool = True):
    """cluster(points, c0, max_iter, threshold) (cluster.cu:27-93): FP32-exact
    assignments and FP64 updates (rounded to FP32) until max_iter iterations
    or |delta - old_delta| <= threshold, delta = 0 and old_delta = threshold
    + 1 at the start (:65-71).  With reference_shift_rule the shift is
    reference_shift(); otherwise the L2 change of the centroid matrix.
    Returns (labels, centroids, iterations, shifts)."""
    p = np.asarray(points, np.float32)
    c = np.asarray(c0, np.float32).copy()
    delta, old_delta = np.float32(0.0), np.float32(threshold) + np.float32(1.0)
    it, shifts, lab = 0, [], None
    while it < max_iter and abs(float(delta) - float(old_delta)) > threshold:
        it += 1
        lab = kmeans_assign_f32(p, c)
        c64, cnt = kmeans_update_f64(lab, p, c)
        cn = c64.astype(np.float32)
        old_delta = delta
        if reference_shift_rule:
            delta = np.float32(reference_shift(p, c, cn, cnt))
        else:
            delta = np.float32(np.sqrt(np.sum((cn - c).astype(np.float64) ** 2)))
        shifts.append(float(delta))
        c = cn
    return lab, c, it, shifts


def propagate_centroids(labels: np.ndarray, centroids: np.ndarray) -> np.ndarray:
    """out[:, i] = centroids[:, labels[i]] (propagation.cu:9-24: a gather of
    the centroid columns by label).  Returns (D, N) float32."""
    c = np.asarray(centroids, np.float32)
    return np.ascontiguousarray(c[:, np.asarray(labels).reshape(-1)])


# 8-neighbourhood in the order of NeighbourKeys (segment_adjacency.cu:112-142)
_NEIGHBOURS = ((-1, -1), (0, -1), (1, -1), (-1, 0), (1, 0), (-1, 1), (0, 1), (1, 1))


def segment_adjacency_edges(labels: np.ndarray):
    """segment_adjacency_edges (segment_adjacency.cu:170-254): for every pixel
    i in index order and every in-image neighbour j in the order NW, N, NE,
    W, E, SW, S, SE with a different label, the edge (i, j).  Returns the
    (sources, targets) arrays."""
    lab = np.ascontiguousarray(labels, np.int32)
    h, w = lab.shape
    flat = lab.ravel()
    idx = np.arange(h * w, dtype=np.int64)
    x, y = idx % w, idx // w
    tgt = np.full((h * w, 8), -1, np.int64)
    for d, (dx, dy) in enumerate(_NEIGHBOURS):
        nx, ny = x + dx, y + dy
        ok = (nx >= 0) & (nx < w) & (ny >= 0) & (ny < h)
        tgt[ok, d] = (ny * w + nx)[ok]
    src = np.repeat(idx, 8)
    tgt = tgt.ravel()
    keep = tgt >= 0
    keep[keep] = flat[src[keep]] != flat[tgt[keep]]
    return src[keep].astype(np.int32), tgt[keep].astype(np.int32)


def segment_adjacency(labels: np.ndarray):
    """segment_adjacency (segment_adjacency.cu:256-289): the distinct
    (labels[i], labels[j]) pairs of the edges, sorted by key then value.
    Returns the (keys, adjacency) arrays."""
    flat = np.ascontiguousarray(labels, np.int32).ravel()
    s, t = segment_adjacency_edges(labels)
    if s.size == 0:
        return np.zeros(0, np.int32), np.zeros(0, np.int32)
    pairs = np.unique(np.stack([flat[s], flat[t]], axis=1), axis=0)
    return pairs[:, 0].astype(np.int32), pairs[:, 1].astype(np.int32)
