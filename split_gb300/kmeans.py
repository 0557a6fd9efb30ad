"""k-means entry points, named after split::device::kmeans
(split/include/split/device/kmeans/*.cuh)."""
from __future__ import annotations

import ctypes as C

import torch

from . import _native as N
from ._util import Workspace, ensure_workspace, ptr, require_cuda, stream_handle

PLANAR, FLOAT4, RGB8 = N.LAYOUT_PLANAR, N.LAYOUT_FLOAT4, N.LAYOUT_RGB8
UNIT_RANGE = 0x100  # or into FLOAT4: colour features promised in [0, 1]
# or into the layout of cluster(): the convergence test measures the centroid
# shift as the reference's cluster() does (3-D, K >= 3; see the C header)
REFERENCE_SHIFT = 0x200


def cluster_workspace(npoints: int, nclusters: int, dim: int) -> int:
    """cluster.cuh:46-47."""
    return N.load().split_kmeans_cluster_workspace_size(npoints, nclusters, dim)


def cluster_workspace_2d(npoints: int, width: int, nclusters: int, dim: int) -> int:
    return N.load().split_kmeans_cluster_workspace_size_2d(npoints, width, nclusters, dim)


def label_points_workspace(npoints: int, nclusters: int) -> int:
    """label.cuh:39-40."""
    return N.load().split_kmeans_assign_workspace_size(npoints, nclusters)


def calculate_centroids_workspace(npoints: int, ncentroids: int, dim: int = 3) -> int:
    """centroids.cuh:39-40."""
    return N.load().split_kmeans_update_workspace_size(npoints, ncentroids, dim)


def default_width(n: int) -> int:
    """A feature list without an image behind it is tiled as rows of this
    width (as include/split_gb300.hpp does); pass the image width for 5-D
    features, whose xy come from it."""
    return n if 0 < n < 4096 else (4096 if n > 0 else 1)


def _features(points: torch.Tensor, layout: int, dim: int | None):
    """Returns (npoints, dim) for a points tensor in the given layout."""
    require_cuda(points, "points")
    layout &= ~(UNIT_RANGE | REFERENCE_SHIFT)
    if layout == PLANAR:
        if points.dtype != torch.float32 or points.dim() != 2:
            raise ValueError("planar points must be a float32 (dim, npoints) tensor")
        return points.shape[1], points.shape[0]
    if layout == FLOAT4:
        if points.dtype != torch.float32 or points.shape[-1] != 4:
            raise ValueError("float4 points must be a float32 (..., 4) tensor")
        return points.numel() // 4, dim or 3
    if layout == RGB8:
        if points.dtype != torch.uint8 or points.shape[-1] != 3:
            raise ValueError("rgb8 points must be a uint8 (..., 3) tensor")
        return points.numel() // 3, dim or 3
    raise ValueError(f"unknown layout {layout}")


def cluster(points: torch.Tensor, centroids: torch.Tensor, labels: torch.Tensor,
            temp: Workspace | None = None, max_iter: int = 10, threshold: float = 1.0, *,
            layout: int = PLANAR, dim: int | None = None, width: int | None = None,
            xy_scale: float = 0.1, iterations_out: torch.Tensor | None = None,
            stream=None) -> Workspace:
    """split::device::kmeans::cluster (cluster.cuh:31-37, cluster.cu:27-93).

    points: planar (dim, N) float32, or packed (N, 4) float32 / (N, 3) uint8
    with ``dim`` 3 or 5 (5 adds xy_scale * (column, row) for image ``width``).
    centroids (dim, K) float32 is updated in place; labels (N,) int32 receives
    the final assignment.  Exactly ``max_iter`` iterations when threshold < 0.
    K from 1 to 2**20: up to 64 in one persistent launch, more through the
    many-cluster path.  Returns the workspace used (pass it back in to reuse
    it).
    """
    n, d = _features(points, layout, dim)
    width = default_width(n) if width is None else width
    require_cuda(centroids, "centroids", torch.float32)
    require_cuda(labels, "labels", torch.int32)
    if centroids.dim() != 2 or centroids.shape[0] != d:
        raise ValueError("centroids must be (dim, K)")
    if labels.numel() != n:
        raise ValueError("labels must hold one entry per point")
    k = centroids.shape[1]
    ws = ensure_workspace(temp, cluster_workspace_2d(n, width, k, d), points.device)
    st = N.load().split_kmeans_cluster(
        ptr(points), layout, d, n, width, xy_scale, ptr(centroids), k, ptr(labels), ws.ptr,
        ws.nbytes, max_iter, threshold, ptr(iterations_out), stream_handle(stream))
    N.check(st, "kmeans.cluster")
    return ws


def label_points(centroids: torch.Tensor, points: torch.Tensor, labels: torch.Tensor,
                 temp: Workspace | None = None, *, layout: int = PLANAR, dim: int | None = None,
                 width: int | None = None, xy_scale: float = 0.1, stream=None) -> Workspace:
    """split::device::kmeans::label_points (label.cuh:27-31, label.cu:74-106):
    nearest centroid by the reference's squared distance, ties to the lowest
    index; K from 1 to 2**20."""
    n, d = _features(points, layout, dim)
    width = default_width(n) if width is None else width
    require_cuda(centroids, "centroids", torch.float32)
    require_cuda(labels, "labels", torch.int32)
    k = centroids.shape[1]
    ws = ensure_workspace(temp, cluster_workspace_2d(n, width, k, d), points.device)
    st = N.load().split_kmeans_assign(ptr(points), layout, d, n, width, xy_scale,
                                      ptr(centroids), k, ptr(labels), ws.ptr, ws.nbytes,
                                      stream_handle(stream))
    N.check(st, "kmeans.label_points")
    return ws


def calculate_centroids(labels: torch.Tensor, points: torch.Tensor, centroids: torch.Tensor,
                        temp: Workspace | None = None, *, layout: int = PLANAR,
                        dim: int | None = None, width: int | None = None,
                        xy_scale: float = 0.1,
                        stream=None) -> Workspace:
    """split::device::kmeans::calculate_centroids (centroids.cuh:26-30).

    Any number of clusters: up to 64 through the k-means kernel's update, more
    (segment labels, K = number of segments) through per-cluster fixed-point
    accumulators.  Empty clusters keep their previous centroid (documented
    divergence); labels outside [0, K) are ignored."""
    n, d = _features(points, layout, dim)
    width = default_width(n) if width is None else width
    require_cuda(centroids, "centroids", torch.float32)
    require_cuda(labels, "labels", torch.int32)
    k = centroids.shape[1]
    need = cluster_workspace_2d(n, width, k, d) if k <= 64 else \
        calculate_centroids_workspace(n, k, d)
    ws = ensure_workspace(temp, need, points.device)
    st = N.load().split_kmeans_update(ptr(labels), ptr(points), layout, d, n, width, xy_scale,
                                      ptr(centroids), k, ws.ptr, ws.nbytes,
                                      stream_handle(stream))
    N.check(st, "kmeans.calculate_centroids")
    return ws


def propagate_centroids(labels: torch.Tensor, centroids: torch.Tensor, points: torch.Tensor,
                        stream=None) -> None:
    """split::device::kmeans::propagate_centroids (propagation.cuh:23-26)."""
    require_cuda(labels, "labels", torch.int32)
    require_cuda(centroids, "centroids", torch.float32)
    require_cuda(points, "points", torch.float32)
    d, k = centroids.shape
    st = N.load().split_kmeans_propagate(ptr(labels), labels.numel(), ptr(centroids), k, d,
                                         ptr(points), stream_handle(stream))
    N.check(st, "kmeans.propagate_centroids")
