"""Connected components, label compression and small-segment merge, named after
split::device::ccl (split/include/split/device/ccl/*.cuh)."""
from __future__ import annotations

import torch

from . import _native as N
from ._util import Workspace, ensure_workspace, ptr, require_cuda, stream_handle

MIN_INDEX, MAX_INDEX = N.LABEL_MIN_INDEX, N.LABEL_MAX_INDEX
MOST_BOUNDARY, REF_CHROMA = N.MERGE_MOST_BOUNDARY, N.MERGE_REF_CHROMA


def connected_components_workspace(width: int, height: int) -> int:
    return N.load().split_ccl_workspace_size(width, height)


def connected_components(labels: torch.Tensor, temp: Workspace | None, out: torch.Tensor,
                         max_iterations: int = 10, *, connectivity: int = 4,
                         convention: int = MAX_INDEX, sizes: torch.Tensor | None = None,
                         stream=None) -> Workspace:
    """split::device::ccl::connected_components (connected_components.cuh:25-29).

    labels: (H, W) int32 cluster labels; out: H*W int32 segment labels.  The
    default convention reproduces the reference's converged labels (maximum
    linear index per 4-connected component).  Union-find always converges, so
    ``max_iterations`` is accepted for signature compatibility only.
    """
    del max_iterations
    require_cuda(labels, "labels", torch.int32)
    require_cuda(out, "out", torch.int32)
    if labels.dim() != 2:
        raise ValueError("labels must be (height, width)")
    h, w = labels.shape
    if out.numel() != h * w:
        raise ValueError("out must hold one entry per pixel")
    ws = ensure_workspace(temp, connected_components_workspace(w, h), labels.device)
    st = N.load().split_ccl(ptr(labels), w, h, connectivity, convention, ptr(out), ptr(sizes),
                            ws.ptr, ws.nbytes, stream_handle(stream))
    N.check(st, "ccl.connected_components")
    return ws


def compress_labels_workspace(n: int) -> int:
    return N.load().split_compress_labels_workspace_size(n)


def compress_labels(labels: torch.Tensor, temp: Workspace | None = None, *,
                    stream=None) -> int:
    """split::device::ccl::compress_labels (compress_labels.cuh:21-23).

    In place; returns the number of distinct labels (synchronises, as the
    reference's return value does).  Labels must lie in [-1, n)."""
    require_cuda(labels, "labels", torch.int32)
    n = labels.numel()
    ws = ensure_workspace(temp, compress_labels_workspace(n), labels.device)
    count = torch.zeros(1, dtype=torch.int32, device=labels.device)
    st = N.load().split_compress_labels(ptr(labels), n, ptr(count), ws.ptr, ws.nbytes,
                                        stream_handle(stream))
    N.check(st, "ccl.compress_labels")
    ws.check("ccl.compress_labels", stream)
    return int(count.item())


def segment_adjacency_edges_workspace(width: int, height: int) -> int:
    return N.load().split_segment_adjacency_edges_workspace_size(width, height)


def segment_adjacency_edges(labels: torch.Tensor, edges: torch.Tensor,
                            temp: Workspace | None = None, *, stream=None) -> int:
    """split::device::ccl::segment_adjacency_edges (segment_adjacency.cuh:14-16).

    labels: (H, W) int32; edges: int32 with room for 16 * H * W entries.
    Writes the m edge sources to edges[:m] and their targets to
    edges[m:2m] and returns m (synchronises, as the reference's return value
    does)."""
    require_cuda(labels, "labels", torch.int32)
    require_cuda(edges, "edges", torch.int32)
    if labels.dim() != 2:
        raise ValueError("labels must be (height, width)")
    h, w = labels.shape
    if edges.numel() < 16 * h * w:
        raise ValueError("edges must hold 16 entries per pixel")
    ws = ensure_workspace(temp, segment_adjacency_edges_workspace(w, h), labels.device)
    count = torch.zeros(1, dtype=torch.int32, device=labels.device)
    st = N.load().split_segment_adjacency_edges(ptr(labels), w, h, ptr(edges), ptr(count),
                                                ws.ptr, ws.nbytes, stream_handle(stream))
    N.check(st, "ccl.segment_adjacency_edges")
    ws.check("ccl.segment_adjacency_edges", stream)
    return int(count.item())


def segment_adjacency_workspace(width: int, height: int) -> int:
    return N.load().split_segment_adjacency_workspace_size(width, height)


def segment_adjacency(labels: torch.Tensor, keys: torch.Tensor, adjacency: torch.Tensor,
                      temp: Workspace | None = None, *, stream=None) -> int:
    """split::device::ccl::segment_adjacency (segment_adjacency.cuh:21-24).

    labels: (H, W) int32; keys, adjacency: int32 with room for 8 * H * W
    entries each.  Writes the distinct (label, neighbouring label) pairs,
    sorted by key then value, and returns their number (synchronises)."""
    require_cuda(labels, "labels", torch.int32)
    require_cuda(keys, "keys", torch.int32)
    require_cuda(adjacency, "adjacency", torch.int32)
    if labels.dim() != 2:
        raise ValueError("labels must be (height, width)")
    h, w = labels.shape
    if keys.numel() < 8 * h * w or adjacency.numel() < 8 * h * w:
        raise ValueError("keys and adjacency must hold 8 entries per pixel")
    ws = ensure_workspace(temp, segment_adjacency_workspace(w, h), labels.device)
    count = torch.zeros(1, dtype=torch.int32, device=labels.device)
    st = N.load().split_segment_adjacency(ptr(labels), w, h, ptr(keys), ptr(adjacency),
                                          ptr(count), ws.ptr, ws.nbytes, stream_handle(stream))
    N.check(st, "ccl.segment_adjacency")
    ws.check("ccl.segment_adjacency", stream)
    return int(count.item())


def merge_small_segments_workspace(width: int, height: int) -> int:
    return N.load().split_merge_small_workspace_size(width, height)


def merge_small_segments(chrominance: torch.Tensor | None, labels: torch.Tensor,
                         temp: Workspace | None = None, P: int = 10, *,
                         policy: int = REF_CHROMA, sizes: torch.Tensor | None = None,
                         stream=None) -> Workspace:
    """split::device::ccl::merge_small_segments (merge_small_segments.cuh:15-19).

    labels: (H, W) int32 segment ids in [0, H*W), relabelled in place.
    policy REF_CHROMA (default, the reference's rule) reads chrominance
    (2, H*W) float32 row 0; MOST_BOUNDARY needs no chrominance."""
    require_cuda(labels, "labels", torch.int32)
    if labels.dim() != 2:
        raise ValueError("labels must be (height, width)")
    h, w = labels.shape
    if chrominance is not None:
        require_cuda(chrominance, "chrominance", torch.float32)
    ws = ensure_workspace(temp, merge_small_segments_workspace(w, h), labels.device)
    st = N.load().split_merge_small(ptr(labels), w, h, P, policy, ptr(chrominance), ptr(sizes),
                                    ws.ptr, ws.nbytes, stream_handle(stream))
    N.check(st, "ccl.merge_small_segments")
    return ws


def merge_smooth_boundaries_workspace(width: int, height: int) -> int:
    """merge_smooth_boundaries.cuh:29-31 (sized by the image; the segment and
    edge counts are not needed)."""
    return N.load().split_merge_smooth_workspace_size(width, height)


def merge_smooth_boundaries(points: torch.Tensor, nsegments: int, labels: torch.Tensor,
                            temp: Workspace | None = None, threshold: float = 0.01, *,
                            stream=None) -> Workspace:
    """split::device::ccl::merge_smooth_boundaries (merge_smooth_boundaries.cuh:20-25).

    points: planar float32 (>= 3, H*W) features (rows 0..2 are read);
    labels: (H, W) int32 segment ids in [0, H*W), merged in place.  Segments
    join the neighbour with the smallest mean feature difference across
    their boundary, among neighbours sharing more than 15 boundary edges with
    a mean below threshold * max |x|.  ``nsegments`` is accepted for
    signature compatibility; ids need not be compressed."""
    del nsegments
    require_cuda(points, "points", torch.float32)
    require_cuda(labels, "labels", torch.int32)
    if labels.dim() != 2:
        raise ValueError("labels must be (height, width)")
    h, w = labels.shape
    if points.dim() != 2 or points.shape[0] < 3 or points.shape[1] != h * w:
        raise ValueError("points must be a planar (>= 3, height * width) tensor")
    ws = ensure_workspace(temp, merge_smooth_boundaries_workspace(w, h), labels.device)
    st = N.load().split_merge_smooth(ptr(labels), w, h, ptr(points), float(threshold), ws.ptr,
                                     ws.nbytes, stream_handle(stream))
    N.check(st, "ccl.merge_smooth_boundaries")
    return ws
