"""The segmentation path as one call (split_pipeline_run): features ->
k-means -> connected components -> small-segment merge -> erosion, plus
Sobel normals of the luminance plane (samples/src/main.cu:154-314)."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import torch

from . import _native as N
from ._util import Workspace, ptr, require_cuda, stream_handle


@dataclass
class Params:
    nclusters: int = 16
    dim: int = 5
    xy_scale: float = 0.1
    kmeans_iters: int = 20
    kmeans_threshold: float = -1.0
    features: int = N.LAYOUT_FLOAT4
    connectivity: int = 8
    convention: int = N.LABEL_MIN_INDEX
    merge_P: int = 256
    merge_policy: int = N.MERGE_MOST_BOUNDARY
    erode_radius: int = 1
    compute_normals: bool = True
    depth: float = 1.0
    beta_mu: float = 1e5     # features = N.FEATURES_LAB_BETA only

    def c(self) -> N.PipelineParams:
        return N.PipelineParams(self.nclusters, self.dim, self.xy_scale, self.kmeans_iters,
                                self.kmeans_threshold, self.features, self.connectivity,
                                self.convention, self.merge_P, self.merge_policy,
                                self.erode_radius, int(self.compute_normals), self.depth,
                                self.beta_mu)


class Pipeline:
    """Resident buffers + workspace for one image size; run() is asynchronous."""

    def __init__(self, width: int, height: int, params: Params, device=None):
        self.width, self.height, self.params = width, height, params
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None \
            else torch.device(device)
        from . import tune
        tune.ensure_once(self.device)   # this GPU's cached launch choices, if any
        self._cp = params.c()
        nbytes = N.load().split_pipeline_workspace_size(width, height, C.byref(self._cp))
        if nbytes == 0:
            raise ValueError("invalid pipeline parameters")
        self.ws = Workspace(nbytes, self.device)
        n = width * height
        self.cluster_labels = torch.empty(n, dtype=torch.int32, device=self.device)
        self.segment_labels = torch.empty((height, width), dtype=torch.int32, device=self.device)
        self.normals = torch.empty((3, n), dtype=torch.float32, device=self.device) \
            if params.compute_normals else None
        self.centroids = torch.empty((params.dim, params.nclusters), dtype=torch.float32,
                                     device=self.device)

    def run(self, rgb: torch.Tensor, init_centroids: torch.Tensor | None = None,
            stage_events=None, stream=None) -> None:
        require_cuda(rgb, "rgb", torch.uint8)
        if init_centroids is not None:
            self.centroids.copy_(init_centroids, non_blocking=True)
        ev = None
        if stage_events is not None:
            if any(e.cuda_event == 0 for e in stage_events):
                raise ValueError("stage events must have been recorded once (torch creates "
                                 "CUDA events lazily)")
            ev = (C.c_void_p * len(stage_events))(*[e.cuda_event for e in stage_events])
        st = N.load().split_pipeline_run(
            ptr(rgb), self.width, self.height, C.byref(self._cp), ptr(self.centroids),
            ptr(self.cluster_labels), ptr(self.segment_labels), ptr(self.normals), self.ws.ptr,
            self.ws.nbytes, ev, stream_handle(stream))
        N.check(st, "pipeline.run")


def launch_count() -> int:
    return int(N.load().split_launch_count())
