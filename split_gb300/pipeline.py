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

    def capture(self, rgb: torch.Tensor):
        """Capture one run on `rgb` into a CUDA graph; replay() then reruns it
        on whatever that buffer and self.centroids hold (copy the next frame
        and its initial centroids in first).  The graph replaces the launch
        sequence's host work and launch gaps."""
        require_cuda(rgb, "rgb", torch.uint8)
        torch.cuda.synchronize(self.device)
        s = torch.cuda.Stream(self.device)
        c0 = self.centroids.clone()
        with torch.cuda.stream(s):
            self.run(rgb, stream=s)        # warm the launch path outside capture
        s.synchronize()
        self.centroids.copy_(c0)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            self.run(rgb, stream=torch.cuda.current_stream())
        self.graph = g
        self._graph_rgb = rgb
        return g

    def replay(self) -> None:
        self.graph.replay()


def launch_count() -> int:
    return int(N.load().split_launch_count())


class HostPipeline:
    """Frames from pinned host memory through the pipeline, with the copies
    overlapped with compute.

    `depth` resident pipelines (slots) take frames in turn.  Uploads, compute
    and downloads run on three CUDA streams joined by events:
      * a slot's upload waits until the slot's previous frame has been
        computed (input buffer free) and downloaded (the centroid buffer is
        both the initial-centroid input and the result);
      * its compute waits for the upload, and for the previous download (the
        output buffers are rewritten);
      * its download waits for the compute.
    So frame f's compute overlaps frame f-1's download and frame f+1's
    upload, and no result is overwritten before it has reached the host.
    With `graphs` (default), each slot's launch sequence is captured once into
    a CUDA graph and every frame replays it.  submit() returns at once;
    wait(ticket) blocks until that frame is in the host buffers given to
    submit()."""

    def __init__(self, width: int, height: int, params: Params, device=None, depth: int = 2,
                 graphs: bool = True):
        if depth < 1:
            raise ValueError("depth must be at least 1")
        self.width, self.height, self.params = width, height, params
        self.slots = [Pipeline(width, height, params, device) for _ in range(depth)]
        self.device = self.slots[0].device
        self.d_rgb = [torch.empty(height * width * 3, dtype=torch.uint8, device=self.device)
                      for _ in range(depth)]
        self.upload, self.compute, self.download = (torch.cuda.Stream(self.device)
                                                    for _ in range(3))
        self._uploaded = [torch.cuda.Event() for _ in range(depth)]
        self._computed = [torch.cuda.Event() for _ in range(depth)]
        self._downloaded = [torch.cuda.Event() for _ in range(depth)]
        self._frame_of_slot = [-1] * depth
        self.frames = 0
        self.graphs = graphs
        if graphs:
            for pipe, buf in zip(self.slots, self.d_rgb):
                buf.zero_()
                pipe.centroids.zero_()
                pipe.capture(buf)

    def submit(self, rgb: torch.Tensor, centroids: torch.Tensor,
               segment_labels: torch.Tensor, normals: torch.Tensor | None = None,
               centroids_out: torch.Tensor | None = None,
               cluster_labels: torch.Tensor | None = None) -> int:
        """Enqueue one frame.  rgb: pinned uint8 H*W*3; centroids: pinned
        (dim, K) initial centroids; outputs: pinned host tensors of the
        pipeline's shapes (segment labels (H, W) int32, normals (3, H*W)
        float32, centroids (dim, K), cluster labels H*W int32)."""
        for name, t in (("rgb", rgb), ("centroids", centroids), ("segment_labels", segment_labels),
                        ("normals", normals), ("centroids_out", centroids_out),
                        ("cluster_labels", cluster_labels)):
            if t is not None and (t.is_cuda or not t.is_pinned()):
                raise ValueError(f"{name}: expected a pinned host tensor")
        if normals is not None and self.slots[0].normals is None:
            raise ValueError("normals requested but the parameters compute none")
        s = self.frames % len(self.slots)
        pipe = self.slots[s]
        busy = self._frame_of_slot[s] >= 0
        with torch.cuda.stream(self.upload):
            if busy:
                self.upload.wait_event(self._computed[s])
                self.upload.wait_event(self._downloaded[s])
            self.d_rgb[s].copy_(rgb.reshape(-1), non_blocking=True)
            pipe.centroids.copy_(centroids, non_blocking=True)
            self._uploaded[s].record(self.upload)
        with torch.cuda.stream(self.compute):
            self.compute.wait_event(self._uploaded[s])
            if busy:
                self.compute.wait_event(self._downloaded[s])
            if self.graphs:
                pipe.replay()
            else:
                pipe.run(self.d_rgb[s], stream=self.compute)
            self._computed[s].record(self.compute)
        with torch.cuda.stream(self.download):
            self.download.wait_event(self._computed[s])
            segment_labels.copy_(pipe.segment_labels, non_blocking=True)
            if normals is not None:
                normals.copy_(pipe.normals, non_blocking=True)
            if centroids_out is not None:
                centroids_out.copy_(pipe.centroids, non_blocking=True)
            if cluster_labels is not None:
                cluster_labels.copy_(pipe.cluster_labels, non_blocking=True)
            self._downloaded[s].record(self.download)
        self._frame_of_slot[s] = self.frames
        self.frames += 1
        return self.frames - 1

    def wait(self, ticket: int) -> None:
        """Block until frame `ticket` has reached its host buffers (a later
        frame of the same slot implies it)."""
        if ticket < 0 or ticket >= self.frames:
            raise ValueError("unknown frame")
        self._downloaded[ticket % len(self.slots)].synchronize()

    def check(self) -> None:
        """Raise if any slot's workspace recorded a device-side error."""
        for p in self.slots:
            p.ws.check("pipeline")
