"""Batches of uneven images through the segmentation path (split_batch_*):
one fixed launch sequence for the whole batch, optionally replayed from a
captured CUDA graph."""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _native as N
from ._util import Workspace, ptr, stream_handle
from .pipeline import Params


class Arena:
    """Device buffers that successive batches bind to instead of allocating
    their own (a serving loop keeps one per batch in flight).  Capacities
    grow when a batch needs more; the workspace is zero-filled once, when it
    is (re)allocated."""

    def __init__(self, device, pixels: int = 0, centroid_floats: int = 0,
                 workspace_bytes: int = 0, normals: bool = True):
        self.device = torch.device(device)
        self.normals_enabled = normals
        self.px = self.cf = self.wsb = 0
        self.ensure(pixels, centroid_floats, workspace_bytes)

    def ensure(self, pixels: int, centroid_floats: int, workspace_bytes: int) -> None:
        d = self.device
        if pixels > self.px:
            self.px = pixels
            self.rgb = torch.zeros(pixels * 3, dtype=torch.uint8, device=d)
            self.cluster_labels = torch.zeros(pixels, dtype=torch.int32, device=d)
            self.segment_labels = torch.zeros(pixels, dtype=torch.int32, device=d)
            self.normals = torch.zeros(pixels * 3, dtype=torch.float32, device=d) \
                if self.normals_enabled else None
            self.labels_host = None   # pinned download buffers, made on first use
        if centroid_floats > self.cf:
            self.cf = centroid_floats
            self.centroids = torch.zeros(centroid_floats, dtype=torch.float32, device=d)
            self.centroids_host = None
        if workspace_bytes > self.wsb:
            self.wsb = workspace_bytes
            self.ws_buf = torch.zeros(workspace_bytes + 256, dtype=torch.uint8, device=d)


    def host_buffers(self):
        """Pinned host buffers for downloads of a whole arena (segment labels,
        centroids), made once per capacity: pinning memory takes milliseconds
        and must stay out of a serving loop."""
        if getattr(self, "labels_host", None) is None:
            self.labels_host = torch.empty(self.px, dtype=torch.int32, pin_memory=True)
        if getattr(self, "centroids_host", None) is None:
            self.centroids_host = torch.empty(self.cf, dtype=torch.float32, pin_memory=True)
        return self.labels_host, self.centroids_host


class Batch:
    """Plan + resident arenas for a list of (width, height, K, iterations)."""

    def __init__(self, shapes, params: Params | None = None, device=None, stream=None,
                 arena: Arena | None = None):
        self.params = params or Params()
        self.shapes = [tuple(int(v) for v in s) for s in shapes]
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None \
            else torch.device(device)
        from . import tune
        tune.ensure_once(self.device)   # this GPU's cached launch choices, if any
        arr = (N.BatchImage * len(self.shapes))(*[N.BatchImage(*s) for s in self.shapes])
        h = C.c_void_p()
        cp = self.params.c()
        N.check(N.load().split_batch_create(arr, len(self.shapes), C.byref(cp), C.byref(h)),
                "batch.create")
        self._h = h
        lib = N.load()
        self.arena_px = lib.split_batch_arena_pixels(h)
        self.offsets = [lib.split_batch_pixel_offset(h, i) for i in range(len(self.shapes))]
        self.coffsets = [lib.split_batch_centroid_offset(h, i) for i in range(len(self.shapes))]
        nc = lib.split_batch_centroid_floats(h)
        d = self.device
        wsb = lib.split_batch_workspace_size(h)
        if arena is None:
            self.rgb = torch.zeros(self.arena_px * 3, dtype=torch.uint8, device=d)
            self.centroids = torch.zeros(nc, dtype=torch.float32, device=d)
            self.cluster_labels = torch.zeros(self.arena_px, dtype=torch.int32, device=d)
            self.segment_labels = torch.zeros(self.arena_px, dtype=torch.int32, device=d)
            self.normals = torch.zeros(self.arena_px * 3, dtype=torch.float32, device=d) \
                if self.params.compute_normals else None
            self.ws = Workspace(wsb, d)
        else:
            if self.params.compute_normals and not arena.normals_enabled:
                raise ValueError("the arena holds no normals")
            arena.ensure(self.arena_px, nc, wsb)
            px = self.arena_px
            self.rgb = arena.rgb[:3 * px]
            self.centroids = arena.centroids[:nc]
            self.cluster_labels = arena.cluster_labels[:px]
            self.segment_labels = arena.segment_labels[:px]
            self.normals = arena.normals[:3 * px] if self.params.compute_normals else None
            self.ws = Workspace.over(arena.ws_buf, wsb)
        N.check(lib.split_batch_bind(h, ptr(self.rgb), ptr(self.centroids),
                                     ptr(self.cluster_labels), ptr(self.segment_labels),
                                     ptr(self.normals), self.ws.ptr, self.ws.nbytes,
                                     stream_handle(stream)), "batch.bind")
        self.graph = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            N.load().split_batch_destroy(h)
            self._h = None

    # ---- arena views
    def npx(self, i):
        w, h = self.shapes[i][:2]
        return w * h

    def rgb_of(self, i):
        w, h = self.shapes[i][:2]
        o = self.offsets[i]
        return self.rgb[3 * o:3 * (o + w * h)].view(h, w, 3)

    def centroids_of(self, i):
        k = self.shapes[i][2]
        o = self.coffsets[i]
        return self.centroids[o:o + self.params.dim * k].view(self.params.dim, k)

    def cluster_labels_of(self, i):
        o = self.offsets[i]
        return self.cluster_labels[o:o + self.npx(i)]

    def segment_labels_of(self, i):
        w, h = self.shapes[i][:2]
        o = self.offsets[i]
        return self.segment_labels[o:o + w * h].view(h, w)

    def normals_of(self, i):
        n = self.npx(i)
        o = 3 * self.offsets[i]
        return self.normals[o:o + 3 * n].view(3, n)

    def load(self, images, init_centroids):
        """Copy host RGB8 images and initial centroids into the arenas."""
        for i, (img, c0) in enumerate(zip(images, init_centroids)):
            self.rgb_of(i).copy_(torch.as_tensor(np.ascontiguousarray(img)), non_blocking=True)
            self.centroids_of(i).copy_(torch.as_tensor(np.ascontiguousarray(c0)),
                                       non_blocking=True)

    # ---- execution
    def run(self, stream=None, stage_events=None):
        """One run of the bound batch; stage_events: None, or
        2 * len(PIPELINE_STAGES) torch CUDA events (recorded once before)
        placed around the stages."""
        if stage_events is None:
            N.check(N.load().split_batch_run(self._h, stream_handle(stream)), "batch.run")
            return
        if any(e.cuda_event == 0 for e in stage_events):
            raise ValueError("stage events must have been recorded once (torch creates "
                             "CUDA events lazily)")
        ev = (C.c_void_p * len(stage_events))(*[e.cuda_event for e in stage_events])
        N.check(N.load().split_batch_run_events(self._h, ev, stream_handle(stream)), "batch.run")

    def capture(self):
        """Capture one run into a CUDA graph (replay with replay())."""
        torch.cuda.synchronize()
        s = torch.cuda.Stream(self.device)
        with torch.cuda.stream(s):
            self.run(s)        # warm the launch path outside capture
        s.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            self.run(torch.cuda.current_stream())
        self.graph = g
        return g

    def replay(self):
        self.graph.replay()
