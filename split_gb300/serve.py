"""Continuous-batching server for the segmentation path.

Requests (an RGB8 image plus its K, iteration count and initial centroids)
arrive open-loop.  The loop admits them in arrival order while their device
footprint fits the HBM budget, packs every admitted request into the next
batch (one fixed launch sequence for the batch, split_batch_*), and keeps up
to two batches in flight: while one batch computes, the host admits new
arrivals and stages the next batch's inputs with asynchronous copies from
pinned memory.  Each in-flight slot owns a resident arena (RGB, centroid,
label, normal and workspace buffers, union-find and merge state included)
that every batch of that slot binds to, so serving allocates no device
memory once the arenas have grown to the largest batch.  A request completes
when its batch's results are back in host memory; its latency runs from its
arrival.

Each request's result is independent of what shares its batch (per-image
tiles, reduction trees and label spaces), so a result served in a mix equals
the same request served alone.
"""
from __future__ import annotations

import collections
import dataclasses
import time

import numpy as np

# device bytes held per pixel of a batch: RGB8 arena (3), float4 features (16),
# three int32 label arenas and sizes (16), normals (12), merge state and hash
# table (44), k-means and tile tables (< 1)
BYTES_PER_PIXEL = 92


@dataclasses.dataclass
class Request:
    rid: int
    rgb: np.ndarray          # (H, W, 3) uint8
    nclusters: int
    iters: int
    centroids: np.ndarray    # (dim, K) float32 initial centroids
    arrival: float = 0.0     # seconds on the server clock
    admitted: float | None = None
    done: float | None = None
    segment_labels: np.ndarray | None = None
    centroids_out: np.ndarray | None = None

    @property
    def pixels(self) -> int:
        return self.rgb.shape[0] * self.rgb.shape[1]

    @property
    def footprint(self) -> int:
        return (self.pixels + 63) // 64 * 64 * BYTES_PER_PIXEL


class Admission:
    """FIFO admission under a byte budget (no GPU: unit-testable on CPU)."""

    def __init__(self, budget_bytes: int):
        self.budget = int(budget_bytes)
        self.in_use = 0
        self.waiting: collections.deque[Request] = collections.deque()
        self.admitted: list[Request] = []

    def arrive(self, req: Request) -> None:
        if req.footprint > self.budget:
            raise ValueError(f"request {req.rid} needs {req.footprint} B, budget {self.budget} B")
        self.waiting.append(req)

    def admit(self, now: float) -> int:
        n = 0
        while self.waiting and self.in_use + self.waiting[0].footprint <= self.budget:
            r = self.waiting.popleft()
            r.admitted = now
            self.in_use += r.footprint
            self.admitted.append(r)
            n += 1
        return n

    def take(self, max_pixels: int | None = None) -> list[Request]:
        """Hand the admitted requests (in order) to the next batch."""
        out, keep, px = [], [], 0
        for r in self.admitted:
            if max_pixels is None or px + r.pixels <= max_pixels or not out:
                out.append(r)
                px += r.pixels
            else:
                keep.append(r)
        self.admitted = keep
        return out

    def release(self, reqs) -> None:
        for r in reqs:
            self.in_use -= r.footprint
        assert self.in_use >= 0


def percentile(values, q):
    v = sorted(values)
    if not v:
        return None
    k = (len(v) - 1) * q / 100.0
    lo = int(k)
    hi = min(lo + 1, len(v) - 1)
    return v[lo] + (v[hi] - v[lo]) * (k - lo)




class _Flight:
    """One batch between launch and the host seeing its results."""

    def __init__(self, reqs, batch, done, labels_h, cents_h):
        self.reqs, self.batch, self.done = reqs, batch, done
        self.labels_h, self.cents_h = labels_h, cents_h


class Server:
    """Serves requests through split_batch on one CUDA device.

    Three streams: uploads of the next batch (host to device), the batch
    launch sequence itself, and downloads of finished results.  All batches
    compute on the one compute stream, so the k-means kernel, a cooperative
    grid that fills the GPU, never shares the GPU with another batch's; the
    copy streams overlap both directions of PCIe/C2C traffic with it.
    `depth` bounds the batches launched but not yet collected.
    """

    def __init__(self, params=None, budget_bytes: int = 40 << 30,
                 max_batch_pixels: int = 64 << 20, depth: int = 2, device=None,
                 keep_results: bool = True, reserve_pixels: int = 0):
        import torch
        from .pipeline import Params
        self.torch = torch
        self.params = params or Params()
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None \
            else torch.device(device)
        self.admission = Admission(budget_bytes)
        self.max_batch_pixels = max_batch_pixels
        self.depth = depth
        self.keep_results = keep_results
        self.h2d = torch.cuda.Stream(self.device)
        self.compute = torch.cuda.Stream(self.device)
        self.d2h = torch.cuda.Stream(self.device)
        self.inflight: collections.deque[_Flight] = collections.deque()
        self.completed: list[Request] = []
        self.batches = 0
        from .batch import Arena
        # one resident arena per slot; batch i uses slot i % depth, which the
        # collection order (oldest first) has freed by the time it launches
        self.arenas = [Arena(self.device, normals=bool(self.params.compute_normals))
                       for _ in range(depth)]
        self.batch_sizes: list[int] = []
        self.t0 = time.perf_counter()
        if reserve_pixels > 0:
            self.reserve(reserve_pixels)

    def reserve(self, pixels: int, max_requests: int = 4096) -> None:
        """Grow every arena up front to hold a batch of `pixels` pixels (so a
        timed serving run allocates nothing)."""
        from .batch import Batch
        side = 8192
        probe = Batch([(side, max(1, (pixels + side - 1) // side), 64, 1)], self.params,
                      self.device, arena=self.arenas[0])
        wsb = probe.ws.nbytes
        del probe
        for a in self.arenas:
            a.ensure(pixels + 64 * max_requests, self.params.dim * 64 * max_requests, wsb)
            if not self.keep_results:
                a.host_buffers()

    def now(self) -> float:
        return time.perf_counter() - self.t0

    def _host(self, a):
        t = self.torch
        if isinstance(a, t.Tensor):
            return a
        return t.from_numpy(np.ascontiguousarray(a))

    def _launch(self, reqs) -> None:
        torch = self.torch
        from .batch import Batch
        shapes = [(r.rgb.shape[1], r.rgb.shape[0], r.nclusters, r.iters) for r in reqs]
        with torch.cuda.stream(self.h2d):
            b = Batch(shapes, self.params, self.device, stream=self.h2d,
                      arena=self.arenas[self.batches % self.depth])
            for i, r in enumerate(reqs):
                b.rgb_of(i).copy_(self._host(r.rgb), non_blocking=True)
                b.centroids_of(i).copy_(self._host(r.centroids), non_blocking=True)
            up = torch.cuda.Event()
            up.record(self.h2d)
        self.compute.wait_event(up)
        b.run(self.compute)
        ran = torch.cuda.Event()
        ran.record(self.compute)
        self.d2h.wait_event(ran)
        with torch.cuda.stream(self.d2h):
            if self.keep_results:
                # results outlive the batch: buffers of their own
                labels_h = torch.empty(b.segment_labels.shape, dtype=torch.int32,
                                       pin_memory=True)
                cents_h = torch.empty(b.centroids.shape, dtype=torch.float32, pin_memory=True)
            else:
                # the slot's buffers, pinned once (the slot is reused only
                # after this batch has been collected)
                lh, ch = self.arenas[self.batches % self.depth].host_buffers()
                labels_h = lh[:b.segment_labels.numel()].view(b.segment_labels.shape)
                cents_h = ch[:b.centroids.numel()].view(b.centroids.shape)
            labels_h.copy_(b.segment_labels, non_blocking=True)
            cents_h.copy_(b.centroids, non_blocking=True)
            done = torch.cuda.Event()
            done.record(self.d2h)
        self.inflight.append(_Flight(reqs, b, done, labels_h, cents_h))
        self.batches += 1
        self.batch_sizes.append(len(reqs))

    def _finish(self, f: _Flight) -> None:
        t = self.now()
        b = f.batch
        b.ws.check("serve: batch")
        for i, r in enumerate(f.reqs):
            r.done = t
            if self.keep_results:
                # views of the batch's pinned download buffers (no host copy)
                o = b.offsets[i]
                h, w = r.rgb.shape[:2]
                r.segment_labels = f.labels_h[o:o + w * h].numpy().reshape(h, w)
                co = b.coffsets[i]
                r.centroids_out = f.cents_h[co:co + self.params.dim * r.nclusters].numpy() \
                    .reshape(self.params.dim, r.nclusters)
        self.admission.release(f.reqs)
        self.completed.extend(f.reqs)

    def _collect(self, block: bool) -> bool:
        """Finish the oldest batches whose results are home; with block, wait
        for the oldest one.  Returns whether anything finished."""
        got = False
        while self.inflight:
            f = self.inflight[0]
            if not f.done.query():
                if not block or got:
                    break
                f.done.synchronize()
            self.inflight.popleft()
            self._finish(f)
            got = True
        return got

    def serve(self, requests, realtime: bool = True):
        """Serve `requests`.  With realtime each request becomes visible at its
        `arrival` (seconds after the call starts); otherwise all are visible
        at once.  Returns the requests in completion order."""
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        total = len(pending) + len(self.completed)
        self.t0 = time.perf_counter()
        if not realtime:
            for r in pending:
                r.arrival = 0.0
        while len(self.completed) < total:
            now = self.now()
            while pending and pending[0].arrival <= now:
                self.admission.arrive(pending.popleft())
            self.admission.admit(now)
            self._collect(block=False)
            if self.admission.admitted and len(self.inflight) < self.depth:
                self._launch(self.admission.take(self.max_batch_pixels))
                continue
            if self.inflight and (len(self.inflight) >= self.depth or not pending):
                self._collect(block=True)
            elif pending:
                # nothing to launch: wait for the next arrival, polling the
                # in-flight batches meanwhile
                time.sleep(min(2e-4, max(0.0, pending[0].arrival - now)))
        self.torch.cuda.synchronize()
        return self.completed

    @staticmethod
    def report(reqs, wall_s: float) -> dict:
        lat = [(r.done - r.arrival) * 1e3 for r in reqs]
        px = sum(r.pixels for r in reqs)
        return {"requests": len(reqs), "p50_ms": round(percentile(lat, 50), 3),
                "p99_ms": round(percentile(lat, 99), 3),
                "mpix_s": round(px / wall_s / 1e6, 1), "wall_s": round(wall_s, 3)}


def poisson_arrivals(seed: int, n: int, rate_per_s: float):
    """Arrival times (seconds) of an open-loop Poisson process."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate_per_s, size=n))
