"""Continuous-batching server for the segmentation path: a binding of the C++
server (split_server_* in include/split_gb300.h).

Requests (an RGB8 image plus its K, iteration count and initial centroids)
arrive open-loop.  The server's worker thread admits them in arrival order
while their device footprint fits the HBM budget, packs every admitted
request into the next batch (split_batch_*), and keeps up to `depth` batches
in flight, with uploads, compute and downloads on three streams.  Each
in-flight slot owns a resident arena that its batches bind to, so serving
allocates no device memory once the arenas have grown (reserve()).  A request
completes when its results are in host memory; its latency runs from its
arrival.

Each request's result is independent of what shares its batch, so a result
served in a mix equals the same request served alone.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import time

import numpy as np

from . import _native as N


@dataclasses.dataclass
class Request:
    rid: int
    rgb: object              # (H, W, 3) uint8: numpy array or (pinned) torch tensor
    nclusters: int
    iters: int
    centroids: object        # (dim, K) float32 initial centroids
    arrival: float = 0.0     # seconds on the server clock
    admitted: float | None = None   # when it was handed to the server
    done: float | None = None
    segment_labels: np.ndarray | None = None
    centroids_out: np.ndarray | None = None

    @property
    def shape(self):
        return tuple(self.rgb.shape[:2])

    @property
    def pixels(self) -> int:
        h, w = self.shape
        return h * w


def footprint(pixels: int, bytes_per_pixel: int) -> int:
    """Device bytes a request of `pixels` holds while admitted (the arena
    starts every image on 64 pixels)."""
    return (pixels + 63) // 64 * 64 * bytes_per_pixel


def bytes_per_pixel(params) -> int:
    cp = params.c()
    return int(N.load().split_server_bytes_per_pixel(C.byref(cp)))


def admission_plan(footprints, pixels, budget: int, max_batch_pixels: int, depth: int):
    """The C++ server's admission and batch-formation policy on the host
    alone: requests arriving at once -> (batch index of each request, number
    of batches, peak bytes in use)."""
    n = len(footprints)
    fp = np.ascontiguousarray(footprints, np.int64)
    px = np.ascontiguousarray(pixels, np.int64)
    out = np.full(n, -1, np.int32)
    peak = C.c_int64(0)
    nb = N.load().split_server_admission_test(
        C.c_void_p(fp.ctypes.data), C.c_void_p(px.ctypes.data), n, budget, max_batch_pixels,
        depth, C.c_void_p(out.ctypes.data), C.byref(peak))
    if nb < 0:
        raise N.SplitError(-nb, "admission_plan")
    return out, nb, peak.value


def percentile(values, q):
    v = sorted(values)
    if not v:
        return None
    k = (len(v) - 1) * q / 100.0
    lo = int(k)
    hi = min(lo + 1, len(v) - 1)
    return v[lo] + (v[hi] - v[lo]) * (k - lo)


class Server:
    """A split_server on one CUDA device.  keep_results: each request gets
    result buffers of its own (otherwise requests that share an input image
    share output buffers, for timing runs)."""

    def __init__(self, params=None, budget_bytes: int = 40 << 30,
                 max_batch_pixels: int = 64 << 20, depth: int = 2, device=None,
                 keep_results: bool = True, reserve_pixels: int = 0):
        import torch
        from .pipeline import Params
        self.torch = torch
        self.params = params or Params()
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None \
            else torch.device(device)
        self.keep_results = keep_results
        self.depth = depth
        cfg = N.ServerConfig(self.params.c(), budget_bytes, max_batch_pixels, depth,
                             self.device.index or 0)
        self._h = C.c_void_p()
        N.check(N.load().split_server_create(C.byref(cfg), C.byref(self._h)), "server.create")
        self.completed: list[Request] = []
        self._scratch = {}
        self._batches0 = 0
        if reserve_pixels > 0:
            self.reserve(reserve_pixels)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            N.load().split_server_destroy(h)
            self._h = None

    def reserve(self, pixels: int, max_requests: int = 4096) -> None:
        """Grow every slot's arena up front to hold a batch of `pixels` pixels
        (so a timed serving run allocates nothing)."""
        N.check(N.load().split_server_reserve(self._h, pixels, max_requests), "server.reserve")

    def counters(self) -> N.ServerCounters:
        c = N.ServerCounters()
        N.check(N.load().split_server_stats(self._h, C.byref(c)), "server.stats")
        return c

    @property
    def batch_sizes(self) -> list[float]:
        """Mean requests per batch since the last serve() started (one entry
        per batch, for compatibility with per-batch lists)."""
        c = self.counters()
        nb = int(c.batches) - self._batches0
        n = len(self.completed)
        return [n / nb] * nb if nb else []

    def _pinned(self, a, dtype):
        t = self.torch
        if isinstance(a, t.Tensor):
            if a.is_pinned():
                return a.contiguous()
            return a.contiguous().pin_memory()
        return t.from_numpy(np.ascontiguousarray(a, dtype=dtype)).pin_memory()

    def _outputs(self, r: Request):
        t = self.torch
        h, w = r.shape
        key = (id(r.rgb), h, w, r.nclusters)
        if not self.keep_results and key in self._scratch:
            return self._scratch[key]
        out = (t.empty((h, w), dtype=t.int32, pin_memory=True),
               t.empty((self.params.dim, r.nclusters), dtype=t.float32, pin_memory=True))
        if not self.keep_results:
            self._scratch[key] = out
        return out

    def serve(self, requests, realtime: bool = True):
        """Serve `requests`.  With realtime each request is submitted at its
        `arrival` (seconds after the call starts); otherwise all at once.
        Returns the requests in completion order."""
        lib = N.load()
        pending = sorted(requests, key=lambda r: r.arrival)
        prepared = []
        for r in pending:
            if not realtime:
                r.arrival = 0.0
            rgb = self._pinned(r.rgb, np.uint8)
            c0 = self._pinned(r.centroids, np.float32)
            lab, cout = self._outputs(r)
            h, w = r.shape
            req = N.ServerRequest(rgb.data_ptr(), w, h, r.nclusters, r.iters, c0.data_ptr(),
                                  lab.data_ptr(), cout.data_ptr(), None, None, None)
            prepared.append((r, req, rgb, c0, lab, cout))
        self._batches0 = int(self.counters().batches)
        self.completed = []
        by_ticket = {}
        comp = (N.Completion * 64)()
        got = C.c_int(0)
        t0 = time.perf_counter()

        def drain(timeout_ms: int) -> None:
            N.check(lib.split_server_poll(self._h, comp, 64, timeout_ms, C.byref(got)),
                    "server.poll")
            for i in range(got.value):
                c = comp[i]
                r, lab, cout = by_ticket.pop(int(c.ticket))
                if c.status != N.OK:
                    raise N.SplitError(c.status, f"serve: request {r.rid}")
                r.done = r.admitted + c.latency_ms * 1e-3
                r.segment_labels = lab.numpy()
                r.centroids_out = cout.numpy()
                self.completed.append(r)

        ticket = C.c_uint64(0)
        for r, req, _rgb, _c0, lab, cout in prepared:
            while realtime:
                wait = r.arrival - (time.perf_counter() - t0)
                if wait <= 0:
                    break
                if by_ticket:
                    drain(max(0, min(int(wait * 1e3), 1)))
                else:
                    time.sleep(min(wait, 1e-3))
            r.admitted = time.perf_counter() - t0
            N.check(lib.split_server_submit(self._h, C.byref(req), C.byref(ticket)),
                    f"serve: submit {r.rid}")
            by_ticket[int(ticket.value)] = (r, lab, cout)
            drain(0)
        while by_ticket:
            drain(100)
        self._keep = prepared   # host buffers stay alive with the results
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
