"""Autotuner for the launch choices of the segmentation path.

What it tunes (split_tune_entry, include/split_gb300.h), per image size class:
  * the k-means work-unit height (16, 32, 64 or 128 rows of 64 columns),
    which trades per-unit reduction overhead against load balance, the
    parallelism of small images and the tail of the launch, and
  * the resident blocks per SM of the cooperative k-means launch.

Every candidate is timed on the GPU in use with the clustering workload of
the class (RGB8 -> float4 features, K = 16, 5-D, 20 iterations), L2 flushed
between runs, median of several CUDA-event timings; the fastest wins.  The
table is applied to the library (split_tune_set) and cached as JSON per GPU
model and SM count, so later processes load it instead of measuring again.

An image's unit height comes from its own pixel count, so it gets the same
reduction tree alone, in a pipeline and in a batch: tuning changes speed and
FP32 rounding of the centroid sums, never which results agree.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import json
import os
import re
import statistics

from . import _native as N

# Candidates of the default autotune.  16- and 32-row units cut the latency of
# a small image alone (512 x 512: 0.29 -> 0.18 ms at 16 rows) but slow batches
# and serving of the same images (more units, each with a reduction and a
# fetch), and an image uses one unit height alone and in a batch; pass
# unit_rows=ALL_UNIT_ROWS to autotune() to tune for single small images.
UNIT_ROWS = (64, 128)
ALL_UNIT_ROWS = (64, 128, 32, 16)
BLOCKS_PER_SM = (0, 2, 1)
# representative sizes of the classes (width, height); a class ends halfway
# (geometrically) between its size and the next one
CLASS_SIZES = ((512, 512), (1280, 720), (1920, 1080), (3840, 2160), (7680, 4320))
INT64_MAX = (1 << 63) - 1


@dataclasses.dataclass(frozen=True)
class Entry:
    max_pixels: int
    kmeans_unit_rows: int = 64
    kmeans_blocks_per_sm: int = 0


def _to_c(entries):
    arr = (N.TuneEntry * max(1, len(entries)))()
    for i, e in enumerate(entries):
        arr[i] = N.TuneEntry(e.max_pixels, e.kmeans_unit_rows, e.kmeans_blocks_per_sm)
    return arr


def apply(entries) -> None:
    """Install `entries` (ascending max_pixels) in the library."""
    entries = list(entries)
    N.check(N.load().split_tune_set(C.cast(_to_c(entries), C.c_void_p), len(entries)),
            "split_tune_set")


def current() -> list[Entry]:
    arr = (N.TuneEntry * N.TUNE_MAX_ENTRIES)()
    n = N.load().split_tune_get(C.cast(arr, C.c_void_p), N.TUNE_MAX_ENTRIES)
    return [Entry(arr[i].max_pixels, arr[i].kmeans_unit_rows, arr[i].kmeans_blocks_per_sm)
            for i in range(n)]


def class_bounds(sizes=CLASS_SIZES) -> list[int]:
    px = [w * h for w, h in sizes]
    return [int((a * b) ** 0.5) for a, b in zip(px, px[1:])] + [INT64_MAX]


def device_key(device=None) -> str:
    import torch
    d = torch.device("cuda", torch.cuda.current_device()) if device is None else \
        torch.device(device)
    p = torch.cuda.get_device_properties(d)
    name = re.sub(r"[^A-Za-z0-9]+", "-", p.name).strip("-")
    return f"{name}-sm{p.multi_processor_count}"


def cache_path(key: str) -> str:
    base = os.environ.get("SPLIT_GB300_TUNE_DIR") or os.path.join(
        os.path.expanduser("~"), ".cache", "split_gb300")
    return os.path.join(base, f"tune-{key}.json")


def save(entries, key: str, detail=None) -> str:
    path = cache_path(key)
    os.makedirs(os.path.dirname(path), exist_ok=True)
    doc = {"device": key, "entries": [dataclasses.asdict(e) for e in entries],
           "detail": detail or {}}
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(doc, f, indent=1)
    os.replace(tmp, path)
    return path


def load_cached(key: str):
    """Entries from the cache file of `key`, or None."""
    try:
        with open(cache_path(key)) as f:
            doc = json.load(f)
        return [Entry(**e) for e in doc["entries"]]
    except (OSError, ValueError, KeyError, TypeError):
        return None


def ensure(device=None) -> list[Entry] | None:
    """Apply the cached table of this GPU if there is one (no measuring)."""
    entries = load_cached(device_key(device))
    if entries is not None:
        apply(entries)
    return entries


_ensured = set()


def ensure_once(device=None) -> None:
    """ensure() the first time a device is used in this process."""
    key = device_key(device)
    if key not in _ensured:
        _ensured.add(key)
        ensure(device)


def pick(timings: dict) -> tuple:
    """The fastest candidate; ties go to the earlier candidate in the
    (unit rows, blocks per SM) order listed above."""
    order = [(r, b) for r in ALL_UNIT_ROWS for b in BLOCKS_PER_SM]
    best = min(order, key=lambda c: (timings.get(c, float("inf")), order.index(c)))
    return best


def measure_class(width, height, device, reps=5, warmup=2, iters=20, seed=0x5EED7777,
                  unit_rows=UNIT_ROWS):
    """CUDA-event milliseconds of split_kmeans_cluster on one image of the
    class for every candidate."""
    import torch
    from . import color, kmeans, synth
    rgb = synth.voronoi_rgb8(seed, width, height, 64, npalette=16, illum_gradient=True,
                             sigma=3.0)
    c0 = synth.pick_centroids(seed, rgb, 16, 5)
    d_rgb = torch.from_numpy(rgb).to(device)
    n = width * height
    feats = torch.empty((n, 4), dtype=torch.float32, device=device)
    color.pack_rgb8(d_rgb, feats)
    labels = torch.empty(n, dtype=torch.int32, device=device)
    cen = torch.empty((5, 16), dtype=torch.float32, device=device)
    c0d = torch.from_numpy(c0).to(device)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=device)
    ws = None
    saved = current()
    out = {}
    try:
        for rows in unit_rows:
            for bps in BLOCKS_PER_SM:
                apply([Entry(INT64_MAX, rows, bps)])
                times = []
                for r in range(warmup + reps):
                    cen.copy_(c0d)
                    flush.zero_()
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record()
                    ws = kmeans.cluster(feats, cen, labels, ws, max_iter=iters, threshold=-1.0,
                                        layout=N.LAYOUT_FLOAT4 | kmeans.UNIT_RANGE, dim=5,
                                        width=width)
                    e1.record()
                    torch.cuda.synchronize()
                    if r >= warmup:
                        times.append(e0.elapsed_time(e1))
                out[(rows, bps)] = statistics.median(times)
    finally:
        apply(saved)
    return out


def autotune(device=None, sizes=CLASS_SIZES, write_cache=True, reps=5, unit_rows=UNIT_ROWS):
    """Measure every class, apply the winners and cache them.  Returns
    (entries, detail) where detail holds the timings."""
    import torch
    d = torch.device("cuda", torch.cuda.current_device()) if device is None else \
        torch.device(device)
    bounds = class_bounds(sizes)
    entries, detail = [], {}
    for (w, h), bound in zip(sizes, bounds):
        t = measure_class(w, h, d, reps=reps, unit_rows=unit_rows)
        rows, bps = pick(t)
        entries.append(Entry(bound, rows, bps))
        detail[f"{w}x{h}"] = {f"rows{r}_bps{b}": round(v, 4) for (r, b), v in t.items()}
        detail[f"{w}x{h}"]["chosen"] = f"rows{rows}_bps{bps}"
    apply(entries)
    if write_cache:
        save(entries, device_key(d), detail)
    return entries, detail
