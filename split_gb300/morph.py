"""Morphology, named after split::device::morph (erode.cuh:16-18)."""
from __future__ import annotations

import torch

from . import _native as N
from ._util import ptr, require_cuda, stream_handle


def erode(labels: torch.Tensor, niterations: int = 1, *, out: torch.Tensor | None = None,
          stream=None) -> torch.Tensor:
    """split::device::morph::erode: square (2n+1)^2 erosion of every label's
    mask, image border as background, eroded pixels -1.  In place (as the
    reference) unless ``out`` is given.  One kernel pass erodes by up to 16;
    larger n runs in passes (square erosions compose: radius a then b is
    radius a + b)."""
    require_cuda(labels, "labels", torch.int32)
    if labels.dim() != 2:
        raise ValueError("labels must be (height, width)")
    if niterations < 0:
        raise ValueError("niterations must be >= 0")
    h, w = labels.shape
    dst = out if out is not None else torch.empty_like(labels)
    if niterations == 0:
        if out is not None:
            dst.copy_(labels)
        return dst if out is not None else labels
    src, left, spare = labels, niterations, None
    while left > 0:
        r = min(16, left)
        if src is dst:
            if spare is None:
                spare = torch.empty_like(labels)
            tgt = spare
        else:
            tgt = dst
        N.check(N.load().split_erode(ptr(src), ptr(tgt), w, h, r, stream_handle(stream)),
                "morph.erode")
        src, left = tgt, left - r
    if src is not dst:
        dst.copy_(src)
    if out is None:
        labels.copy_(dst)
        return labels
    return dst
