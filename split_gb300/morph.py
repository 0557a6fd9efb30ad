"""Morphology, named after split::device::morph (erode.cuh:16-18)."""
from __future__ import annotations

import torch

from . import _native as N
from ._util import ptr, require_cuda, stream_handle


def erode(labels: torch.Tensor, niterations: int = 1, *, out: torch.Tensor | None = None,
          stream=None) -> torch.Tensor:
    """split::device::morph::erode: square (2n+1)^2 erosion of every label's
    mask, image border as background, eroded pixels -1.  In place (as the
    reference) unless ``out`` is given."""
    require_cuda(labels, "labels", torch.int32)
    if labels.dim() != 2:
        raise ValueError("labels must be (height, width)")
    h, w = labels.shape
    dst = out if out is not None else torch.empty_like(labels)
    st = N.load().split_erode(ptr(labels), ptr(dst), w, h, niterations, stream_handle(stream))
    N.check(st, "morph.erode")
    if out is None:
        labels.copy_(dst)
        return labels
    return dst
