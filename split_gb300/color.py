"""Feature preparation (samples/src/main.cu:164-223; color/detail/conversion.inl)."""
from __future__ import annotations

import torch

from . import _native as N
from ._util import ptr, require_cuda, stream_handle


def pack_rgb8(rgb: torch.Tensor, features4: torch.Tensor | None = None,
              luminance: torch.Tensor | None = None, stream=None) -> None:
    """RGB8 (..., 3) -> float4 features (r, g, b, 0) / 255 and/or L*/100."""
    require_cuda(rgb, "rgb", torch.uint8)
    n = rgb.numel() // 3
    st = N.load().split_pack_rgb8(ptr(rgb), n, ptr(features4), ptr(luminance),
                                  stream_handle(stream))
    N.check(st, "color.pack_rgb8")
