"""Shape from shading, named after split::device::sfs (sobel_normals.cuh:17-20)."""
from __future__ import annotations

import torch

from . import _native as N
from ._util import ptr, require_cuda, stream_handle


def sobel_normals(heights: torch.Tensor, normals: torch.Tensor, depth: float,
                  stream=None) -> None:
    """heights (H, W) float32 -> normals (3, H*W) float32 planar."""
    require_cuda(heights, "heights", torch.float32)
    require_cuda(normals, "normals", torch.float32)
    h, w = heights.shape
    st = N.load().split_sobel_normals(ptr(heights), w, h, depth, ptr(normals),
                                      stream_handle(stream))
    N.check(st, "sfs.sobel_normals")


def sobel_normals_rgb8(rgb: torch.Tensor, normals: torch.Tensor, depth: float = 1.0,
                       stream=None) -> None:
    """RGB8 (H, W, 3) -> normals of the luminance height map (L*/100)."""
    require_cuda(rgb, "rgb", torch.uint8)
    require_cuda(normals, "normals", torch.float32)
    h, w = rgb.shape[:2]
    st = N.load().split_sobel_normals_rgb8(ptr(rgb), w, h, depth, ptr(normals),
                                           stream_handle(stream))
    N.check(st, "sfs.sobel_normals_rgb8")
