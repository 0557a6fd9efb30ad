"""Feature preparation (samples/src/main.cu:164-223; color/detail/conversion.inl)."""
from __future__ import annotations

import torch

from . import _native as N
from ._util import Workspace, ensure_workspace, ptr, require_cuda, stream_handle


def pack_rgb8(rgb: torch.Tensor, features4: torch.Tensor | None = None,
              luminance: torch.Tensor | None = None, stream=None) -> None:
    """RGB8 (..., 3) -> float4 features (r, g, b, 0) / 255 and/or L*/100."""
    require_cuda(rgb, "rgb", torch.uint8)
    n = rgb.numel() // 3
    st = N.load().split_pack_rgb8(ptr(rgb), n, ptr(features4), ptr(luminance),
                                  stream_handle(stream))
    N.check(st, "color.pack_rgb8")


def rgb_to_ic(rgb: torch.Tensor, ic: torch.Tensor, stream=None) -> None:
    """The sample's intensity / chroma planes (samples/src/main.cu:169-179,
    color::convert_color_space with rgb_to_ic, conversion.inl:99-108): RGB8
    (N x 3 bytes) -> ic (3, N) float32: intensity, r / intensity,
    g / intensity of the channels clamped to >= 1/255.  Rows 1-2 are the
    chroma input of ccl.merge_small_segments' reference rule."""
    require_cuda(rgb, "rgb", torch.uint8)
    require_cuda(ic, "ic", torch.float32)
    n = rgb.numel() // 3
    if ic.shape != (3, n) or not ic.is_contiguous():
        raise ValueError("ic must be a contiguous (3, N) float32 tensor")
    N.check(N.load().split_rgb8_to_ic(ptr(rgb), n, ptr(ic), stream_handle(stream)),
            "color.rgb_to_ic")


def pack_lab_beta(rgb: torch.Tensor, features: torch.Tensor, luminance: torch.Tensor | None = None,
                  mu: float = 1e5, temp: Workspace | None = None, stream=None) -> Workspace:
    """The sample's k-means features (samples/src/main.cu:169-173, :215-225):
    color::convert_color_space(rgb_to_lab) then color::beta_feature in place
    of L* (beta_feature.cuh:12-15), fused into two passes over RGB8.
    features: (N, 4) float32 -> (beta, a*, b*, 0), or (3, N) planar."""
    require_cuda(rgb, "rgb", torch.uint8)
    require_cuda(features, "features", torch.float32)
    n = rgb.numel() // 3
    if features.dim() == 2 and features.shape == (n, 4):
        layout = N.LAYOUT_FLOAT4
    elif features.dim() == 2 and features.shape == (3, n):
        layout = N.LAYOUT_PLANAR
    else:
        raise ValueError("features must be (N, 4) or (3, N) float32")
    if luminance is not None:
        require_cuda(luminance, "luminance", torch.float32)
    ws = ensure_workspace(temp, N.load().split_pack_lab_beta_workspace_size(n), rgb.device)
    st = N.load().split_pack_lab_beta(ptr(rgb), n, float(mu), layout, ptr(features),
                                      ptr(luminance), ws.ptr, ws.nbytes, stream_handle(stream))
    N.check(st, "color.pack_lab_beta")
    return ws
