"""Shape from shading, named after split::device::sfs (sobel_normals.cuh:17-20)."""
from __future__ import annotations

import torch

from . import _native as N
from ._util import Workspace, ensure_workspace, ptr, require_cuda, stream_handle


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


def estimate_normals(shading_intensity: torch.Tensor, light_vector, normals: torch.Tensor,
                     smoothness_weight: float, *, max_iter: int = 1500, tol: float = 1e-5,
                     temp: Workspace | None = None, iterations_out: torch.Tensor | None = None,
                     stream=None) -> Workspace:
    """split::device::sfs::estimate_normals (estimate_normals.cuh:14-18).

    shading_intensity: (H, W) float32; light_vector: 3 floats (any length);
    normals: (3, H*W) float32 out.  Relaxation to |b - A x| <= tol |b| or
    max_iter sweeps, as the reference's SOR (omega 1, 1e-5, 1500)."""
    require_cuda(shading_intensity, "shading_intensity", torch.float32)
    require_cuda(normals, "normals", torch.float32)
    h, w = shading_intensity.shape
    if normals.numel() != 3 * h * w:
        raise ValueError("normals must hold 3 x H*W floats")
    lib = N.load()
    ws = ensure_workspace(temp, lib.split_estimate_normals_workspace_size(w, h),
                          shading_intensity.device)
    lx, ly, lz = (float(v) for v in light_vector)
    st = lib.split_estimate_normals(ptr(shading_intensity), w, h, lx, ly, lz,
                                    float(smoothness_weight), int(max_iter), float(tol),
                                    ptr(normals), ptr(iterations_out), ws.ptr, ws.nbytes,
                                    stream_handle(stream))
    N.check(st, "sfs.estimate_normals")
    return ws
