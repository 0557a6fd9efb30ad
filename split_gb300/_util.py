"""Shared helpers of the Python layer: device pointers, streams, workspaces."""
from __future__ import annotations

import ctypes as C

import torch

from . import _native as N


def ptr(t: torch.Tensor | None):
    if t is None:
        return None
    return C.c_void_p(t.data_ptr())


def stream_handle(stream: torch.cuda.Stream | None = None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def require_cuda(t: torch.Tensor, name: str, dtype: torch.dtype | None = None) -> None:
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor")
    if dtype is not None and t.dtype != dtype:
        raise ValueError(f"{name} must have dtype {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")


class Workspace:
    """Caller-owned scratch memory for the device entry points.

    Plays the role of the reference's ``thrust::device_ptr<void> temp`` block
    sized by the ``*_workspace`` queries.  It is zero-filled once on creation;
    every entry point leaves it ready for the next call.
    """

    def __init__(self, nbytes: int, device: torch.device | str | int | None = None):
        nbytes = max(int(nbytes), 256)
        dev = torch.device("cuda", torch.cuda.current_device()) if device is None else \
            torch.device(device)
        self.buf = torch.zeros(nbytes + 256, dtype=torch.uint8, device=dev)
        off = (-self.buf.data_ptr()) % 256
        self.view = self.buf[off:off + nbytes]
        self.nbytes = nbytes

    @classmethod
    def over(cls, buf: torch.Tensor, nbytes: int) -> "Workspace":
        """A workspace inside an existing uint8 device buffer (kept, not
        zeroed: the entry points leave their state ready for the next call,
        whatever layout that call carves)."""
        ws = cls.__new__(cls)
        nbytes = max(int(nbytes), 256)
        off = (-buf.data_ptr()) % 256
        if buf.numel() < off + nbytes:
            raise ValueError("buffer too small for the workspace")
        ws.buf = buf
        ws.view = buf[off:off + nbytes]
        ws.nbytes = nbytes
        return ws

    @property
    def ptr(self):
        return C.c_void_p(self.view.data_ptr())

    def status(self, stream=None) -> int:
        out = C.c_int(0)
        N.check(N.load().split_workspace_status(self.ptr, stream_handle(stream), C.byref(out)),
                "split_workspace_status")
        return out.value

    def check(self, where: str, stream=None) -> None:
        st = self.status(stream)
        if st != N.OK:
            raise N.SplitError(st, where + " (device)")


def ensure_workspace(ws: Workspace | None, nbytes: int, device) -> Workspace:
    if ws is None or ws.nbytes < nbytes:
        return Workspace(nbytes, device)
    return ws
