"""GB300-native (sm_103a) segmentation hot path of nitronoid/split.

Device entry points live in libsplit_gb300.so behind the C ABI of
include/split_gb300.h; the modules here mirror the reference's namespaces
(split::device::kmeans / ccl / morph / sfs / color) over torch CUDA tensors.
"""
from . import _native
from ._native import SplitError
from ._util import Workspace

__all__ = ["SplitError", "Workspace", "kmeans", "ccl", "morph", "sfs", "color", "synth",
           "version"]


def version() -> str:
    return _native.load().split_version().decode()


def __getattr__(name):
    import importlib
    if name in ("kmeans", "ccl", "morph", "sfs", "color", "synth", "pipeline"):
        return importlib.import_module(f".{name}", __name__)
    raise AttributeError(name)
