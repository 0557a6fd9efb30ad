"""ctypes bindings of libsplit_gb300.so (the C ABI declared in include/split_gb300.h).

The library is built in-tree by ``split_gb300.build``.  Loading fails loudly when
it is missing: there is no fallback implementation of any entry point.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

_lib = None

# status codes (split_status in include/split_gb300.h)
OK, ERR_INVALID, ERR_WORKSPACE, ERR_NOT_CONVERGED, ERR_CUDA, ERR_OVERFLOW, ERR_TIMEOUT, \
    ERR_UNSUPPORTED = range(8)
LAYOUT_PLANAR, LAYOUT_FLOAT4, LAYOUT_RGB8 = 0, 1, 2
LABEL_MIN_INDEX, LABEL_MAX_INDEX = 0, 1
MERGE_MOST_BOUNDARY, MERGE_REF_CHROMA = 0, 1

_vp, _sz, _i32, _i64, _f32, _u64 = C.c_void_p, C.c_size_t, C.c_int, C.c_int64, C.c_float, \
    C.c_uint64

_SIGS = {
    "split_version": (C.c_char_p, []),
    "split_status_string": (C.c_char_p, [_i32]),
    "split_workspace_status": (_i32, [_vp, _vp, C.POINTER(C.c_int)]),
    "split_kmeans_set_wait_test": (None, [C.c_uint, _i32]),
    "split_kmeans_cluster_workspace_size": (_sz, [_i64, _i32, _i32]),
    "split_kmeans_cluster_workspace_size_2d": (_sz, [_i64, _i32, _i32, _i32]),
    "split_kmeans_cluster": (_i32, [_vp, _i32, _i32, _i64, _i32, _f32, _vp, _i32, _vp, _vp, _sz,
                                    _i32, _f32, _vp, _vp]),
    "split_kmeans_cluster_noalloc": (_i32, [_vp, _i32, _i32, _i64, _i32, _f32, _vp, _i32, _vp,
                                            _i32, _f32, _vp, _vp, _vp]),
    "split_kmeans_assign_workspace_size": (_sz, [_i64, _i32]),
    "split_kmeans_assign": (_i32, [_vp, _i32, _i32, _i64, _i32, _f32, _vp, _i32, _vp, _vp, _sz,
                                   _vp]),
    "split_kmeans_update_workspace_size": (_sz, [_i64, _i32, _i32]),
    "split_kmeans_update": (_i32, [_vp, _vp, _i32, _i32, _i64, _i32, _f32, _vp, _i32, _vp, _sz,
                                   _vp]),
    "split_kmeans_propagate": (_i32, [_vp, _i64, _vp, _i32, _i32, _vp, _vp]),
    "split_ccl_workspace_size": (_sz, [_i32, _i32]),
    "split_ccl": (_i32, [_vp, _i32, _i32, _i32, _i32, _vp, _vp, _vp, _sz, _vp]),
    "split_compress_labels_workspace_size": (_sz, [_i64]),
    "split_compress_labels": (_i32, [_vp, _i64, _vp, _vp, _sz, _vp]),
    "split_segment_adjacency_edges_workspace_size": (_sz, [_i32, _i32]),
    "split_segment_adjacency_edges": (_i32, [_vp, _i32, _i32, _vp, _vp, _vp, _sz, _vp]),
    "split_segment_adjacency_workspace_size": (_sz, [_i32, _i32]),
    "split_segment_adjacency": (_i32, [_vp, _i32, _i32, _vp, _vp, _vp, _vp, _sz, _vp]),
    "split_merge_small_workspace_size": (_sz, [_i32, _i32]),
    "split_merge_small": (_i32, [_vp, _i32, _i32, _i32, _i32, _vp, _vp, _vp, _sz, _vp]),
    "split_erode": (_i32, [_vp, _vp, _i32, _i32, _i32, _vp]),
    "split_erode_mapped": (_i32, [_vp, _vp, _i32, _i32, _i32, _vp, _vp]),
    "split_sobel_normals": (_i32, [_vp, _i32, _i32, _f32, _vp, _vp]),
    "split_sobel_normals_rgb8": (_i32, [_vp, _i32, _i32, _f32, _vp, _vp]),
    "split_pack_rgb8": (_i32, [_vp, _i64, _vp, _vp, _vp]),
    "split_rgb8_to_ic": (_i32, [_vp, _i64, _vp, _vp]),
    "split_pipeline_workspace_size": (_sz, [_i32, _i32, _vp]),
    "split_pipeline_run": (_i32, [_vp, _i32, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp, _vp]),
    "split_launch_count": (C.c_ulonglong, []),
    "split_tune_set": (C.c_int, [C.c_void_p, C.c_int]),
    "split_merge_smooth_workspace_size": (C.c_size_t, [C.c_int, C.c_int]),
    "split_pack_lab_beta_workspace_size": (C.c_size_t, [C.c_int64]),
    "split_estimate_normals_workspace_size": (C.c_size_t, [C.c_int, C.c_int]),
    "split_estimate_normals": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_float,
                                         C.c_float, C.c_float, C.c_int, C.c_float, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]),
    "split_pack_lab_beta": (C.c_int, [C.c_void_p, C.c_int64, C.c_float, C.c_int, C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]),
    "split_merge_smooth": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_float,
                                     C.c_void_p, C.c_size_t, C.c_void_p]),
    "split_tune_get": (C.c_int, [C.c_void_p, C.c_int]),
    "split_batch_create": (_i32, [_vp, _i32, _vp, _vp]),
    "split_batch_destroy": (None, [_vp]),
    "split_batch_workspace_size": (_sz, [_vp]),
    "split_batch_arena_pixels": (_i64, [_vp]),
    "split_batch_pixel_offset": (_i64, [_vp, _i32]),
    "split_batch_centroid_floats": (_i64, [_vp]),
    "split_batch_centroid_offset": (_i64, [_vp, _i32]),
    "split_batch_bind": (_i32, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    "split_batch_run": (_i32, [_vp, _vp]),
    "split_batch_run_events": (_i32, [_vp, _vp, _vp]),
    "split_server_bytes_per_pixel": (_sz, [_vp]),
    "split_server_create": (_i32, [_vp, _vp]),
    "split_server_reserve": (_i32, [_vp, _i64, _i32]),
    "split_server_submit": (_i32, [_vp, _vp, _vp]),
    "split_server_poll": (_i32, [_vp, _vp, _i32, _i32, _vp]),
    "split_server_stats": (_i32, [_vp, _vp]),
    "split_server_destroy": (_i32, [_vp]),
    "split_server_admission_test": (_i32, [_vp, _vp, _i32, _i64, _i64, _i32, _vp, _vp]),
}


class PipelineParams(C.Structure):
    """split_pipeline_params (include/split_gb300.h)."""
    _fields_ = [("nclusters", C.c_int), ("dim", C.c_int), ("xy_scale", C.c_float),
                ("kmeans_iters", C.c_int), ("kmeans_threshold", C.c_float),
                ("features", C.c_int), ("connectivity", C.c_int), ("convention", C.c_int),
                ("merge_P", C.c_int), ("merge_policy", C.c_int), ("erode_radius", C.c_int),
                ("compute_normals", C.c_int), ("depth", C.c_float), ("beta_mu", C.c_float)]


FEATURES_LAB_BETA = 3   # split_pipeline_params.features: the sample's Lab + beta


PIPELINE_STAGES = ("pack", "kmeans", "ccl", "merge", "erode", "normals")


class ServerConfig(C.Structure):
    """split_server_config (include/split_gb300.h)."""
    _fields_ = [("params", PipelineParams), ("hbm_budget_bytes", C.c_size_t),
                ("max_batch_pixels", C.c_int64), ("max_inflight", C.c_int), ("device", C.c_int)]


class ServerRequest(C.Structure):
    """split_request (include/split_gb300.h)."""
    _fields_ = [("rgb", C.c_void_p), ("width", C.c_int), ("height", C.c_int),
                ("nclusters", C.c_int), ("kmeans_iters", C.c_int), ("centroids", C.c_void_p),
                ("segment_labels", C.c_void_p), ("centroids_out", C.c_void_p),
                ("normals", C.c_void_p), ("cluster_labels", C.c_void_p), ("user", C.c_void_p)]


class Completion(C.Structure):
    """split_completion (include/split_gb300.h)."""
    _fields_ = [("ticket", C.c_uint64), ("user", C.c_void_p), ("status", C.c_int),
                ("pixels", C.c_int64), ("latency_ms", C.c_double)]


class ServerCounters(C.Structure):
    """split_server_counters (include/split_gb300.h)."""
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("batches", C.c_uint64),
                ("in_use_bytes", C.c_size_t), ("peak_in_use_bytes", C.c_size_t),
                ("bytes_per_pixel", C.c_size_t), ("budget_bytes", C.c_size_t)]


class BatchImage(C.Structure):
    """split_batch_image (include/split_gb300.h)."""
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("nclusters", C.c_int),
                ("kmeans_iters", C.c_int)]


class TuneEntry(C.Structure):
    """split_tune_entry (include/split_gb300.h)."""
    _fields_ = [("max_pixels", C.c_int64), ("kmeans_unit_rows", C.c_int),
                ("kmeans_blocks_per_sm", C.c_int)]


TUNE_MAX_ENTRIES = 64


class SplitError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        super().__init__(f"{where}: {status_string(status)} (status {status})")


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load the native library (optionally building it first)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise ImportError(
                f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; "
                "g.build()'` (or python split_gb300/build.py)")
        _build.build_library()
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols() -> list[str]:
    return list(_SIGS)


def status_string(status: int) -> str:
    return load().split_status_string(status).decode()


def check(status: int, where: str) -> None:
    if status != OK:
        raise SplitError(status, where)
