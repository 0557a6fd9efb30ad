"""The C-ABI library loads on a machine without a GPU and exports every
entry point declared in include/*.h; host-only queries work.  CPU only."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import split_synth as synth
from split_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions(header="split_gb300.h"):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(split_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    lib = _native.load()
    names = declared_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n
        assert n in _native.exported_symbols(), f"{n} has no ctypes signature"
    # the input generators live in their own library, not in the product's
    slib = synth.load()
    for n in declared_functions("split_synth.h"):
        assert hasattr(slib, n), n
        assert n in synth.exported_symbols(), n
        assert not hasattr(lib, n), f"{n} is linked into libsplit_gb300.so"


def test_version_and_status_strings():
    lib = _native.load()
    assert b"sm_103a" in lib.split_version()
    for s in range(8):
        assert lib.split_status_string(s)


def test_workspace_queries():
    lib = _native.load()
    assert lib.split_ccl_workspace_size(3840, 2160) >= 256
    ws = lib.split_kmeans_cluster_workspace_size_2d(3840 * 2160, 3840, 16, 5)
    assert 256 < ws < 64 << 20
    # without the width the bound covers the worst case (width 1)
    assert lib.split_kmeans_cluster_workspace_size(3840 * 2160, 16, 5) >= ws
    assert lib.split_merge_small_workspace_size(3840, 2160) > 3840 * 2160 * 16
    # a bit per value in [-1, n) and a prefix per 32-bit word, after the header
    words = (1000 + 1 + 31) // 32
    assert lib.split_compress_labels_workspace_size(1000) >= 256 + 8 * words
    assert lib.split_compress_labels_workspace_size(3840 * 2160) < 4 * 3840 * 2160 // 8
    p = _native.PipelineParams(16, 5, 0.1, 20, -1.0, 1, 8, 0, 256, 0, 1, 1, 1.0)
    assert lib.split_pipeline_workspace_size(3840, 2160, C.byref(p)) > 0
    # the kept span sums of a clustering: about 0.5 B per pixel on top of the
    # state, which one assignment does not need
    state = lib.split_kmeans_assign_workspace_size(3840 * 2160, 16)
    assert 0.4 * 3840 * 2160 < ws - state < 0.6 * 3840 * 2160
    assert lib.split_kmeans_cluster_workspace_size_2d(3840 * 2160, 3840, 16, 5) >= \
        lib.split_kmeans_cluster_workspace_size_2d(1920 * 1080, 1920, 16, 5)
    # more than 64 clusters: the many-cluster k-means, with its own workspace
    many = _native.PipelineParams(1000, 5, 0.1, 20, -1.0, 1, 8, 0, 256, 0, 1, 1, 1.0)
    assert lib.split_pipeline_workspace_size(3840, 2160, C.byref(many)) > 0
    assert lib.split_kmeans_cluster_workspace_size_2d(3840 * 2160, 3840, 1000, 5) >= \
        2 * 5 * 1000 * 4 + 2 * 5 * 1000 * 8
    for k, d in ((0, 5), ((1 << 20) + 1, 5), (16, 4)):
        bad = _native.PipelineParams(k, d, 0.1, 20, -1.0, 1, 8, 0, 256, 0, 1, 1, 1.0)
        assert lib.split_pipeline_workspace_size(3840, 2160, C.byref(bad)) == 0


def test_invalid_arguments_rejected_on_host():
    lib = _native.load()
    # null pointers and bad sizes fail before touching the device
    assert lib.split_ccl(None, 4, 4, 4, 0, None, None, None, 0, None) == _native.ERR_INVALID
    assert lib.split_erode(None, None, 4, 4, 1, None) == _native.ERR_INVALID
    assert lib.split_kmeans_cluster(None, 0, 3, 10, 1, 0.1, None, 4, None, None, 0, 1, -1.0,
                                    None, None) == _native.ERR_INVALID
    # the many-cluster path checks its arguments the same way (pointers that
    # are never dereferenced: every case fails before any device call)
    fake = C.c_void_p(256)
    big = (1 << 20) + 1
    assert lib.split_kmeans_assign(fake, 0, 3, 100, 10, 0.1, fake, big, fake, fake, 1 << 30,
                                   None) == _native.ERR_INVALID
    assert lib.split_kmeans_cluster(fake, 0x200, 5, 100, 10, 0.1, fake, 100, fake, fake, 1 << 30,
                                    5, 1e-3, None, None) == _native.ERR_INVALID   # shift: 3-D only
    assert lib.split_kmeans_cluster(fake, 0, 4, 100, 10, 0.1, fake, 100, fake, fake, 1 << 30, 5,
                                    -1.0, None, None) == _native.ERR_INVALID      # D = 3 or 5
    assert lib.split_kmeans_cluster(fake, 0, 5, 100, 10, 0.1, fake, 100, fake, fake, 64, 5, -1.0,
                                    None, None) == _native.ERR_WORKSPACE


def test_synth_deterministic():
    a = synth.voronoi_rgb8(11, 97, 61, 12, npalette=5, illum_gradient=True, sigma=3.0)
    b = synth.voronoi_rgb8(11, 97, 61, 12, npalette=5, illum_gradient=True, sigma=3.0)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, synth.voronoi_rgb8(12, 97, 61, 12, npalette=5,
                                                    illum_gradient=True, sigma=3.0))
    c = synth.pick_centroids(11, a, 8, 5)
    assert c.shape == (5, 8) and np.isfinite(c).all()
    # distinct picks
    assert len({tuple(c[:, k]) for k in range(8)}) == 8


def test_maze_shape():
    m = synth.maze_labels(5, 512, 512)
    frac = (m == 0).mean()
    assert 0.4 < frac < 0.55            # the serpentine covers about half
    assert len(np.unique(m)) > 500      # plus many small blobs


def test_python_layer_rejects_cpu_tensors():
    torch = pytest.importorskip("torch")
    from split_gb300 import ccl, kmeans
    x = torch.zeros((4, 4), dtype=torch.int32)
    with pytest.raises(ValueError):
        ccl.connected_components(x, None, x)
    with pytest.raises(ValueError):
        kmeans.cluster(torch.zeros((3, 8)), torch.zeros((3, 2)), torch.zeros(8, dtype=torch.int32))
