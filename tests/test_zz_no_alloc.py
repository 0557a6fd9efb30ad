"""The allocation-free k-means entry point (split_kmeans_cluster_noalloc).

It exists for callers that cannot allocate device memory where they cluster
(a latency-critical serving loop, where cudaMalloc would synchronise the
device; plugins whose device memory is owned by someone else); its scratch is
a fixed device array inside the library instead of a caller workspace.  These
checks call it through the C ABI and compare it with the workspace entry point
(split_kmeans_cluster) on the same inputs, twice in a row, since the second
call reuses the array the first call left behind.  The file is collected last
so that a failure here comes after every other test has run; it also passes on
its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from split_gb300 import _native, synth

pytestmark = pytest.mark.gpu


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _workspace_run(torch, pts, layout, dim, n, w, c0, labels_shape, iters):
    lib = _native.load()
    nbytes = lib.split_kmeans_cluster_workspace_size_2d(n, w, c0.shape[1], dim)
    ws = torch.zeros(nbytes + 256, dtype=torch.uint8, device=pts.device)
    off = (-ws.data_ptr()) % 256
    cent = c0.clone()
    lab = torch.empty(labels_shape, dtype=torch.int32, device=pts.device)
    st = lib.split_kmeans_cluster(_ptr(pts), layout, dim, n, w, 0.1, _ptr(cent), c0.shape[1],
                                  _ptr(lab), C.c_void_p(ws.data_ptr() + off), nbytes, iters,
                                  -1.0, None, C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == _native.OK
    return lab, cent


def _noalloc_run(torch, pts, layout, dim, n, w, c0, labels_shape, iters):
    lib = _native.load()
    cent = c0.clone()
    lab = torch.empty(labels_shape, dtype=torch.int32, device=pts.device)
    its = torch.full((1,), -1, dtype=torch.int32, device=pts.device)
    status = torch.full((1,), -1, dtype=torch.int32, device=pts.device)
    st = lib.split_kmeans_cluster_noalloc(
        _ptr(pts), layout, dim, n, w, 0.1, _ptr(cent), c0.shape[1], _ptr(lab), iters, -1.0,
        _ptr(its), _ptr(status), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == _native.OK
    torch.cuda.synchronize()
    assert int(status.item()) == _native.OK
    assert int(its.item()) == iters
    return lab, cent


@pytest.mark.parametrize("layout,dim", [(_native.LAYOUT_RGB8, 5), (_native.LAYOUT_PLANAR, 3)])
def test_noalloc_matches_workspace_entry_point(layout, dim):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("a CUDA device is required")
    dev = torch.device("cuda", 0)
    # two different images in a row: the second call must not see the first
    # call's leftovers in the shared array
    for seed, (w, h) in ((31, (640, 360)), (32, (333, 257))):
        rgb = synth.voronoi_rgb8(seed, w, h, 40, npalette=12, illum_gradient=True, sigma=3.0)
        c0 = torch.from_numpy(synth.pick_centroids(seed, rgb, 12, dim)).to(dev)
        if layout == _native.LAYOUT_RGB8:
            pts = torch.from_numpy(rgb.reshape(-1, 3).copy()).to(dev)
        else:
            pts = torch.from_numpy(synth.features(rgb, dim)).to(dev)
        n = w * h
        ref_lab, ref_c = _workspace_run(torch, pts, layout, dim, n, w, c0, (n,), 8)
        lab, cent = _noalloc_run(torch, pts, layout, dim, n, w, c0, (n,), 8)
        # the same computation in the same fixed order: identical results
        assert torch.equal(lab, ref_lab)
        assert torch.equal(cent, ref_c)


def test_noalloc_any_image_size():
    """The array holds per-image state only, so an image larger than a 4K
    frame (4096 x 2304, 2304 tiles of 64 x 64) clusters like the workspace
    entry point does, bit for bit."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    w, h = 4096, 2304
    rgb = synth.voronoi_rgb8(33, w, h, 128, npalette=16, illum_gradient=True, sigma=3.0)
    c0 = torch.from_numpy(synth.pick_centroids(33, rgb, 16, 5)).to(dev)
    pts = torch.from_numpy(rgb.reshape(-1, 3).copy()).to(dev)
    n = w * h
    ref_lab, ref_c = _workspace_run(torch, pts, _native.LAYOUT_RGB8, 5, n, w, c0, (n,), 6)
    lab, cent = _noalloc_run(torch, pts, _native.LAYOUT_RGB8, 5, n, w, c0, (n,), 6)
    assert torch.equal(lab, ref_lab)
    assert torch.equal(cent, ref_c)


def test_noalloc_rejects_what_its_array_cannot_hold():
    """More than 64 clusters (or a dimension other than 3 and 5) would need
    more state than the array holds: refused before any work is queued."""
    torch = pytest.importorskip("torch")
    lib = _native.load()
    dev = torch.device("cuda", 0)
    w = h = 64
    pts = torch.zeros((w * h, 3), dtype=torch.uint8, device=dev)
    lab = torch.zeros(w * h, dtype=torch.int32, device=dev)
    for k, dim in ((65, 3), (8, 4)):
        cent = torch.zeros((dim, k), dtype=torch.float32, device=dev)
        st = lib.split_kmeans_cluster_noalloc(_ptr(pts), _native.LAYOUT_RGB8, dim, w * h, w,
                                              0.1, _ptr(cent), k, _ptr(lab), 1, -1.0, None,
                                              None, None)
        assert st == _native.ERR_INVALID, (k, dim)
