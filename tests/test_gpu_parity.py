"""GPU parity tests: the CUDA path through the C ABI against the oracle."""
import numpy as np
import pytest

import oracle
from split_gb300 import synth

pytestmark = pytest.mark.gpu


def _t(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


# ---------------------------------------------------------------- k-means
@pytest.mark.parametrize("dim,layout", [(3, 0), (3, 1), (3, 2), (5, 0), (5, 1), (5, 2)])
def test_kmeans_lockstep(cuda, dim, layout):
    import torch
    from split_gb300 import kmeans
    w, h, k = 200, 150, 8
    rgb = synth.voronoi_rgb8(7, w, h, 32, sigma=4.0)
    feats = synth.features(rgb, dim)
    c0 = synth.pick_centroids(7, rgb, k, dim)
    if layout == 0:
        pts = _t(feats, cuda)
    elif layout == 1:
        f4 = np.zeros((w * h, 4), np.float32)
        f4[:, :3] = feats[:3].T
        pts = _t(f4, cuda)
    else:
        pts = _t(rgb.reshape(-1, 3), cuda)
    cent = _t(c0, cuda)
    labels = torch.empty(w * h, dtype=torch.int32, device=cuda)
    ws = None
    c = c0.copy()
    for it in range(6):
        ws = kmeans.cluster(pts, cent, labels, ws, max_iter=1, threshold=-1.0, layout=layout,
                            dim=dim, width=w)
        gl = labels.cpu().numpy()
        gc = cent.cpu().numpy()
        exact = oracle.kmeans_assign_f32(feats, c)
        assert np.array_equal(gl, exact), f"iteration {it}: labels differ from the f32 oracle"
        ref, cnt = oracle.kmeans_update_f64(gl, feats, c)
        assert (cnt > 0).all()
        rel = np.abs(gc - ref) / np.maximum(np.abs(ref), 1e-30)
        assert rel.max() <= 1e-5, f"iteration {it}: centroid rel err {rel.max():.3g}"
        c = gc
    ws.check("kmeans")


def test_kmeans_full_run_equals_steps(cuda):
    import torch
    from split_gb300 import kmeans
    w, h, k = 160, 120, 8
    rgb = synth.voronoi_rgb8(3, w, h, 32, sigma=4.0)
    pts = _t(rgb.reshape(-1, 3), cuda)
    c0 = synth.pick_centroids(3, rgb, k, 5)
    a = _t(c0, cuda)
    la = torch.empty(w * h, dtype=torch.int32, device=cuda)
    kmeans.cluster(pts, a, la, None, max_iter=10, threshold=-1.0, layout=2, dim=5, width=w)
    b = _t(c0, cuda)
    lb = torch.empty_like(la)
    for _ in range(10):
        kmeans.cluster(pts, b, lb, None, max_iter=1, threshold=-1.0, layout=2, dim=5, width=w)
    assert torch.equal(a, b) and torch.equal(la, lb)


# ---------------------------------------------------------------- CCL
@pytest.mark.parametrize("shape", [(1, 1), (1, 37), (41, 1), (97, 131), (256, 256), (67, 300)])
@pytest.mark.parametrize("conn", [4, 8])
@pytest.mark.parametrize("conv", [0, 1])
def test_ccl_random(cuda, shape, conn, conv):
    import torch
    from split_gb300 import ccl
    rng = np.random.default_rng(shape[0] * 1000 + shape[1])
    lab = rng.integers(0, 3, size=shape).astype(np.int32)
    out = torch.empty(shape, dtype=torch.int32, device=cuda)
    ccl.connected_components(_t(lab, cuda), None, out, connectivity=conn, convention=conv)
    assert np.array_equal(out.cpu().numpy(), oracle.ccl(lab, conn, conv))


def test_ccl_maze(cuda):
    import torch
    from split_gb300 import ccl
    lab = synth.maze_labels(11, 512, 384)
    for conn in (4, 8):
        out = torch.empty(lab.shape, dtype=torch.int32, device=cuda)
        sizes = torch.zeros(lab.size, dtype=torch.int32, device=cuda)
        ccl.connected_components(_t(lab, cuda), None, out, connectivity=conn, convention=0,
                                 sizes=sizes)
        ref = oracle.ccl(lab, conn, 0)
        got = out.cpu().numpy()
        assert np.array_equal(got, ref)
        roots, counts = np.unique(ref, return_counts=True)
        assert np.array_equal(sizes.cpu().numpy()[roots], counts)


# ---------------------------------------------------------------- merge
@pytest.mark.parametrize("policy", [0, 1])
def test_merge_small(cuda, policy):
    import torch
    from split_gb300 import ccl
    w, h = 240, 180
    rng = np.random.default_rng(5)
    lab = rng.integers(0, 4, size=(h // 4, w // 4)).repeat(4, 0).repeat(4, 1)
    lab[rng.random((h, w)) < 0.05] = 7
    seg = oracle.ccl(lab.astype(np.int32), 8, 0)
    chroma = (rng.integers(0, 256, size=(2, h * w)) / 256.0).astype(np.float32)
    ref = oracle.merge_small(seg, 24, policy, chroma)
    g = _t(seg, cuda)
    ccl.merge_small_segments(_t(chroma, cuda), g, None, 24, policy=policy)
    assert np.array_equal(g.cpu().numpy(), ref)


# ---------------------------------------------------------------- erosion / normals
@pytest.mark.parametrize("shape", [(64, 64), (67, 129), (3, 5), (200, 320)])
@pytest.mark.parametrize("radius", [1, 2, 3])
def test_erode(cuda, shape, radius):
    import torch
    from split_gb300 import morph
    rng = np.random.default_rng(shape[0] + radius)
    lab = rng.integers(0, 3, size=(shape[0] // 3 + 1, shape[1] // 3 + 1)).repeat(3, 0).repeat(3, 1)
    lab = np.ascontiguousarray(lab[: shape[0], : shape[1]]).astype(np.int32)
    out = morph.erode(_t(lab, cuda), radius, out=torch.empty(shape, dtype=torch.int32,
                                                            device=cuda))
    assert np.array_equal(out.cpu().numpy(), oracle.erode(lab, radius))


@pytest.mark.parametrize("shape", [(64, 64), (67, 129), (1, 1), (2, 3), (130, 256)])
def test_sobel_normals(cuda, shape):
    import torch
    from split_gb300 import sfs
    rng = np.random.default_rng(shape[0])
    hgt = rng.random(shape, dtype=np.float32)
    out = torch.empty((3, hgt.size), dtype=torch.float32, device=cuda)
    sfs.sobel_normals(_t(hgt, cuda), out, 1.0)
    ref = oracle.sobel_normals_f64(hgt, 1.0)
    got = out.cpu().numpy().astype(np.float64)
    cosang = np.clip((got * ref).sum(0) / np.linalg.norm(got, axis=0), -1, 1)
    assert np.arccos(cosang).max() <= 1e-4


# widths: 256 (TMA staging); 257, 333, 98, 1 (row pitch not a multiple of 16
# bytes: plain staging, with rows at every 4-byte misalignment)
@pytest.mark.parametrize("w,h", [(256, 96), (257, 95), (333, 71), (98, 40), (1, 9)])
def test_sobel_normals_rgb8(cuda, w, h):
    import torch
    from split_gb300 import sfs
    rgb = synth.voronoi_rgb8(9 + w, w, h, 16, sigma=3.0)
    out = torch.empty((3, w * h), dtype=torch.float32, device=cuda)
    sfs.sobel_normals_rgb8(_t(rgb, cuda), out, 1.0)
    lum = oracle.luminance_f64(rgb).reshape(h, w)
    # FP64 normals of the FP64 luminance; the device computes L* in FP32
    ref = oracle.sobel_normals_f64(lum.astype(np.float32), 1.0)
    got = out.cpu().numpy().astype(np.float64)
    cosang = np.clip((got * ref).sum(0) / np.linalg.norm(got, axis=0), -1, 1)
    assert np.arccos(cosang).max() <= 1e-4


# With float4 features and normals both requested, the pipeline writes the
# features in the normals pass (one read of the bytes).  Everything must equal
# a run that packs the features alone, and the normals the standalone RGB8
# normals, bit for bit.  Widths cover TMA staging (512) and plain staging.
@pytest.mark.parametrize("w,h", [(512, 384), (333, 250), (98, 61)])
def test_pipeline_features_in_normals_pass_match_separate_passes(cuda, w, h):
    import torch
    from split_gb300 import pipeline, sfs
    rgb = synth.voronoi_rgb8(41 + w, w, h, 24, sigma=4.0)
    c0 = synth.pick_centroids(41 + w, rgb, 16, 5)
    g = _t(rgb, cuda)
    fused = pipeline.Pipeline(w, h, pipeline.Params(merge_P=64), cuda)
    fused.run(g, _t(c0, cuda))
    sep = pipeline.Pipeline(w, h, pipeline.Params(merge_P=64, compute_normals=False), cuda)
    sep.run(g, _t(c0, cuda))
    ref = torch.empty((3, w * h), dtype=torch.float32, device=cuda)
    sfs.sobel_normals_rgb8(g, ref, 1.0)
    torch.cuda.synchronize()
    fused.ws.check("fused pipeline")
    sep.ws.check("separate passes")
    assert torch.equal(fused.cluster_labels, sep.cluster_labels)
    assert torch.equal(fused.segment_labels, sep.segment_labels)
    assert torch.equal(fused.centroids, sep.centroids)
    assert torch.equal(fused.normals.view(3, -1), ref)


@pytest.mark.parametrize("k", [1, 5, 16, 33, 64])
def test_kmeans_assign_pruning_exact(cuda, k):
    """Candidate pruning must not change any argmin: arbitrary planar 5-D
    features (negative values, duplicates, NaN rows) against the exact
    FP32 oracle."""
    import torch
    from split_gb300 import kmeans
    rng = np.random.default_rng(k)
    n = 70001
    pts = rng.normal(0, 3, size=(5, n)).astype(np.float32)
    pts[:, 100:200] = pts[:, 100:101]          # duplicates
    pts[2, 5000:5100] = np.nan                 # NaN features
    cent = rng.normal(0, 3, size=(5, k)).astype(np.float32)
    if k > 1:
        cent[:, 1] = cent[:, 0]                # duplicate centroid: ties
    lab = torch.empty(n, dtype=torch.int32, device=cuda)
    kmeans.label_points(_t(cent, cuda), _t(pts, cuda), lab, None, dim=5)
    assert np.array_equal(lab.cpu().numpy(), oracle.kmeans_assign_f32(pts, cent))


def test_kmeans_unit_range_flag(cuda):
    """The unit-range promise on packed features changes no label.  It moves
    whole spans onto the fast path, whose spans with two candidate clusters
    sum in another fixed order than the per-batch path: the centroids agree
    to a few ulp (and each run is deterministic)."""
    import torch
    from split_gb300 import color, kmeans
    w, h = 333, 211
    rgb = synth.voronoi_rgb8(21, w, h, 40, npalette=8, illum_gradient=True, sigma=3.0)
    d_rgb = _t(rgb, cuda)
    f4 = torch.empty((w * h, 4), dtype=torch.float32, device=cuda)
    color.pack_rgb8(d_rgb, f4)
    c0 = _t(synth.pick_centroids(21, rgb, 12, 5), cuda)
    out = []
    for layout in (kmeans.FLOAT4, kmeans.FLOAT4 | kmeans.UNIT_RANGE, kmeans.RGB8):
        cent = c0.clone()
        lab = torch.empty(w * h, dtype=torch.int32, device=cuda)
        pts = d_rgb.view(-1, 3) if layout == kmeans.RGB8 else f4
        kmeans.cluster(pts, cent, lab, None, max_iter=5, threshold=-1.0, layout=layout, dim=5,
                       width=w)
        out.append((lab.cpu().numpy(), cent.cpu().numpy()))
    for lab, cent in out[1:]:
        assert np.array_equal(lab, out[0][0])
        rel = np.abs(cent - out[0][1]) / np.maximum(np.abs(out[0][1]), 1e-30)
        assert rel.max() <= 1e-6, rel.max()
    # the per-batch paths (float4 without the promise, and RGB8 at a width
    # that is not a multiple of 4) are the same computation
    assert np.array_equal(out[2][1], out[0][1])


def test_workspace_reuse_across_sizes(cuda):
    """One workspace serving images of different sizes in turn (its internal
    layout moves with the size): merge and whole-pipeline results stay exact."""
    import torch
    from split_gb300 import ccl, pipeline
    from split_gb300._util import Workspace
    rng = np.random.default_rng(77)
    ws = Workspace(ccl.merge_small_segments_workspace(700, 500), cuda)
    for (w, h) in [(700, 500), (123, 77), (640, 480), (31, 900), (700, 500)]:
        lab = rng.integers(0, 4, size=(h // 3 + 1, w // 3 + 1)).repeat(3, 0).repeat(3, 1)
        lab = np.ascontiguousarray(lab[:h, :w]).astype(np.int32)
        lab[rng.random(lab.shape) < 0.03] = 9
        seg = oracle.ccl(lab, 8, 0)
        g = _t(seg, cuda)
        ccl.merge_small_segments(None, g, ws, 20, policy=ccl.MOST_BOUNDARY)
        assert np.array_equal(g.cpu().numpy(), oracle.merge_small(seg, 20, 0)), (w, h)
        ws.check("merge")
    params = pipeline.Params(merge_P=64)
    big = pipeline.Pipeline(512, 384, params, cuda)
    import ctypes as C
    from split_gb300 import _native as N
    from split_gb300._util import ptr, stream_handle
    for i, (w, h) in enumerate([(512, 384), (200, 100), (333, 250), (512, 384)]):
        rgb = synth.voronoi_rgb8(300 + i, w, h, 24, sigma=4.0)
        c0 = synth.pick_centroids(300 + i, rgb, 16, 5)
        alone = pipeline.Pipeline(w, h, params, cuda)
        alone.run(_t(rgb, cuda), _t(c0, cuda))
        cent = _t(c0, cuda)
        out = [torch.empty(w * h, dtype=torch.int32, device=cuda) for _ in range(2)]
        nrm = torch.empty(3 * w * h, dtype=torch.float32, device=cuda)
        cp = params.c()
        st = N.load().split_pipeline_run(ptr(_t(rgb, cuda)), w, h, C.byref(cp), ptr(cent),
                                         ptr(out[0]), ptr(out[1]), ptr(nrm), big.ws.ptr,
                                         big.ws.nbytes, None, stream_handle())
        assert st == 0
        torch.cuda.synchronize()
        assert torch.equal(out[1].view(h, w), alone.segment_labels), (w, h)
        assert torch.equal(cent, alone.centroids), (w, h)
        big.ws.check("pipeline")


# ---------------------------------------------------------------- edge cases
@pytest.mark.parametrize("radius", [5, 8, 16, 17, 29, 40])
def test_erode_large_radius(cuda, radius):
    """Up to 16 in one kernel pass; beyond that the binding runs passes of at
    most 16 (out-of-place and in place, as the reference's erode(labels, n))."""
    import torch
    from split_gb300 import morph
    rng = np.random.default_rng(radius)
    lab = rng.integers(0, 3, size=(12, 15)).repeat(41, 0).repeat(37, 1)[:470, :537]
    lab = np.ascontiguousarray(lab).astype(np.int32)
    want = oracle.erode(lab, radius)
    assert (want >= 0).any()
    d = _t(lab, cuda)
    out = morph.erode(d, radius, out=torch.empty(lab.shape, dtype=torch.int32, device=cuda))
    assert np.array_equal(out.cpu().numpy(), want)
    assert np.array_equal(d.cpu().numpy(), lab)          # the input is left alone
    morph.erode(d, radius)                                 # in place
    assert np.array_equal(d.cpu().numpy(), want)


@pytest.mark.parametrize("fill", ["uniform", "checker"])
def test_ccl_degenerate_images(cuda, fill):
    """One component covering the image, and every pixel its own component
    under 4-connectivity (a checkerboard joins diagonally under 8)."""
    import torch
    from split_gb300 import ccl
    h, w = 333, 517
    if fill == "uniform":
        lab = np.full((h, w), 5, np.int32)
    else:
        lab = ((np.arange(h)[:, None] + np.arange(w)[None, :]) % 2).astype(np.int32)
    for conn in (4, 8):
        for conv in (0, 1):
            out = torch.empty((h, w), dtype=torch.int32, device=cuda)
            ccl.connected_components(_t(lab, cuda), None, out, connectivity=conn,
                                     convention=conv)
            assert np.array_equal(out.cpu().numpy(), oracle.ccl(lab, conn, conv))


@pytest.mark.parametrize("policy", [0, 1])
def test_merge_all_small_and_none_small(cuda, policy):
    import torch
    from split_gb300 import ccl
    rng = np.random.default_rng(9)
    h, w = 96, 160
    lab = rng.integers(0, 6, size=(h // 2, w // 2)).repeat(2, 0).repeat(2, 1).astype(np.int32)
    seg = oracle.ccl(lab, 8, 0)
    chroma = (rng.integers(0, 256, size=(2, h * w)) / 256.0).astype(np.float32)
    for P in (1, h * w + 1):          # nothing small / everything small
        ref = oracle.merge_small(seg, P, policy, chroma)
        g = _t(seg, cuda)
        ccl.merge_small_segments(_t(chroma, cuda), g, None, P, policy=policy)
        assert np.array_equal(g.cpu().numpy(), ref), P


def test_kmeans_k64_many_iterations(cuda):
    """K at its maximum (64) over 5-D features, 32 iterations, in lockstep:
    labels equal the FP32-exact assignment, centroids the FP64 update of the
    device's labels (empty clusters keep their centroid on both sides)."""
    import torch
    from split_gb300 import kmeans
    w, h, k = 300, 211, 64
    rgb = synth.voronoi_rgb8(77, w, h, 150, npalette=40, illum_gradient=True, sigma=5.0)
    feats = synth.features(rgb, 5)
    c = synth.pick_centroids(77, rgb, k, 5)
    pts = _t(feats, cuda)
    cent = _t(c, cuda)
    labels = torch.empty(w * h, dtype=torch.int32, device=cuda)
    ws = None
    for it in range(32):
        ws = kmeans.cluster(pts, cent, labels, ws, max_iter=1, threshold=-1.0, layout=0,
                            dim=5, width=w)
        gl = labels.cpu().numpy()
        gc = cent.cpu().numpy()
        assert np.array_equal(gl, oracle.kmeans_assign_f32(feats, c)), f"iteration {it}"
        ref, _ = oracle.kmeans_update_f64(gl, feats, c)
        rel = np.abs(gc - ref) / np.maximum(np.abs(ref), 1e-30)
        assert rel.max() <= 1e-5, f"iteration {it}: centroid rel err {rel.max():.3g}"
        c = gc
    ws.check("kmeans")


def test_ccl_stress_8192_maze(cuda):
    """Labelling stress case: 8192 x 8192 maze (one serpentine corridor over
    half the image, path > 10^7 px) plus random wall blobs; 4- and
    8-connected, both conventions, bit-exact, with component sizes."""
    import torch
    from split_gb300 import ccl
    n = 8192
    lab = synth.maze_labels(2024, n, n)
    d_lab = _t(lab, cuda)
    out = torch.empty((n, n), dtype=torch.int32, device=cuda)
    sizes = torch.zeros(n * n, dtype=torch.int32, device=cuda)
    ws = None
    for conn in (4, 8):
        for conv in (0, 1):
            sizes.zero_()
            ws = ccl.connected_components(d_lab, ws, out, connectivity=conn, convention=conv,
                                          sizes=sizes)
            ref = oracle.ccl(lab, conn, conv)
            got = out.cpu().numpy()
            assert np.array_equal(got, ref), (conn, conv)
            roots, counts = np.unique(ref, return_counts=True)
            assert np.array_equal(sizes.cpu().numpy()[roots], counts)
            if conn == 4 and conv == 0:
                assert counts.max() > n * n // 3       # the serpentine corridor
                assert len(roots) > 10 ** 4
    ws.check("ccl")


def test_merge_stress_8192_maze(cuda):
    """Merge stress case: the 8192 x 8192 maze's 8-connected components (the
    corridor and 1.39 M pieces of its random blobs, 108,519 of them at least
    64 px) merged below 64 px into the neighbour sharing most boundary,
    bit-exact against the oracle."""
    import torch
    from split_gb300 import ccl
    n = 8192
    lab = synth.maze_labels(2024, n, n)
    seg = oracle.ccl(lab, 8, 0)
    g = _t(seg, cuda)
    ws = ccl.merge_small_segments(None, g, None, 64, policy=ccl.MOST_BOUNDARY)
    torch.cuda.synchronize()
    ws.check("merge")
    want = oracle.merge_small(seg, 64, 0)
    got = g.cpu().numpy()
    assert np.array_equal(got, want), f"{int((got != want).sum())} labels differ"
    assert len(np.unique(want)) < len(np.unique(seg))


@pytest.mark.parametrize("layout,dim", [(0, 3), (1, 3), (2, 3), (2, 5), (0, 5)])
def test_segment_means_many_clusters(cuda, layout, dim):
    """calculate_centroids with K = number of segments (thousands): per-segment
    FP64 means of the member features within 1e-5 relative; empty segments
    keep their input centroid; eroded (-1) pixels are ignored; the result
    does not depend on the run (fixed-point sums)."""
    import torch
    from split_gb300 import kmeans
    w, h = 517, 333
    rgb = synth.voronoi_rgb8(88, w, h, 600, sigma=4.0)
    feats = synth.features(rgb, dim)
    seg = oracle.ccl(oracle.kmeans_assign_f32(
        synth.features(rgb, 3), synth.pick_centroids(88, rgb, 8, 3)).reshape(h, w), 8, 0)
    lab, nseg = oracle.compress_labels(seg)
    lab = lab.reshape(-1).astype(np.int32)
    lab[::97] = -1                          # eroded pixels
    k = nseg + 5                            # a few empty clusters at the end
    assert k > 64
    c_in = np.random.default_rng(1).random((dim, k)).astype(np.float32)
    if layout == 0:
        pts = _t(feats, cuda)
    elif layout == 1:
        f4 = np.zeros((w * h, 4), np.float32)
        f4[:, :3] = feats[:3].T
        pts = _t(f4, cuda)
    else:
        pts = _t(rgb.reshape(-1, 3), cuda)
    outs = []
    for _ in range(2):
        cent = _t(c_in, cuda)
        kmeans.calculate_centroids(_t(lab, cuda), pts, cent, layout=layout, dim=dim, width=w)
        outs.append(cent.cpu().numpy())
    assert np.array_equal(outs[0], outs[1])
    got = outs[0]
    ref, cnt = oracle.kmeans_update_f64(lab, feats, c_in)
    assert (cnt[nseg:] == 0).all() and (cnt > 0).sum() > 64
    # clusters without members (the trailing ones, and segments whose pixels
    # were all marked eroded) keep their input centroid exactly
    np.testing.assert_array_equal(got[:, cnt == 0], c_in[:, cnt == 0])
    rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-30)
    assert rel.max() <= 1e-5


@pytest.mark.parametrize("threshold", [0.01, 0.02, 0.1])
def test_merge_smooth_boundaries(cuda, threshold):
    """Smooth-boundary merge, bit-exact against the oracle on seeded blobs
    with Lab-like features (L in [0, 100], a, b in [-60, 60]) plus noise."""
    import torch
    from split_gb300 import ccl
    w, h = 300, 211
    rng = np.random.default_rng(int(threshold * 1000))
    blocks = rng.integers(0, 6, size=(h // 6 + 1, w // 6 + 1)).repeat(6, 0).repeat(6, 1)[:h, :w]
    seg = oracle.ccl(blocks.astype(np.int32), 8, 0)
    # block classes c and c + 3 share a colour: adjacent segments of those
    # classes have smooth boundaries, the others sharp ones
    base = np.stack([rng.uniform(0, 100, 3), rng.uniform(-60, 60, 3), rng.uniform(-60, 60, 3)])
    pts = base[:, (blocks % 3).ravel()] + rng.normal(0, 0.5, size=(3, w * h))
    pts = np.ascontiguousarray(pts, dtype=np.float32)
    ref = oracle.merge_smooth(seg, pts, threshold)
    g = _t(seg, cuda)
    ws = ccl.merge_smooth_boundaries(_t(pts, cuda), 0, g, None, threshold)
    got = g.cpu().numpy()
    ws.check("merge_smooth")
    assert np.array_equal(got, ref)
    assert len(np.unique(ref)) < len(np.unique(seg))      # something merged
    # the workspace is left clean: a second call on the merged labels agrees too
    ref2 = oracle.merge_smooth(ref, pts, threshold)
    ccl.merge_smooth_boundaries(_t(pts, cuda), 0, g, ws, threshold)
    assert np.array_equal(g.cpu().numpy(), ref2)


def test_pipeline_lab_beta_features(cuda):
    """The pipeline with the sample's (beta, a*, b*) features: the features
    equal the fused pack's, the k-means labels are the FP32-exact assignment
    of the final iteration's input over them, and the integer stages match
    the oracle given those labels."""
    import os
    import sys
    import torch
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_golden
    from split_gb300 import _native, color, kmeans, pipeline
    rgb = make_golden.lab_beta_inputs()
    h, w = rgb.shape[:2]
    n = w * h
    d_rgb = torch.from_numpy(rgb).to(cuda)
    f4 = torch.empty((n, 4), dtype=torch.float32, device=cuda)
    color.pack_lab_beta(d_rgb, f4)
    feats = f4[:, :3].T.contiguous().cpu().numpy()
    k = 6
    c0 = feats[:, np.linspace(0, n - 1, k).astype(int)].copy()
    p = pipeline.Params(nclusters=k, dim=3, kmeans_iters=8, features=_native.FEATURES_LAB_BETA,
                        merge_P=32)
    pipe = pipeline.Pipeline(w, h, p, cuda)
    pipe.run(d_rgb, torch.from_numpy(c0).to(cuda))
    torch.cuda.synchronize()
    pipe.ws.check("pipeline")
    # the same clustering through the k-means entry point on the packed features
    cent = torch.from_numpy(c0).to(cuda)
    lab = torch.empty(n, dtype=torch.int32, device=cuda)
    kmeans.cluster(f4, cent, lab, None, max_iter=8, threshold=-1.0, layout=kmeans.FLOAT4,
                   dim=3, width=w)
    cl = pipe.cluster_labels.cpu().numpy()
    assert np.array_equal(cl, lab.cpu().numpy())
    assert np.array_equal(pipe.centroids.cpu().numpy(), cent.cpu().numpy())
    seg = oracle.ccl(cl.reshape(h, w), 8, 0)
    seg = oracle.merge_small(seg, 32, 0)
    assert np.array_equal(pipe.segment_labels.cpu().numpy(), oracle.erode(seg, 1))


@pytest.mark.parametrize("shape,light,lam,tol", [((24, 32), (0.3, -0.2, 1.0), 0.5, 1e-5),
                                                ((61, 47), (-1.0, 0.5, 2.0), 1.0, 1e-6),
                                                ((1, 40), (0.0, 0.0, 1.0), 0.25, 1e-5),
                                                ((33, 1), (0.2, 0.9, 0.4), 2.0, 1e-5)])
def test_estimate_normals(cuda, shape, light, lam, tol):
    """SOR shape-from-shading normals against the FP64 restatement of the same
    relaxation: within 1e-4 rad, sweep counts within one, unit length, z >= 0."""
    import torch
    from split_gb300 import sfs
    rng = np.random.default_rng(shape[0] * 7 + shape[1])
    s = rng.random(shape, dtype=np.float32)
    ref, ref_it = oracle.estimate_normals_rb(s, light, lam, 5000, tol)
    out = torch.empty((3, s.size), dtype=torch.float32, device=cuda)
    its = torch.zeros(1, dtype=torch.int32, device=cuda)
    ws = sfs.estimate_normals(_t(s, cuda), light, out, lam, max_iter=5000, tol=tol,
                              iterations_out=its)
    torch.cuda.synchronize()
    ws.check("estimate_normals")
    got = out.cpu().numpy().astype(np.float64)
    assert abs(int(its.item()) - ref_it) <= 1, (int(its.item()), ref_it)
    np.testing.assert_allclose(np.linalg.norm(got, axis=0), 1.0, atol=1e-6)
    assert (got[2] >= 0).all()
    ang = np.arctan2(np.linalg.norm(np.cross(got.T, ref.T), axis=1), (got * ref).sum(0))
    assert ang.max() <= 1e-4


def test_estimate_normals_limits(cuda):
    import torch
    from split_gb300 import _native, sfs
    s = torch.rand((8, 8), device=cuda)
    out = torch.empty((3, 64), device=cuda)
    sfs.estimate_normals(s, (1.0, 1.0, 1.0), out, 0.5, max_iter=0)   # no sweep: x0
    torch.cuda.synchronize()
    assert torch.equal(out[2], torch.ones(64, device=cuda)) and (out[:2] == 0).all()
    with pytest.raises(_native.SplitError):
        sfs.estimate_normals(s, (1.0, 1.0, 1.0), out, 0.0)       # no smoothness: singular
    with pytest.raises(_native.SplitError):
        sfs.estimate_normals(s, (0.0, 0.0, 0.0), out, 0.5)       # no light direction


def test_pipeline_reference_chroma_merge(cuda):
    """The pipeline with the reference's chroma merge rule: the merge reads
    the sample's r / intensity plane (rgb_to_ic), and the segment labels
    equal the oracle's CCL -> chroma merge -> erosion of the pipeline's own
    k-means labels."""
    import torch
    from split_gb300 import _native, pipeline
    w, h = 301, 187
    # colour-only features on a noisy image: hundreds of small fragments
    rgb = synth.voronoi_rgb8(91, w, h, 60, sigma=8.0)
    p = pipeline.Params(nclusters=12, dim=3, kmeans_iters=6, merge_P=48,
                        merge_policy=_native.MERGE_REF_CHROMA)
    c0 = synth.pick_centroids(91, rgb, p.nclusters, p.dim)
    pipe = pipeline.Pipeline(w, h, p, cuda)
    pipe.run(torch.from_numpy(rgb).to(cuda), torch.from_numpy(c0).to(cuda))
    torch.cuda.synchronize()
    pipe.ws.check("pipeline")
    cl = pipe.cluster_labels.cpu().numpy().reshape(h, w)
    seg = oracle.ccl(cl, 8, 0)
    chroma = oracle.rgb_to_ic_f32(rgb)[1:]
    merged = oracle.merge_small(seg, 48, 1, chroma)
    assert len(np.unique(merged)) < len(np.unique(seg))     # something merged
    # and the rule is the chroma one, not the boundary one
    assert not np.array_equal(merged, oracle.merge_small(seg, 48, 0))
    assert np.array_equal(pipe.segment_labels.cpu().numpy(), oracle.erode(merged, 1))


@pytest.mark.parametrize("shape,policy", [((2160, 3840), 0), ((311, 97), 0), ((311, 97), 1),
                                          ((1, 5000), 0)])
def test_merge_every_pixel_its_own_segment(cuda, shape, policy):
    """Every pixel its own segment (all smaller than P): about 8 distinct
    (segment, neighbour) pairs per pixel, far more than the pair table holds
    at once.  The merge decides the segments in rounds over hash classes and
    equals the oracle (which sorts every edge), bit for bit; a workspace
    reused afterwards for a normal image is still exact."""
    import torch
    from split_gb300 import ccl
    h, w = shape
    rng = np.random.default_rng(h + w)
    # ids in raster order, or shuffled for the chroma rule (which leaves
    # labels already in sorted order as they are)
    ids = np.arange(h * w, dtype=np.int32)
    lab = (rng.permutation(ids) if policy else ids).astype(np.int32).reshape(h, w)
    chroma = (rng.integers(0, 256, size=(2, h * w)) / 256.0).astype(np.float32)
    g = _t(lab, cuda)
    ws = ccl.merge_small_segments(_t(chroma, cuda) if policy else None, g, None, 4,
                                  policy=policy)
    torch.cuda.synchronize()
    ws.check("merge")
    want = oracle.merge_small(lab, 4, policy, chroma if policy else None)
    assert np.array_equal(g.cpu().numpy(), want)
    # the same workspace on an ordinary image afterwards
    blk = rng.integers(0, 4, size=(h // 4 + 1, w // 4 + 1)).repeat(4, 0).repeat(4, 1)[:h, :w]
    seg = oracle.ccl(np.ascontiguousarray(blk).astype(np.int32), 8, 0)
    g2 = _t(seg, cuda)
    ccl.merge_small_segments(None, g2, ws, 24, policy=0)
    ws.check("merge after")
    assert np.array_equal(g2.cpu().numpy(), oracle.merge_small(seg, 24, 0))


@pytest.mark.parametrize("layout", [1, 2])
def test_kmeans_kept_span_sums_change_nothing(cuda, layout):
    """The span sums kept from the first iteration are the same integers as
    freshly summed ones: a workspace with room for them, one without (the
    clustering state only), and a reused workspace that last held another
    image's sums all give bit-identical labels and centroids."""
    import torch
    from split_gb300 import _native, kmeans
    from split_gb300._util import Workspace
    lib = _native.load()
    w, h, k, iters = 640, 480, 16, 8
    rgb = synth.voronoi_rgb8(19, w, h, 96, npalette=16, sigma=3.0)
    other = synth.voronoi_rgb8(20, w, h, 40, npalette=8, sigma=5.0)
    c0 = synth.pick_centroids(19, rgb, k, 5)
    n = w * h

    def points(img):
        if layout == 2:
            return _t(img.reshape(-1, 3), cuda)
        f4 = np.zeros((n, 4), np.float32)
        f4[:, :3] = synth.features(img, 3).T
        return _t(f4, cuda)

    lay = layout | (kmeans.UNIT_RANGE if layout == 1 else 0)
    full = Workspace(lib.split_kmeans_cluster_workspace_size_2d(n, w, k, 5), cuda)
    small = Workspace(lib.split_kmeans_assign_workspace_size(n, k), cuda)
    assert small.nbytes < full.nbytes
    def run(ws, img):
        # through the C ABI: the Python wrapper would replace a small workspace
        pts = points(img)
        cent = _t(c0, cuda)
        lab = torch.empty(n, dtype=torch.int32, device=cuda)
        _native.check(lib.split_kmeans_cluster(pts.data_ptr(), lay, 5, n, w, 0.1,
                                               cent.data_ptr(), k, lab.data_ptr(), ws.ptr,
                                               ws.nbytes, iters, -1.0, None, None), "cluster")
        torch.cuda.synchronize()
        ws.check("kmeans")
        return lab.cpu().numpy(), cent.cpu().numpy()

    out = [run(full, rgb), run(small, rgb)]
    run(full, other)            # leave another image's sums in the workspace
    out.append(run(full, rgb))
    for lab, cent in out[1:]:
        assert np.array_equal(lab, out[0][0]) and np.array_equal(cent, out[0][1])
