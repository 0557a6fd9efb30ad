"""label_points and cluster with more than 64 clusters (the reference's
label.cu:74-106 and cluster.cu:27-93 set no limit on K): the many-cluster
path against the oracle's FP32-exact assignment and FP64 update."""
import numpy as np
import pytest

import oracle
from split_gb300 import synth

pytestmark = pytest.mark.gpu


def _t(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def _points(rgb, feats, layout, dev):
    w, h = rgb.shape[1], rgb.shape[0]
    if layout == 0:
        return _t(feats, dev)
    if layout == 1:
        f4 = np.zeros((w * h, 4), np.float32)
        f4[:, :3] = feats[:3].T
        return _t(f4, dev)
    return _t(rgb.reshape(-1, 3), dev)


@pytest.mark.parametrize("k", [65, 300, 2100])
@pytest.mark.parametrize("dim,layout", [(3, 0), (3, 1), (3, 2), (5, 0), (5, 1), (5, 2)])
def test_label_points_many_clusters(cuda, k, dim, layout):
    """Bit-exact labels against the FP32-exact oracle, including exact ties
    (duplicated centroids go to the lower index) and more centroids than one
    shared-memory chunk holds (2100 > 1024 / 2048)."""
    import torch
    from split_gb300 import kmeans
    w, h = 97, 61
    rgb = synth.voronoi_rgb8(11, w, h, 40, sigma=6.0)
    feats = synth.features(rgb, dim)
    c = synth.pick_centroids(5, rgb, k, dim)
    c[:, k - 1] = c[:, 3]          # an exact tie: pixels nearest to 3 stay with 3
    c[:, 40] = c[:, k - 2]         # and one where the lower copy is the later pick
    labels = torch.full((w * h,), -7, dtype=torch.int32, device=cuda)
    ws = kmeans.label_points(_t(c, cuda), _points(rgb, feats, layout, cuda), labels,
                             layout=layout, dim=dim, width=w)
    torch.cuda.synchronize()
    ws.check("label_points")
    exact = oracle.kmeans_assign_f32(feats, c)
    assert np.array_equal(labels.cpu().numpy(), exact)
    assert not (exact == k - 1).any()


@pytest.mark.parametrize("dim,layout", [(3, 0), (3, 2), (5, 1), (5, 2)])
def test_cluster_many_clusters_lockstep(cuda, dim, layout):
    """One iteration per call: labels equal the FP32-exact assignment of the
    GPU's own centroids, and the centroids equal the FP64 mean of those labels
    (empty clusters keep theirs) within 1e-5 relative: features are summed
    exactly after rounding to multiples of 2^-24."""
    import torch
    from split_gb300 import kmeans
    w, h, k = 120, 90, 100
    rgb = synth.voronoi_rgb8(21, w, h, 60, sigma=5.0)
    feats = synth.features(rgb, dim)
    c0 = synth.pick_centroids(21, rgb, k, dim)
    pts = _points(rgb, feats, layout, cuda)
    cent = _t(c0, cuda)
    labels = torch.empty(w * h, dtype=torch.int32, device=cuda)
    its = torch.full((1,), -1, dtype=torch.int32, device=cuda)
    ws, c = None, c0.copy()
    for it in range(5):
        ws = kmeans.cluster(pts, cent, labels, ws, max_iter=1, threshold=-1.0, layout=layout,
                            dim=dim, width=w, iterations_out=its)
        gl, gc = labels.cpu().numpy(), cent.cpu().numpy()
        assert int(its.item()) == 1
        assert np.array_equal(gl, oracle.kmeans_assign_f32(feats, c)), f"iteration {it}"
        ref, cnt = oracle.kmeans_update_f64(gl, feats, c)
        rel = np.abs(gc - ref) / np.maximum(np.abs(ref), 1e-30)
        assert rel.max() <= 1e-5, f"iteration {it}: centroid rel err {rel.max():.3g}"
        assert np.array_equal(gc[:, cnt == 0], c[:, cnt == 0])
        c = gc
    ws.check("kmeans")


def test_cluster_many_clusters_run_equals_steps(cuda):
    """Ten iterations in one call (queued launches, device-side decision)
    equal ten calls of one iteration, bit for bit."""
    import torch
    from split_gb300 import kmeans
    w, h, k = 150, 100, 96
    rgb = synth.voronoi_rgb8(4, w, h, 64, sigma=4.0)
    pts = _t(rgb.reshape(-1, 3), cuda)
    c0 = synth.pick_centroids(4, rgb, k, 5)
    a, la = _t(c0, cuda), torch.empty(w * h, dtype=torch.int32, device=cuda)
    its = torch.full((1,), -1, dtype=torch.int32, device=cuda)
    kmeans.cluster(pts, a, la, None, max_iter=10, threshold=-1.0, layout=2, dim=5, width=w,
                   iterations_out=its)
    b, lb = _t(c0, cuda), torch.empty_like(la)
    for _ in range(10):
        kmeans.cluster(pts, b, lb, None, max_iter=1, threshold=-1.0, layout=2, dim=5, width=w)
    assert int(its.item()) == 10
    assert torch.equal(a, b) and torch.equal(la, lb)


@pytest.mark.parametrize("rule", ["l2", "reference"])
@pytest.mark.parametrize("thr", [1e-3, 1e-2])
def test_cluster_many_clusters_threshold(cuda, rule, thr):
    """cluster(..., 100, threshold) stops at the oracle's iteration, under
    the L2 shift and under the reference's own shift measure."""
    import torch
    from split_gb300 import kmeans
    w, h, k = 128, 96, 80
    rgb = synth.voronoi_rgb8(8, w, h, 50, sigma=5.0)
    feats = synth.features(rgb, 3)
    c0 = synth.pick_centroids(8, rgb, k, 3)
    cent = _t(c0, cuda)
    labels = torch.empty(w * h, dtype=torch.int32, device=cuda)
    its = torch.full((1,), -1, dtype=torch.int32, device=cuda)
    layout = kmeans.PLANAR | (kmeans.REFERENCE_SHIFT if rule == "reference" else 0)
    ws = kmeans.cluster(_t(feats, cuda), cent, labels, None, max_iter=100, threshold=thr,
                        layout=layout, dim=3, width=w, iterations_out=its)
    torch.cuda.synchronize()
    ws.check("kmeans")
    olab, oc, oit, _ = oracle.kmeans_cluster_threshold(feats, c0, 100, thr,
                                                       reference_shift_rule=rule == "reference")
    assert int(its.item()) == oit
    assert (labels.cpu().numpy() != olab).sum() <= 8   # near-ties after ulp-level drift
    rel = np.abs(cent.cpu().numpy() - oc) / np.maximum(np.abs(oc), 1e-30)
    assert rel.max() <= 1e-4


def test_many_clusters_limits(cuda):
    """The reference's shift is 3-D only; zero iterations leave the inputs
    alone and report 0."""
    import torch
    from split_gb300 import _native, kmeans
    w, h = 64, 48
    rgb = synth.voronoi_rgb8(2, w, h, 30)
    pts = _t(rgb.reshape(-1, 3), cuda)
    lab = torch.full((w * h,), -3, dtype=torch.int32, device=cuda)
    c5 = _t(synth.pick_centroids(2, rgb, 70, 5), cuda)
    with pytest.raises(_native.SplitError):
        kmeans.cluster(pts, c5, lab, None, max_iter=5, threshold=1e-3,
                       layout=kmeans.RGB8 | kmeans.REFERENCE_SHIFT, dim=5, width=w)
    before = c5.clone()
    its = torch.full((1,), -1, dtype=torch.int32, device=cuda)
    kmeans.cluster(pts, c5, lab, None, max_iter=0, threshold=-1.0, layout=kmeans.RGB8, dim=5,
                   width=w, iterations_out=its)
    torch.cuda.synchronize()
    assert int(its.item()) == 0
    assert torch.equal(c5, before) and bool((lab == -3).all())


@pytest.mark.parametrize("k", [16, 100])
@pytest.mark.parametrize("layout", [0, 1])
def test_label_points_infinite_features(cuda, k, layout):
    """A pixel with an infinite feature makes its warp's pruning bound
    infinite; the labels still equal the FP32-exact oracle (that pixel gets 0,
    every distance being infinite) and never name a cluster past K."""
    import torch
    from split_gb300 import kmeans
    w, h = 96, 40
    rgb = synth.voronoi_rgb8(13, w, h, 30, sigma=3.0)
    feats = synth.features(rgb, 3)
    c = synth.pick_centroids(13, rgb, k, 3)
    rng = np.random.default_rng(k)
    bad = rng.choice(w * h, 25, replace=False)
    feats[rng.integers(0, 3, bad.size), bad] = np.where(np.arange(bad.size) % 2, np.inf, -np.inf)
    labels = torch.empty(w * h, dtype=torch.int32, device=cuda)
    kmeans.label_points(_t(c, cuda), _points(rgb, feats, layout, cuda), labels,
                        layout=layout, dim=3, width=w)
    exact = oracle.kmeans_assign_f32(feats, c)
    got = labels.cpu().numpy()
    assert np.array_equal(got, exact)
    assert (got[bad] == 0).all() and got.max() < k


def test_cluster_many_clusters_large_features(cuda):
    """Features from 2^32 up (below the fixed-point format's 2^38) take the
    general 96-bit sums instead of the one-word form: one iteration still
    equals the FP32-exact assignment and the FP64 mean."""
    import torch
    from split_gb300 import kmeans
    w, h, k = 90, 70, 72
    rgb = synth.voronoi_rgb8(17, w, h, 40, sigma=5.0)
    feats = synth.features(rgb, 3) * np.float32(2.0 ** 34)
    feats[:, ::7] *= np.float32(1.0 / 1024.0)       # some warps mix small and large values
    c0 = np.ascontiguousarray(feats[:, np.random.default_rng(17).choice(w * h, k, replace=False)])
    cent = _t(c0, cuda)
    labels = torch.empty(w * h, dtype=torch.int32, device=cuda)
    ws = kmeans.cluster(_t(feats, cuda), cent, labels, None, max_iter=1, threshold=-1.0,
                        layout=kmeans.PLANAR, dim=3, width=w)
    torch.cuda.synchronize()
    ws.check("kmeans")
    gl = labels.cpu().numpy()
    assert np.array_equal(gl, oracle.kmeans_assign_f32(feats, c0))
    ref, _ = oracle.kmeans_update_f64(gl, feats, c0)
    rel = np.abs(cent.cpu().numpy() - ref) / np.maximum(np.abs(ref), 1e-30)
    assert rel.max() <= 1e-6


def test_pipeline_many_clusters(cuda):
    """The single-image pipeline with K = 100: its clustering equals a
    standalone cluster() call bit for bit, and labelling, merge and erosion
    equal the oracle's on its cluster labels."""
    import torch
    from split_gb300 import color, kmeans, pipeline
    w, h, k = 320, 200, 100
    rgb = synth.voronoi_rgb8(31, w, h, 120, npalette=24, sigma=3.0)
    c0 = synth.pick_centroids(31, rgb, k, 5)
    params = pipeline.Params(nclusters=k, kmeans_iters=6, merge_P=32)
    pipe = pipeline.Pipeline(w, h, params, cuda)
    d_rgb = _t(rgb, cuda)
    pipe.run(d_rgb, _t(c0, cuda))
    torch.cuda.synchronize()
    pipe.ws.check("pipeline")
    f4 = torch.empty((w * h, 4), dtype=torch.float32, device=cuda)
    color.pack_rgb8(d_rgb, f4)
    cent = _t(c0, cuda)
    lab = torch.empty(w * h, dtype=torch.int32, device=cuda)
    kmeans.cluster(f4, cent, lab, None, max_iter=6, threshold=-1.0,
                   layout=kmeans.FLOAT4 | kmeans.UNIT_RANGE, dim=5, width=w)
    assert torch.equal(lab, pipe.cluster_labels) and torch.equal(cent, pipe.centroids)
    seg = oracle.ccl(lab.cpu().numpy().reshape(h, w), 8, 0)
    want = oracle.erode(oracle.merge_small(seg, 32, 0), 1)
    assert np.array_equal(pipe.segment_labels.cpu().numpy(), want)
