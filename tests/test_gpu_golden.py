"""The CUDA path (through the C ABI) against the reference's own outputs
(tests/golden/reference_golden.npz)."""
import os
import sys

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402

G = np.load(os.path.join(HERE, "golden", "reference_golden.npz"))


@pytest.fixture(scope="module")
def inp():
    return make_golden.inputs()


def _t(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


@pytest.mark.parametrize("name,src", [("ccl_maze", "maze"), ("ccl_blocks", "blocks"),
                                      ("ccl_km", None)])
def test_ccl_reference_convention(cuda, inp, name, src):
    import torch
    from split_gb300 import ccl
    lab = inp[src] if src else G["km_cluster10_labels"].astype(np.int32).reshape(512, 512)
    out = torch.empty(lab.shape, dtype=torch.int32, device=cuda)
    ccl.connected_components(_t(lab, cuda), None, out, connectivity=4, convention=ccl.MAX_INDEX)
    assert np.array_equal(out.cpu().numpy(), G[name])


def test_compress_labels(cuda):
    from split_gb300 import ccl
    lab = _t(G["ccl_blocks"], cuda).view(-1)
    n = ccl.compress_labels(lab)
    assert n == int(G["compress_blocks_count"])
    assert np.array_equal(lab.view(200, 280).cpu().numpy(), G["compress_blocks"])


def test_compress_labels_with_eroded_pixels(cuda):
    # -1 (eroded) ranks first, as the sample expects (main.cu:302-314)
    from split_gb300 import ccl
    lab = G["erode2_blocks"]
    want, n = oracle.compress_labels(lab)
    g = _t(lab, cuda).view(-1)
    assert ccl.compress_labels(g) == n
    assert np.array_equal(g.cpu().numpy(), want.reshape(-1))


def test_merge_reference_chroma(cuda, inp):
    from split_gb300 import ccl
    g = _t(G["compress_blocks"], cuda)
    ccl.merge_small_segments(_t(inp["chroma"], cuda), g, None, 24, policy=ccl.REF_CHROMA)
    assert np.array_equal(g.cpu().numpy(), G["merge_blocks_P24"])


@pytest.mark.parametrize("name,src,r", [("erode1_km", "ccl_km", 1), ("erode2_blocks", "ccl_blocks", 2)])
def test_erode(cuda, name, src, r):
    import torch
    from split_gb300 import morph
    lab = G[src]
    out = morph.erode(_t(lab, cuda), r, out=torch.empty(lab.shape, dtype=torch.int32, device=cuda))
    assert np.array_equal(out.cpu().numpy(), G[name])


def test_sobel_normals(cuda, inp):
    import torch
    from split_gb300 import sfs
    h = inp["heights"]
    out = torch.empty((3, h.size), dtype=torch.float32, device=cuda)
    sfs.sobel_normals(_t(h, cuda), out, 1.0)
    got = out.cpu().numpy().astype(np.float64)
    ref = G["sobel_normals"].astype(np.float64)
    ang = np.arccos(np.clip((got * ref).sum(0) / np.linalg.norm(got, axis=0), -1, 1))
    assert ang.max() <= 1e-3       # the reference's own FP32 drift
    f64 = oracle.sobel_normals_f64(h, 1.0)
    ang = np.arccos(np.clip((got * f64).sum(0) / np.linalg.norm(got, axis=0), -1, 1))
    assert ang.max() <= 1e-4


def test_label_points(cuda, inp):
    import torch
    from split_gb300 import kmeans
    pts, c0 = inp["km_points"], inp["km_c0"]
    lab = torch.empty(pts.shape[1], dtype=torch.int32, device=cuda)
    kmeans.label_points(_t(c0, cuda), _t(pts, cuda), lab, None, width=512)
    _, d1, d2 = oracle.kmeans_assign_f64(pts, c0)
    near = (d2 - d1) <= 1e-5 * d2
    ref = G["km_label_points"].astype(np.int32)
    assert ((lab.cpu().numpy() != ref) & ~near).sum() == 0


def test_cluster_10_iterations(cuda, inp):
    import torch
    from split_gb300 import kmeans
    pts, c0 = inp["km_points"], inp["km_c0"]
    cent = _t(c0, cuda)
    lab = torch.empty(pts.shape[1], dtype=torch.int32, device=cuda)
    kmeans.cluster(_t(pts, cuda), cent, lab, None, max_iter=10, threshold=-1.0, width=512)
    assert (lab.cpu().numpy() != G["km_cluster10_labels"]).mean() <= 1e-3
    rc = G["km_cluster10_centroids"]
    assert (np.abs(cent.cpu().numpy() - rc) / np.abs(rc)).max() <= 1e-3


@pytest.mark.parametrize("planar", [False, True])
def test_lab_beta_features(cuda, planar):
    """Fused Lab + beta features against the reference's own FP32 sequence
    (clamp, rgb_to_lab, beta_feature): L*, a*, b* within 1e-3, beta identical."""
    import torch
    import make_golden
    from split_gb300 import color
    g = np.load(os.path.join(HERE, "golden", "lab_beta_golden.npz"))
    rgb = make_golden.lab_beta_inputs()
    n = rgb.shape[0] * rgb.shape[1]
    d_rgb = torch.from_numpy(rgb).to(cuda)
    feats = torch.empty((3, n) if planar else (n, 4), dtype=torch.float32, device=cuda)
    lum = torch.empty(n, dtype=torch.float32, device=cuda)
    color.pack_lab_beta(d_rgb, feats, lum, float(g["mu"]))
    f = feats.cpu().numpy()
    f = f if planar else f[:, :3].T
    np.testing.assert_allclose(lum.cpu().numpy(), g["luminance"], atol=1e-3)
    np.testing.assert_allclose(f[1:], g["features"][1:], atol=1e-3)
    assert np.array_equal(f[0], g["features"][0])
    if not planar:
        assert (feats[:, 3] == 0).all()


def test_rgb_to_ic(cuda):
    """Intensity / chroma planes on the GPU equal the reference's own FP32
    code bit for bit (golden fixture), and the restatement on a larger
    random image including black and white pixels."""
    import torch
    import make_golden
    from split_gb300 import color
    g = np.load(os.path.join(HERE, "golden", "ic_golden.npz"))
    rgb = make_golden.lab_beta_inputs()
    n = rgb.shape[0] * rgb.shape[1]
    ic = torch.empty((3, n), dtype=torch.float32, device=cuda)
    color.rgb_to_ic(torch.from_numpy(rgb).to(cuda), ic)
    assert np.array_equal(ic.cpu().numpy().view(np.uint32), g["ic"].view(np.uint32))
    rng = np.random.default_rng(77)
    big = rng.integers(0, 256, size=(1001, 777, 3), dtype=np.uint8)
    big[0, :5] = 0
    big[1, :5] = 255
    m = big.shape[0] * big.shape[1]
    ic2 = torch.empty((3, m), dtype=torch.float32, device=cuda)
    color.rgb_to_ic(torch.from_numpy(big).to(cuda), ic2)
    ref = oracle.rgb_to_ic_f32(big)
    assert np.array_equal(ic2.cpu().numpy().view(np.uint32), ref.view(np.uint32))


THR = np.load(os.path.join(HERE, "golden", "kmeans_threshold_golden.npz"))


@pytest.mark.parametrize("i", range(len(THR["thresholds"])))
def test_cluster_threshold_stops_where_the_reference_stops(cuda, inp, i):
    """cluster(..., 100, threshold) with the reference's shift rule
    (SPLIT_KMEANS_REFERENCE_SHIFT): the device's convergence test stops at
    the compiled reference's iteration, and the result equals the oracle's
    run of the same rule (FP32-exact assignments, FP64 updates)."""
    import torch
    from split_gb300 import kmeans
    pts, c0 = inp["km_points"], inp["km_c0"]
    thr = float(THR["thresholds"][i])
    cent = _t(c0, cuda)
    lab = torch.empty(pts.shape[1], dtype=torch.int32, device=cuda)
    its = torch.full((1,), -1, dtype=torch.int32, device=cuda)
    ws = kmeans.cluster(_t(pts, cuda), cent, lab, None, max_iter=100, threshold=thr,
                        layout=kmeans.PLANAR | kmeans.REFERENCE_SHIFT, width=512,
                        iterations_out=its)
    torch.cuda.synchronize()
    ws.check("kmeans")
    assert int(its.item()) == int(THR[f"iters_{i}"])
    olab, oc, oit, _ = oracle.kmeans_cluster_threshold(pts, c0, 100, thr)
    assert oit == int(its.item())
    gl = lab.cpu().numpy()
    assert (gl != olab).sum() <= 8            # near-ties after ulp-level centroid differences
    rel = np.abs(cent.cpu().numpy() - oc) / np.maximum(np.abs(oc), 1e-30)
    assert rel.max() <= 1e-4
    # the same rule written by the reference itself: within its FP32 drift
    assert (gl != THR[f"labels_{i}"]).mean() <= 2e-3


def test_cluster_threshold_rule_limits(cuda, inp):
    """The reference's shift is defined for 3-D features and K >= 3 only."""
    import torch
    from split_gb300 import _native, kmeans
    pts = _t(inp["km_points"], cuda)
    lab = torch.empty(pts.shape[1], dtype=torch.int32, device=cuda)
    for k in (1, 2):
        cent = _t(inp["km_c0"][:, :k], cuda)
        with pytest.raises(_native.SplitError):
            kmeans.cluster(pts, cent, lab, None, max_iter=5, threshold=1e-3,
                           layout=kmeans.PLANAR | kmeans.REFERENCE_SHIFT, width=512)
    f5 = _t(np.concatenate([inp["km_points"], inp["km_points"][:2]]), cuda)
    with pytest.raises(_native.SplitError):
        kmeans.cluster(f5, _t(np.zeros((5, 8), np.float32), cuda), lab, None, max_iter=5,
                       threshold=1e-3, layout=kmeans.PLANAR | kmeans.REFERENCE_SHIFT, width=512)


def test_propagate_centroids(cuda):
    """propagate_centroids (propagation.cu:9-24) on the reference's final
    labels and centroids: bit-exact against the oracle's gather and against
    the SHA-256 of the reference's own render."""
    import torch
    from split_gb300 import kmeans
    labels = THR["labels_0"].astype(np.int32)
    cent = THR["centroids_0"]
    out = torch.empty((3, labels.size), dtype=torch.float32, device=cuda)
    kmeans.propagate_centroids(_t(labels, cuda), _t(cent, cuda), out)
    got = out.cpu().numpy()
    assert np.array_equal(got, oracle.propagate_centroids(labels, cent))
    assert make_golden.sha(got) == str(THR["propagate_sha"])
    # labels outside [0, K) render as zeros
    bad = labels.copy()
    bad[::97] = -1
    bad[1::101] = cent.shape[1]
    kmeans.propagate_centroids(_t(bad, cuda), _t(cent, cuda), out)
    want = oracle.propagate_centroids(np.clip(bad, 0, cent.shape[1] - 1), cent)
    want[:, (bad < 0) | (bad >= cent.shape[1])] = 0.0
    assert np.array_equal(out.cpu().numpy(), want)


SMOOTH = np.load(os.path.join(HERE, "golden", "smooth_golden.npz"))


@pytest.mark.parametrize("i", range(len(SMOOTH["thresholds"])))
def test_merge_smooth_boundaries(cuda, i):
    """merge_smooth_boundaries on the device equals the compiled reference's
    output (built with the one-token reduction fix) bit for bit."""
    from split_gb300 import ccl
    rgb, lab, pts, s = make_golden.smooth_inputs()
    assert make_golden.sha(lab) == str(SMOOTH["labels_sha"])
    g = _t(lab, cuda)
    ws = ccl.merge_smooth_boundaries(_t(pts, cuda), s, g, None, float(SMOOTH["thresholds"][i]))
    ws.check("merge_smooth")
    assert np.array_equal(g.cpu().numpy(), SMOOTH[f"merged_{i}"])
