"""The oracle restatement pinned against the reference's own outputs
(tests/golden/reference_golden.npz, made by tests/golden/make_golden.py from
the reference compiled for the CPU).  CPU only."""
import os
import sys

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402

GOLDEN = np.load(os.path.join(HERE, "golden", "reference_golden.npz"))


@pytest.fixture(scope="module")
def inp():
    return make_golden.inputs()


def test_generated_inputs_unchanged(inp):
    for k in ("km_rgb", "maze", "blocks", "chroma", "heights"):
        assert make_golden.sha(inp[k]) == str(GOLDEN["sha_" + k]), k


def test_label_points(inp):
    # reference: float (x-c)^2 sums; oracle f32 fma chain.  Identical except
    # where the best-vs-second gap is below 1e-5 relative.
    lab, d1, d2 = oracle.kmeans_assign_f64(inp["km_points"], inp["km_c0"])
    ref = GOLDEN["km_label_points"].astype(np.int32)
    near = (d2 - d1) <= 1e-5 * d2
    assert ((lab != ref) & ~near).sum() == 0
    f32 = oracle.kmeans_assign_f32(inp["km_points"], inp["km_c0"])
    assert ((f32 != ref) & ~near).sum() == 0


def test_calculate_centroids(inp):
    ref_lab = GOLDEN["km_label_points"].astype(np.int32)
    c, cnt = oracle.kmeans_update_f64(ref_lab, inp["km_points"], inp["km_c0"])
    assert (cnt > 0).all()
    ref = GOLDEN["km_calculate_centroids"].astype(np.float64)
    # The reference sums up to 57k members per cluster sequentially in FP32
    # (reduce_by_key, centroids.cu:78-90): it sits up to a few 1e-4 from the
    # exact mean.  A sequential FP32 sum times the FP32 reciprocal count
    # (centroids.cu:60-63, :96-100) reproduces it to within 2 ulp.
    assert (np.abs(ref - c) / np.abs(c)).max() <= 1e-3
    pts = inp["km_points"]
    for k in range(ref.shape[1]):
        m = ref_lab == k
        for d in range(pts.shape[0]):
            s = np.cumsum(pts[d, m], dtype=np.float32)[-1]
            emu = np.float32(s * (np.float32(1) / np.float32(m.sum())))
            assert abs(np.float32(ref[d, k]) - emu) <= 2 * np.spacing(emu)


def test_cluster_10_iterations(inp):
    pts, c = inp["km_points"], inp["km_c0"].copy()
    for _ in range(10):
        lab = oracle.kmeans_assign_f32(pts, c)
        c64, _ = oracle.kmeans_update_f64(lab, pts, c)
        c = c64.astype(np.float32)
    ref_lab = GOLDEN["km_cluster10_labels"].astype(np.int32)
    # two trajectories (reference: FP32 sequential sums; oracle: FP64 means)
    # through 10 iterations: labels differ only where rounding moved a
    # near-tie pixel, centroids by the reference's accumulation error
    assert (lab != ref_lab).mean() <= 1e-3
    ref_c = GOLDEN["km_cluster10_centroids"]
    assert (np.abs(ref_c - c) / np.abs(c)).max() <= 1e-3


@pytest.mark.parametrize("name,key", [("ccl_maze", "maze"), ("ccl_blocks", "blocks")])
def test_connected_components(inp, name, key):
    assert np.array_equal(oracle.ccl(inp[key], 4, 1), GOLDEN[name])


def test_connected_components_on_kmeans_labels():
    km = GOLDEN["km_cluster10_labels"].astype(np.int32).reshape(512, 512)
    assert np.array_equal(oracle.ccl(km, 4, 1), GOLDEN["ccl_km"])


def test_compress_labels():
    comp, n = oracle.compress_labels(GOLDEN["ccl_blocks"])
    assert n == int(GOLDEN["compress_blocks_count"])
    assert np.array_equal(comp, GOLDEN["compress_blocks"])


def test_merge_reference_chroma(inp):
    out = oracle.merge_small(GOLDEN["compress_blocks"], 24, 1, inp["chroma"])
    assert np.array_equal(out, GOLDEN["merge_blocks_P24"])


def test_erode():
    assert np.array_equal(oracle.erode(GOLDEN["ccl_km"], 1), GOLDEN["erode1_km"])
    assert np.array_equal(oracle.erode(GOLDEN["ccl_blocks"], 2), GOLDEN["erode2_blocks"])


def test_sobel_normals(inp):
    o = oracle.sobel_normals_f64(inp["heights"], 1.0)
    r = GOLDEN["sobel_normals"].astype(np.float64)
    ang = np.arccos(np.clip((o * r).sum(0) / np.linalg.norm(r, axis=0), -1, 1))
    # the reference's FP32 prefix-scan formulation drifts from FP64
    assert ang.max() <= 1e-3


def test_lab_beta_restatement_against_reference():
    """The FP64 restatement of the sample's Lab + beta features against the
    reference's own FP32 code: L*, a*, b* within 2e-3, beta identical."""
    import make_golden
    g = np.load(os.path.join(HERE, "golden", "lab_beta_golden.npz"))
    rgb = make_golden.lab_beta_inputs()
    assert make_golden.sha(rgb) == str(g["rgb_sha"])
    feats, lum = oracle.lab_beta_f64(rgb, float(g["mu"]))
    np.testing.assert_allclose(lum, g["luminance"], atol=2e-3)
    np.testing.assert_allclose(feats[1:], g["features"][1:], atol=2e-3)
    assert np.array_equal(feats[0], g["features"][0])
    assert set(np.unique(feats[0])) == {-1e5, 0.0, 1e5}


def test_ic_restatement_against_reference():
    """The FP32 restatement of the sample's intensity / chroma planes equals
    the reference's own code (clamp, rgb_to_ic) bit for bit."""
    import make_golden
    g = np.load(os.path.join(HERE, "golden", "ic_golden.npz"))
    rgb = make_golden.lab_beta_inputs()
    assert make_golden.sha(rgb) == str(g["rgb_sha"])
    ic = oracle.rgb_to_ic_f32(rgb)
    assert ic.dtype == np.float32 and ic.shape == g["ic"].shape
    assert np.array_equal(ic.view(np.uint32), g["ic"].view(np.uint32))
    # black pixels take the clamp: intensity 1/255 and chroma 1, up to the
    # FP32 rounding of (3 / 255) * (1 / 3) and its reciprocal
    black = oracle.rgb_to_ic_f32(np.zeros((1, 3), np.uint8))
    np.testing.assert_allclose(black[:, 0], [1 / 255, 1.0, 1.0], rtol=1e-6)


THR = np.load(os.path.join(HERE, "golden", "kmeans_threshold_golden.npz"))


def test_threshold_golden_input_unchanged(inp):
    assert make_golden.sha(inp["km_rgb"]) == str(THR["sha_km_rgb"])


@pytest.mark.parametrize("i", range(len(THR["thresholds"])))
def test_kmeans_threshold_stops_where_the_reference_stops(inp, i):
    """cluster(points, c0, 100, threshold): the oracle's restatement of the
    reference's shift (which reads overwritten workspace words) stops at the
    reference's iteration; its shifts follow the printed ones within the FP32
    drift of the reference's centroid sums; the labels agree except on a few
    tenths of a percent of pixels while the clustering is still moving."""
    thr = float(THR["thresholds"][i])
    lab, c, iters, shifts = oracle.kmeans_cluster_threshold(inp["km_points"], inp["km_c0"], 100,
                                                            thr)
    assert iters == int(THR[f"iters_{i}"])
    ref_shifts = THR[f"shifts_{i}"]
    assert len(shifts) == len(ref_shifts)
    assert np.abs(np.array(shifts) - ref_shifts).max() <= 1e-3
    assert (lab != THR[f"labels_{i}"]).mean() <= 2e-3
    assert np.abs(c - THR[f"centroids_{i}"]).max() <= 5e-3


def test_kmeans_threshold_intended_rule_differs():
    """The L2 change of the centroid matrix stops elsewhere on this input:
    the reference's rule is what pins its iteration counts."""
    d = make_golden.inputs()
    counts = [oracle.kmeans_cluster_threshold(d["km_points"], d["km_c0"], 100, float(t),
                                              reference_shift_rule=False)[2]
              for t in THR["thresholds"]]
    assert counts != [int(THR[f"iters_{i}"]) for i in range(len(counts))]


def test_propagate_centroids():
    out = oracle.propagate_centroids(THR["labels_0"].astype(np.int32), THR["centroids_0"])
    assert make_golden.sha(out) == str(THR["propagate_sha"])


SMOOTH = np.load(os.path.join(HERE, "golden", "smooth_golden.npz"))


@pytest.mark.parametrize("i", range(len(SMOOTH["thresholds"])))
def test_merge_smooth_boundaries(i):
    """The smooth-boundary merge restatement equals the compiled reference
    (merge_smooth_boundaries.cu:134-243, built with thrust::minimum as the
    reduction its comment describes) bit for bit."""
    rgb, lab, pts, s = make_golden.smooth_inputs()
    assert make_golden.sha(rgb) == str(SMOOTH["rgb_sha"])
    assert make_golden.sha(lab) == str(SMOOTH["labels_sha"]) and s == int(SMOOTH["nsegments"])
    got = oracle.merge_smooth(lab, pts, float(SMOOTH["thresholds"][i]))
    assert np.array_equal(got, SMOOTH[f"merged_{i}"])


ADJ = np.load(os.path.join(HERE, "golden", "adjacency_golden.npz"))
ADJ_CASES = ("segments", "random", "row", "column", "flat")


@pytest.fixture(scope="module")
def adj_inputs():
    return make_golden.adjacency_inputs()


@pytest.mark.parametrize("name", ADJ_CASES)
def test_segment_adjacency_restatement(adj_inputs, name):
    """The oracle's edge list and sorted distinct pairs equal the reference's
    (segment_adjacency.cu:170-289), element by element."""
    lab = adj_inputs[name]
    assert make_golden.sha(lab) == str(ADJ[f"sha_{name}"])
    src, tgt = oracle.segment_adjacency_edges(lab)
    assert np.array_equal(src, ADJ[f"{name}_src"]) and np.array_equal(tgt, ADJ[f"{name}_tgt"])
    keys, adj = oracle.segment_adjacency(lab)
    assert np.array_equal(keys, ADJ[f"{name}_keys"]) and np.array_equal(adj, ADJ[f"{name}_adj"])
