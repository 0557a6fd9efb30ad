"""Generate tests/golden/reference_golden.npz from the reference's own code.

Runs nitronoid/split's segmentation entry points, compiled for the CPU by
oracle/refbuild.py (needs the reference sources), on seeded synthetic inputs
and stores their outputs.  Inputs are not stored: they are regenerated from
the seeds by split_gb300.synth, and a SHA-256 of each generated input is kept
so a generator change is caught.

    python tests/golden/make_golden.py            # reference_golden.npz
    python tests/golden/make_golden.py lab_beta   # lab_beta_golden.npz
    python tests/golden/make_golden.py ic         # ic_golden.npz
    python tests/golden/make_golden.py threshold  # kmeans_threshold_golden.npz
    python tests/golden/make_golden.py smooth     # smooth_golden.npz
    python tests/golden/make_golden.py adjacency  # adjacency_golden.npz

Known limit of the CPU build: CCCL 3.0.1's host sort orders negative int keys
after non-negative ones, so compress_labels is only recorded on non-negative
labels (the reference's GPU build sorts with CUB and is not affected); the
same holds for segment_adjacency.  The CPU build's segment_adjacency_edges
runs Thrust's in-place remove_if, which races with more than one OpenMP
thread: the adjacency fixtures are made with one thread.
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

OUT = os.path.join(HERE, "reference_golden.npz")
OUT_LAB = os.path.join(HERE, "lab_beta_golden.npz")
OUT_IC = os.path.join(HERE, "ic_golden.npz")
OUT_THR = os.path.join(HERE, "kmeans_threshold_golden.npz")
OUT_SMOOTH = os.path.join(HERE, "smooth_golden.npz")
OUT_ADJ = os.path.join(HERE, "adjacency_golden.npz")
SMOOTH_THRESHOLDS = (0.01, 0.03, 0.1)
THRESHOLDS = (1e-3, 1e-2, 0.0145)


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def inputs():
    """Seeded inputs shared by make_golden and the tests (same recipe)."""
    from split_gb300 import synth
    d = {}
    # k-means case: the 512 x 512 Voronoi + noise recipe, 32 cells, sigma 4
    rgb = synth.voronoi_rgb8(0x51, 512, 512, 32, sigma=4.0)
    d["km_rgb"] = rgb
    d["km_points"] = synth.features(rgb, 3)
    d["km_c0"] = synth.pick_centroids(0x51, rgb, 8, 3)
    # labelling: a maze image and a blocky random label image
    d["maze"] = synth.maze_labels(0x52, 256, 192)
    rng = np.random.default_rng(0x53)
    blk = rng.integers(0, 4, size=(50, 70)).repeat(4, 0).repeat(4, 1)
    blk[rng.random(blk.shape) < 0.04] = 9
    d["blocks"] = blk.astype(np.int32)
    # chroma for the merge: multiples of 1/256, so float sums are exact
    d["chroma"] = (rng.integers(0, 256, size=(2, blk.size)) / 256.0).astype(np.float32)
    # heights for the normals
    d["heights"] = rng.random((48, 64), dtype=np.float32)
    return d


def lab_beta_inputs():
    """RGB8 image for the sample's Lab + beta features: Voronoi cells with
    noise, plus dark, mid and bright grey patches (achromatic pixels, so that
    beta takes -mu, 0 and +mu)."""
    from split_gb300 import synth
    rgb = synth.voronoi_rgb8(0x54, 128, 96, 24, sigma=2.0).copy()
    rng = np.random.default_rng(0x55)
    for (y0, x0, v) in ((8, 8, 18), (40, 60, 128), (60, 10, 250), (70, 90, 235)):
        patch = v + rng.integers(-2, 3, size=(16, 24, 1))
        rgb[y0:y0 + 16, x0:x0 + 24] = np.clip(patch, 0, 255).astype(np.uint8)
    return rgb


def main_lab_beta():
    from oracle import ref
    from split_gb300 import synth
    rgb = lab_beta_inputs()
    feats, lum = ref.lab_beta(synth.features(rgb, 3), 1e5)
    np.savez_compressed(OUT_LAB, rgb_sha=sha(rgb), features=feats, luminance=lum, mu=1e5)
    print(f"wrote {OUT_LAB}")


def main_ic():
    """Intensity / chroma planes of the Lab + beta input image, from the
    compiled reference (ref_rgb_to_ic)."""
    from oracle import ref
    from split_gb300 import synth
    rgb = lab_beta_inputs()
    ic = ref.rgb_to_ic(synth.features(rgb, 3))
    np.savez_compressed(OUT_IC, rgb_sha=sha(rgb), ic=ic)
    print(f"wrote {OUT_IC}")


def smooth_inputs():
    """Segments and features for the smooth-boundary merge: a Voronoi image
    with gentle noise; segments are the 8-connected components of its colours
    quantised to 3 bits per channel, compressed to [0, S); features are the
    colours scaled to [0, 100].  Returns (rgb, labels (H, W), points (3, N),
    S)."""
    import oracle
    from split_gb300 import synth
    rgb = synth.voronoi_rgb8(0x56, 160, 120, 40, sigma=2.0)
    q = (rgb // 32).astype(np.int32)
    cls = q[..., 0] * 64 + q[..., 1] * 8 + q[..., 2]
    seg = oracle.ccl(cls, 8, 0)
    lab, s = oracle.compress_labels(seg)
    pts = synth.features(rgb, 3) * np.float32(100.0)
    return rgb, lab.reshape(seg.shape), np.ascontiguousarray(pts, np.float32), s


def main_smooth():
    """merge_smooth_boundaries of the reference (merge_smooth_boundaries.cu:
    134-243, built with the one-token reduction fix recorded in
    oracle/refbuild.py) at a few thresholds."""
    from oracle import ref
    rgb, lab, pts, s = smooth_inputs()
    g = {"rgb_sha": np.array(sha(rgb)), "labels_sha": np.array(sha(lab)),
         "nsegments": np.array(s), "thresholds": np.array(SMOOTH_THRESHOLDS)}
    for i, t in enumerate(SMOOTH_THRESHOLDS):
        g[f"merged_{i}"] = ref.merge_smooth_boundaries(pts, lab, s, t)
    np.savez_compressed(OUT_SMOOTH, **g)
    print(f"wrote {OUT_SMOOTH} ({os.path.getsize(OUT_SMOOTH) / 1024:.0f} KiB)")


def adjacency_inputs():
    """Label images for segment adjacency: the smooth-merge segments (160 x
    120, compressed), seeded random labels in [0, 10) (37 x 53, most pixels
    on a boundary), a single row and a single column, and one value only."""
    _, seg, _, _ = smooth_inputs()
    rng = np.random.default_rng(0xAD)
    return {"segments": seg.astype(np.int32),
            "random": rng.integers(0, 10, size=(37, 53)).astype(np.int32),
            "row": rng.integers(0, 3, size=(1, 41)).astype(np.int32),
            "column": rng.integers(0, 3, size=(29, 1)).astype(np.int32),
            "flat": np.full((9, 14), 7, np.int32)}


def main_adjacency():
    """segment_adjacency_edges and segment_adjacency of the reference
    (segment_adjacency.cu:170-289) on adjacency_inputs()."""
    os.environ["OMP_NUM_THREADS"] = "1"
    from oracle import ref
    g = {}
    for name, lab in adjacency_inputs().items():
        g[f"sha_{name}"] = np.array(sha(lab))
        src, tgt = ref.segment_adjacency_edges(lab)
        keys, adj = ref.segment_adjacency(lab)
        g[f"{name}_src"], g[f"{name}_tgt"] = src, tgt
        g[f"{name}_keys"], g[f"{name}_adj"] = keys, adj
    np.savez_compressed(OUT_ADJ, **g)
    print(f"wrote {OUT_ADJ} ({os.path.getsize(OUT_ADJ) / 1024:.0f} KiB)")


def main_threshold():
    """cluster(points, c0, 100, threshold) on the 512 x 512 k-means input, for
    a few thresholds: the reference's iteration count (cluster.cu:71), the
    shifts it printed, its labels and centroids; and the SHA-256 of its
    propagate_centroids render of the final labels (propagation.cu:9-24)."""
    from oracle import ref
    d = inputs()
    g = {"sha_km_rgb": np.array(sha(d["km_rgb"])), "thresholds": np.array(THRESHOLDS)}
    for i, thr in enumerate(THRESHOLDS):
        lab, c, iters, shifts = ref.kmeans_cluster_threshold(d["km_points"], d["km_c0"], 100, thr)
        g[f"iters_{i}"] = np.array(iters)
        g[f"shifts_{i}"] = np.array(shifts, np.float64)
        g[f"labels_{i}"] = lab.astype(np.uint8)
        g[f"centroids_{i}"] = c
        if i == 0:
            out = ref.propagate_centroids(lab, c)
            g["propagate_sha"] = np.array(sha(out))
    np.savez_compressed(OUT_THR, **g)
    print(f"wrote {OUT_THR} ({os.path.getsize(OUT_THR) / 1024:.0f} KiB)")


def main():
    from oracle import ref
    d = inputs()
    g = {}
    for k in ("km_rgb", "maze", "blocks", "chroma", "heights"):
        g["sha_" + k] = np.array(sha(d[k]))
    pts, c0 = d["km_points"], d["km_c0"]
    # one assignment step and one update step
    lab1 = ref.label_points(pts, c0)
    g["km_label_points"] = lab1.astype(np.uint8)
    g["km_calculate_centroids"] = ref.calculate_centroids(lab1, pts, c0.shape[1])
    # the full 10-iteration clustering (threshold < 0: exactly 10)
    lab10, c10 = ref.kmeans_cluster(pts, c0, 10)
    g["km_cluster10_labels"] = lab10.astype(np.uint8)
    g["km_cluster10_centroids"] = c10
    # connected components (4-connected, converged max-index labels)
    km_img = lab10.reshape(512, 512)
    g["ccl_km"] = ref.connected_components(km_img)
    g["ccl_maze"] = ref.connected_components(d["maze"])
    g["ccl_blocks"] = ref.connected_components(d["blocks"])
    # compression of the component labels (non-negative)
    comp, ncomp = ref.compress_labels(g["ccl_blocks"])
    g["compress_blocks"] = comp
    g["compress_blocks_count"] = np.array(ncomp)
    # merge of segments < 24 px, reference chroma rule, on compressed labels
    g["merge_blocks_P24"] = ref.merge_small_segments(d["chroma"], comp, 24)
    # erosion of the component labels, n = 1 and n = 2
    g["erode1_km"] = ref.erode(g["ccl_km"], 1)
    g["erode2_blocks"] = ref.erode(g["ccl_blocks"], 2)
    # Sobel normals of a height map, depth 1
    g["sobel_normals"] = ref.sobel_normals(d["heights"], 1.0)
    np.savez_compressed(OUT, **g)
    print(f"wrote {OUT} ({os.path.getsize(OUT) / 1024:.0f} KiB)")


if __name__ == "__main__" and sys.argv[1:] == ["lab_beta"]:
    main_lab_beta()
elif __name__ == "__main__" and sys.argv[1:] == ["ic"]:
    main_ic()
elif __name__ == "__main__" and sys.argv[1:] == ["threshold"]:
    main_threshold()
elif __name__ == "__main__" and sys.argv[1:] == ["smooth"]:
    main_smooth()
elif __name__ == "__main__" and sys.argv[1:] == ["adjacency"]:
    main_adjacency()
elif __name__ == "__main__":
    main()
