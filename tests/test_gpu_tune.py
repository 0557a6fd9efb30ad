"""Tuned launch choices on the GPU: 16- to 128-row k-means units keep the parity
bar, an image keeps bit-identical results alone and in a batch whatever the
table says for other sizes, the allocation-free entry point follows the
table, and the autotuner produces and caches a valid table."""
import numpy as np
import pytest

import oracle
from split_gb300 import synth, tune

pytestmark = pytest.mark.gpu


@pytest.fixture
def table():
    saved = tune.current()
    yield tune
    tune.apply(saved)


def _t(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


@pytest.mark.parametrize("rows,layout", [(128, 0), (128, 1), (128, 2), (32, 1), (16, 0), (16, 2)])
def test_kmeans_lockstep_unit_heights(cuda, table, rows, layout):
    import torch
    from split_gb300 import kmeans
    table.apply([tune.Entry(tune.INT64_MAX, rows, 2)])
    w, h, k = 300, 333, 12
    rgb = synth.voronoi_rgb8(21, w, h, 40, sigma=4.0)
    feats = synth.features(rgb, 5)
    c = synth.pick_centroids(21, rgb, k, 5)
    if layout == 0:
        pts = _t(feats, cuda)
    elif layout == 1:
        f4 = np.zeros((w * h, 4), np.float32)
        f4[:, :3] = feats[:3].T
        pts = _t(f4, cuda)
    else:
        pts = _t(rgb.reshape(-1, 3), cuda)
    cent = _t(c, cuda)
    labels = torch.empty(w * h, dtype=torch.int32, device=cuda)
    ws = None
    for it in range(5):
        ws = kmeans.cluster(pts, cent, labels, ws, max_iter=1, threshold=-1.0, layout=layout,
                            dim=5, width=w)
        gl, gc = labels.cpu().numpy(), cent.cpu().numpy()
        assert np.array_equal(gl, oracle.kmeans_assign_f32(feats, c)), f"iteration {it}"
        ref, _ = oracle.kmeans_update_f64(gl, feats, c)
        rel = np.abs(gc - ref) / np.maximum(np.abs(ref), 1e-30)
        assert rel.max() <= 1e-5, f"iteration {it}: {rel.max():.3g}"
        c = gc
    ws.check("kmeans")


def test_batch_equals_single_under_mixed_table(cuda, table):
    """The four images take 16-, 32-, 64- and 128-row units, and the blocks
    per SM differ by class: every image still matches its own single-image
    pipeline bit for bit."""
    import torch
    from split_gb300 import batch, pipeline
    table.apply([tune.Entry(50_000, 16, 1), tune.Entry(100_000, 32, 2),
                 tune.Entry(500_000, 64, 0), tune.Entry(tune.INT64_MAX, 128, 0)])
    shapes = [(333, 201, 8, 5), (640, 480, 16, 6), (97, 311, 32, 4), (1024, 700, 16, 7)]
    params = pipeline.Params(merge_P=64)
    imgs, cents = [], []
    for i, (w, h, k, _) in enumerate(shapes):
        rgb = synth.voronoi_rgb8(500 + i, w, h, max(4, w * h // 4000), npalette=8,
                                 illum_gradient=True, sigma=4.0)
        imgs.append(rgb)
        cents.append(synth.pick_centroids(500 + i, rgb, k, params.dim))
    b = batch.Batch(shapes, params, cuda)
    b.load(imgs, cents)
    b.run()
    torch.cuda.synchronize()
    b.ws.check("batch")
    for i, (w, h, k, iters) in enumerate(shapes):
        p = pipeline.Params(**{**params.__dict__, "nclusters": k, "kmeans_iters": iters})
        pipe = pipeline.Pipeline(w, h, p, cuda)
        pipe.run(_t(imgs[i], cuda), _t(cents[i], cuda))
        torch.cuda.synchronize()
        assert np.array_equal(b.centroids_of(i).cpu().numpy(), pipe.centroids.cpu().numpy())
        assert np.array_equal(b.segment_labels_of(i).cpu().numpy(),
                              pipe.segment_labels.cpu().numpy())


def test_noalloc_follows_table(cuda, table):
    import torch
    from test_zz_no_alloc import _noalloc_run, _workspace_run
    from split_gb300 import _native
    table.apply([tune.Entry(tune.INT64_MAX, 128, 1)])
    w, h, k = 640, 360, 16
    rgb = synth.voronoi_rgb8(31, w, h, 48, sigma=3.0)
    pts = _t(rgb.reshape(-1, 3), cuda)
    c0 = _t(synth.pick_centroids(31, rgb, k, 5), cuda)
    a = _workspace_run(torch, pts, _native.LAYOUT_RGB8, 5, w * h, w, c0, (w * h,), 8)
    for _ in range(2):
        b = _noalloc_run(torch, pts, _native.LAYOUT_RGB8, 5, w * h, w, c0, (w * h,), 8)
        assert torch.equal(a[0], b[0]) and torch.equal(a[1], b[1])


def test_autotune_small_classes(cuda, table, tmp_path, monkeypatch):
    monkeypatch.setenv("SPLIT_GB300_TUNE_DIR", str(tmp_path))
    entries, detail = tune.autotune(cuda, sizes=((256, 256), (640, 480)), reps=2)
    assert [e.max_pixels for e in entries] == tune.class_bounds(((256, 256), (640, 480)))
    for e in entries:
        assert e.kmeans_unit_rows in tune.UNIT_ROWS
        assert e.kmeans_blocks_per_sm in tune.BLOCKS_PER_SM
    assert tune.current() == entries
    assert set(detail) == {"256x256", "640x480"}
    tune.apply([])
    assert tune.ensure(cuda) == entries and tune.current() == entries
