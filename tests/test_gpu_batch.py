"""Batches: every image's results equal the single-image pipeline's, eagerly
and replayed from a captured CUDA graph; the merge, labelling and erosion
results also equal the oracle's."""
import numpy as np
import pytest

import oracle
from split_gb300 import synth

pytestmark = pytest.mark.gpu

SHAPES = [(128, 96, 4, 6), (333, 201, 8, 5), (256, 256, 16, 8), (97, 311, 32, 4),
          (640, 128, 8, 10), (64, 64, 4, 3), (1000, 37, 16, 6), (513, 257, 32, 7),
          (1, 700, 4, 2), (720, 1, 8, 3)]


def _images(shapes, dim):
    imgs, cents = [], []
    for i, (w, h, k, _) in enumerate(shapes):
        rgb = synth.voronoi_rgb8(100 + i, w, h, max(4, (w * h) // 4000), npalette=8,
                                 illum_gradient=True, sigma=4.0)
        imgs.append(rgb)
        cents.append(synth.pick_centroids(100 + i, rgb, k, dim))
    return imgs, cents


def _single(torch, rgb, c0, k, iters, params, dev):
    from split_gb300 import pipeline
    p = pipeline.Params(**{**params.__dict__, "nclusters": k, "kmeans_iters": iters})
    h, w = rgb.shape[:2]
    pipe = pipeline.Pipeline(w, h, p, dev)
    pipe.run(torch.from_numpy(rgb).to(dev), torch.from_numpy(c0).to(dev))
    torch.cuda.synchronize()
    pipe.ws.check("pipeline")
    return (pipe.cluster_labels.cpu().numpy(), pipe.centroids.cpu().numpy(),
            pipe.segment_labels.cpu().numpy(), pipe.normals.cpu().numpy())


@pytest.mark.parametrize("features", [1, 2])
def test_batch_equals_single_images(cuda, features):
    import torch
    from split_gb300 import batch, pipeline
    params = pipeline.Params(features=features, merge_P=64)
    imgs, cents = _images(SHAPES, params.dim)
    b = batch.Batch(SHAPES, params, cuda)
    b.load(imgs, cents)
    b.run()
    torch.cuda.synchronize()
    for i, (w, h, k, iters) in enumerate(SHAPES):
        cl, ce, sl, nr = _single(torch, imgs[i], cents[i], k, iters, params, cuda)
        assert np.array_equal(b.cluster_labels_of(i).cpu().numpy(), cl), f"image {i} labels"
        assert np.array_equal(b.centroids_of(i).cpu().numpy(), ce), f"image {i} centroids"
        assert np.array_equal(b.segment_labels_of(i).cpu().numpy(), sl), f"image {i} segments"
        assert np.array_equal(b.normals_of(i).cpu().numpy(), nr), f"image {i} normals"
        # integer stages against the oracle, given the device's cluster labels
        seg = oracle.ccl(cl.reshape(h, w), 8, 0)
        seg = oracle.merge_small(seg, 64, 0)
        assert np.array_equal(sl, oracle.erode(seg, 1)), f"image {i} oracle"


def test_batch_graph_replay(cuda):
    import torch
    from split_gb300 import batch, pipeline
    params = pipeline.Params(merge_P=64)
    imgs, cents = _images(SHAPES[:6], params.dim)
    b = batch.Batch(SHAPES[:6], params, cuda)
    b.load(imgs, cents)
    b.run()
    torch.cuda.synchronize()
    ref_seg = b.segment_labels.clone()
    ref_cen = b.centroids.clone()
    b.capture()
    for _ in range(3):
        b.load(imgs, cents)       # the run updates the centroids in place
        b.replay()
        torch.cuda.synchronize()
        assert torch.equal(b.segment_labels, ref_seg)
        assert torch.equal(b.centroids, ref_cen)


def test_arena_reuse_across_compositions(cuda):
    """Batches of different compositions bound in turn to one resident arena
    (the serving loop's pattern, growing it twice) give the same results as
    batches with their own fresh buffers."""
    import torch
    from split_gb300 import batch, pipeline
    params = pipeline.Params(merge_P=64)
    arena = batch.Arena(cuda)
    comps = [SHAPES[:3], SHAPES[3:8], SHAPES[1:2], SHAPES[5:10], SHAPES[:6]]
    for comp in comps:
        imgs, cents = _images(comp, params.dim)
        a = batch.Batch(comp, params, cuda, arena=arena)
        a.load(imgs, cents)
        a.run()
        f = batch.Batch(comp, params, cuda)
        f.load(imgs, cents)
        f.run()
        torch.cuda.synchronize()
        a.ws.check("arena batch")
        for i in range(len(comp)):
            assert torch.equal(a.segment_labels_of(i), f.segment_labels_of(i))
            assert torch.equal(a.centroids_of(i), f.centroids_of(i))
            assert torch.equal(a.normals_of(i), f.normals_of(i))


# K = 32 on the 97 x 311 image fragments it into ~8500 segments of ~3.5 px
# (more (segment, neighbour) pairs than the merge table holds; see below)
LAB_SHAPES = [s if s != (97, 311, 32, 4) else (97, 311, 8, 4) for s in SHAPES]


def _lab_inputs(torch, cuda, shapes, params, seed=300):
    from split_gb300 import color
    imgs = [synth.voronoi_rgb8(seed + i, w, h, max(4, (w * h) // 4000), npalette=8,
                               illum_gradient=True, sigma=4.0) for i, (w, h, _, _) in enumerate(shapes)]
    cents = []
    for (w, h, k, _), rgb in zip(shapes, imgs):
        # initial centroids: the Lab + beta features of k evenly spaced pixels
        n = w * h
        f4 = torch.empty((n, 4), dtype=torch.float32, device=cuda)
        color.pack_lab_beta(torch.from_numpy(rgb).to(cuda), f4, mu=params.beta_mu)
        idx = np.linspace(0, n - 1, k).astype(np.int64)
        c = f4[:, :3].cpu().numpy()[idx].T
        if params.dim == 5:
            xy = np.stack([idx % w, idx // w]).astype(np.float32) * np.float32(params.xy_scale)
            c = np.concatenate([c, xy])
        cents.append(np.ascontiguousarray(c, np.float32))
    return imgs, cents


@pytest.mark.parametrize("dim", [3, 5])
def test_batch_lab_beta_equals_single(cuda, dim):
    """The sample's Lab + beta features in a batch (per-image maxima over the
    tile grid): every image's cluster labels, centroids, segments and normals
    equal its single-image pipeline run bit for bit."""
    import torch
    from split_gb300 import _native, batch, pipeline
    params = pipeline.Params(features=_native.FEATURES_LAB_BETA, dim=dim, merge_P=64)
    imgs, cents = _lab_inputs(torch, cuda, LAB_SHAPES, params)
    b = batch.Batch(LAB_SHAPES, params, cuda)
    b.load(imgs, cents)
    b.run()
    torch.cuda.synchronize()
    b.ws.check("batch")
    for i, (w, h, k, iters) in enumerate(LAB_SHAPES):
        cl, ce, sl, nr = _single(torch, imgs[i], cents[i], k, iters, params, cuda)
        assert np.array_equal(b.cluster_labels_of(i).cpu().numpy(), cl), f"image {i} labels"
        assert np.array_equal(b.centroids_of(i).cpu().numpy(), ce), f"image {i} centroids"
        assert np.array_equal(b.segment_labels_of(i).cpu().numpy(), sl), f"image {i} segments"
        assert np.array_equal(b.normals_of(i).cpu().numpy(), nr), f"image {i} normals"


def test_merge_of_many_small_segments(cuda):
    """A 97 x 311 image cut into ~8500 segments of ~3.5 px has more (segment,
    neighbour) pairs than half the single-image merge table holds: the merge
    splits the small segments into classes and decides them round by round,
    and the pipeline's segments still equal the oracle's CCL -> merge ->
    erosion of its own k-means labels, bit for bit."""
    import torch
    from split_gb300 import _native, pipeline
    params = pipeline.Params(features=_native.FEATURES_LAB_BETA, dim=3, merge_P=64)
    shape = [(97, 311, 32, 4)]
    imgs, cents = _lab_inputs(torch, cuda, shape, params, seed=303)
    p = pipeline.Params(**{**params.__dict__, "nclusters": 32, "kmeans_iters": 4})
    pipe = pipeline.Pipeline(97, 311, p, cuda)
    pipe.run(torch.from_numpy(imgs[0]).to(cuda), torch.from_numpy(cents[0]).to(cuda))
    torch.cuda.synchronize()
    pipe.ws.check("pipeline")
    cl = pipe.cluster_labels.cpu().numpy().reshape(311, 97)
    seg = oracle.ccl(cl, 8, 0)
    assert len(np.unique(seg)) > 8000
    want = oracle.erode(oracle.merge_small(seg, 64, 0), 1)
    assert np.array_equal(pipe.segment_labels.cpu().numpy(), want)
