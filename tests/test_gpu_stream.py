"""Streaming frames from host memory (pipeline.HostPipeline): with several
frames of different content in flight and the slots reused, every frame's
host results equal a plain Pipeline.run of that frame, bit for bit."""
import pytest

from split_gb300 import synth

pytestmark = pytest.mark.gpu


def test_host_pipeline_matches_plain(cuda):
    import torch
    from split_gb300 import pipeline
    w, h = 640, 360
    params = pipeline.Params(merge_P=64)
    frames, outs = [], []
    for i in range(5):
        rgb = synth.voronoi_rgb8(700 + i, w, h, 40, sigma=3.0)
        c0 = synth.pick_centroids(700 + i, rgb, params.nclusters, params.dim)
        frames.append((torch.from_numpy(rgb).pin_memory(), torch.from_numpy(c0).pin_memory()))
    hp = pipeline.HostPipeline(w, h, params, cuda, depth=2)
    for rgb, c0 in frames:
        o = (torch.empty((h, w), dtype=torch.int32).pin_memory(),
             torch.empty((3, w * h), dtype=torch.float32).pin_memory(),
             torch.empty((params.dim, params.nclusters), dtype=torch.float32).pin_memory(),
             torch.empty(w * h, dtype=torch.int32).pin_memory())
        hp.submit(rgb, c0, *o)
        outs.append(o)
    for t in range(len(frames)):
        hp.wait(t)
    hp.check()
    ref = pipeline.Pipeline(w, h, params, cuda)
    for (rgb, c0), (seg, nrm, cen, lab) in zip(frames, outs):
        ref.run(rgb.to(cuda), c0.to(cuda))
        torch.cuda.synchronize()
        assert torch.equal(seg, ref.segment_labels.cpu())
        assert torch.equal(nrm, ref.normals.cpu())
        assert torch.equal(cen, ref.centroids.cpu())
        assert torch.equal(lab, ref.cluster_labels.cpu())


def test_host_pipeline_rejects_device_buffers(cuda):
    import torch
    from split_gb300 import pipeline
    hp = pipeline.HostPipeline(64, 64, pipeline.Params(), cuda, depth=1)
    rgb = torch.zeros(64 * 64 * 3, dtype=torch.uint8, device=cuda)
    c0 = torch.zeros((5, 16), dtype=torch.float32).pin_memory()
    seg = torch.empty((64, 64), dtype=torch.int32).pin_memory()
    with pytest.raises(ValueError):
        hp.submit(rgb, c0, seg)
