"""Serving through the C++ server (split_server_*): a request's results are
identical whether it is served alone or batched with others, and equal the
single-image pipeline's; the HBM budget bounds what is admitted."""
import numpy as np
import pytest

import split_synth as synth

pytestmark = pytest.mark.gpu

SHAPES = [(640, 480, 16, 8), (333, 201, 8, 6), (1024, 768, 16, 10), (97, 311, 32, 4),
          (1280, 720, 16, 7), (64, 64, 4, 3), (513, 257, 32, 9), (1920, 1080, 16, 12)]


def _requests(dim, arrivals=None):
    from split_gb300.serve import Request
    out = []
    for i, (w, h, k, iters) in enumerate(SHAPES):
        rgb = synth.voronoi_rgb8(300 + i, w, h, max(4, w * h // 5000), npalette=12,
                                 illum_gradient=True, sigma=3.0)
        c0 = synth.pick_centroids(300 + i, rgb, k, dim)
        t = 0.0 if arrivals is None else float(arrivals[i])
        out.append(Request(i, rgb, k, iters, c0, t))
    return out


def test_alone_equals_mix(cuda):
    import torch
    from split_gb300 import pipeline
    from split_gb300.serve import Server, poisson_arrivals
    params = pipeline.Params(merge_P=64)
    # mixed: everything visible at once, so several requests share each batch
    mix = Server(params, device=cuda, depth=2)
    done = mix.serve(_requests(params.dim), realtime=False)
    assert len(done) == len(SHAPES)
    assert max(mix.batch_sizes) > 1
    # open-loop arrivals: batches form from whatever has arrived
    arr = poisson_arrivals(7, len(SHAPES), 400.0)
    live = Server(params, device=cuda, depth=2).serve(_requests(params.dim, arr))
    by_id = {r.rid: r for r in done}
    live_by_id = {r.rid: r for r in live}
    for i, (w, h, k, iters) in enumerate(SHAPES):
        alone = Server(params, device=cuda).serve(_requests(params.dim)[i:i + 1],
                                                  realtime=False)[0]
        for other in (by_id[i], live_by_id[i]):
            assert np.array_equal(other.segment_labels, alone.segment_labels), f"request {i}"
            assert np.array_equal(other.centroids_out, alone.centroids_out), f"request {i}"
        # and the single-image pipeline agrees
        p = pipeline.Params(**{**params.__dict__, "nclusters": k, "kmeans_iters": iters})
        pipe = pipeline.Pipeline(w, h, p, cuda)
        r = _requests(params.dim)[i]
        pipe.run(torch.from_numpy(r.rgb).to(cuda), torch.from_numpy(r.centroids).to(cuda))
        torch.cuda.synchronize()
        assert np.array_equal(pipe.segment_labels.cpu().numpy(), alone.segment_labels)
        assert np.array_equal(pipe.centroids.cpu().numpy(), alone.centroids_out)


def test_budget_bounds_batches(cuda):
    from split_gb300 import pipeline
    from split_gb300.serve import Server, bytes_per_pixel, footprint
    params = pipeline.Params(merge_P=64)
    reqs = _requests(params.dim)
    bpp = bytes_per_pixel(params)
    budget = max(footprint(r.pixels, bpp) for r in reqs) * 2
    s = Server(params, budget_bytes=budget, device=cuda, depth=2)
    done = s.serve(reqs, realtime=False)
    assert sorted(r.rid for r in done) == list(range(len(SHAPES)))
    c = s.counters()
    assert c.in_use_bytes == 0 and 0 < c.peak_in_use_bytes <= budget
    assert c.bytes_per_pixel == bpp and c.completed == c.submitted == len(SHAPES)
    # the budget holds all but the largest request at once: it waits for a
    # later batch
    assert c.batches >= 2
    for r in done:
        assert r.done >= r.admitted >= r.arrival
