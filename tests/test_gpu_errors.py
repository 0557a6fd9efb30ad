"""Device-side error paths that are safe to provoke: a bounded wait that runs
out.  A cooperative k-means launch in which one block leaves at its first
grid barrier without arriving (a host-set launch parameter, so the barrier's
count never completes) and a short poll limit: the other blocks give up after
the limit, every block returns, the call reports SPLIT_ERR_TIMEOUT through
the workspace's status word, and the GPU stays usable (the next call on the
same workspace gives the normal result).  Nothing here waits without a
limit."""
import numpy as np
import pytest

import split_synth as synth

pytestmark = pytest.mark.gpu


def _inputs(cuda):
    import torch
    from split_gb300 import color
    w, h = 256, 256
    rgb = synth.voronoi_rgb8(404, w, h, 24, sigma=3.0)
    f4 = torch.empty((w * h, 4), dtype=torch.float32, device=cuda)
    color.pack_rgb8(torch.from_numpy(rgb).to(cuda), f4)
    c0 = torch.from_numpy(synth.pick_centroids(404, rgb, 8, 5)).to(cuda)
    return w, h, f4, c0


@pytest.mark.parametrize("skip_block", [0, 5])
def test_grid_barrier_wait_runs_out(cuda, skip_block):
    import torch
    from split_gb300 import _native, kmeans
    from split_gb300._util import Workspace
    lib = _native.load()
    w, h, f4, c0 = _inputs(cuda)
    layout = kmeans.FLOAT4 | kmeans.UNIT_RANGE
    ws = Workspace(kmeans.cluster_workspace_2d(w * h, w, 8, 5), cuda)
    # reference result on a clean workspace
    ref_c = c0.clone()
    ref_l = torch.empty(w * h, dtype=torch.int32, device=cuda)
    kmeans.cluster(f4, ref_c, ref_l, ws, max_iter=6, threshold=-1.0, layout=layout, dim=5,
                   width=w)
    ws.check("clean run")
    # 16 units of 64 x 64: a grid of 16 blocks, so block 5 exists
    lib.split_kmeans_set_wait_test(4096, skip_block)
    try:
        c = c0.clone()
        lab = torch.empty_like(ref_l)
        kmeans.cluster(f4, c, lab, ws, max_iter=6, threshold=-1.0, layout=layout, dim=5,
                       width=w)
        torch.cuda.synchronize()
    finally:
        lib.split_kmeans_set_wait_test(0, -1)
    assert ws.status() == _native.ERR_TIMEOUT
    # the limit back to its default and no block skipping: the same call
    # completes normally, with the clean run's results
    c = c0.clone()
    kmeans.cluster(f4, c, lab, ws, max_iter=6, threshold=-1.0, layout=layout, dim=5, width=w)
    ws.check("after the timeout")
    assert torch.equal(lab, ref_l) and torch.equal(c, ref_c)
