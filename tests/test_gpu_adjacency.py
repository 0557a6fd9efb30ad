"""segment_adjacency_edges / segment_adjacency on the GPU (C ABI through
split_gb300.ccl) against the reference's own outputs (golden fixtures made
by tests/golden/make_golden.py adjacency) and against the oracle at larger
sizes, with negative and extreme labels and with every pixel its own
segment.  Integer outputs: bit-exact."""
import os
import sys

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402

ADJ = np.load(os.path.join(HERE, "golden", "adjacency_golden.npz"))


def _run(cuda, lab):
    import torch
    from split_gb300 import ccl
    h, w = lab.shape
    d = torch.from_numpy(np.ascontiguousarray(lab, np.int32)).to(cuda)
    edges = torch.full((16 * h * w,), -7, dtype=torch.int32, device=cuda)
    m = ccl.segment_adjacency_edges(d, edges)
    keys = torch.full((8 * h * w,), -7, dtype=torch.int32, device=cuda)
    adj = torch.full((8 * h * w,), -7, dtype=torch.int32, device=cuda)
    k = ccl.segment_adjacency(d, keys, adj)
    e = edges.cpu().numpy()
    return e[:m], e[m:2 * m], keys[:k].cpu().numpy(), adj[:k].cpu().numpy(), e[2 * m:]


@pytest.mark.parametrize("name", ("segments", "random", "row", "column", "flat"))
def test_against_reference(cuda, name):
    lab = make_golden.adjacency_inputs()[name]
    src, tgt, keys, adj, rest = _run(cuda, lab)
    assert np.array_equal(src, ADJ[f"{name}_src"]) and np.array_equal(tgt, ADJ[f"{name}_tgt"])
    assert np.array_equal(keys, ADJ[f"{name}_keys"]) and np.array_equal(adj, ADJ[f"{name}_adj"])
    # nothing written past the 2 m edge words
    assert (rest == -7).all()


@pytest.mark.parametrize("shape,low,high,seed", [
    ((257, 311), -5, 5, 1),                 # negative labels: signed (key, value) order
    ((64, 4099), -2**31, 2**31 - 1, 2),     # extreme ints: every digit of the sort key varies
    ((1, 1), 0, 1, 3),
    ((3, 2), -1, 1, 4),
])
def test_against_oracle_random(cuda, shape, low, high, seed):
    rng = np.random.default_rng(seed)
    lab = rng.integers(low, high, size=shape, endpoint=True).astype(np.int32)
    src, tgt, keys, adj, _ = _run(cuda, lab)
    s2, t2 = oracle.segment_adjacency_edges(lab)
    k2, a2 = oracle.segment_adjacency(lab)
    assert np.array_equal(src, s2) and np.array_equal(tgt, t2)
    assert np.array_equal(keys, k2) and np.array_equal(adj, a2)


def test_every_pixel_its_own_segment(cuda):
    """The edge bound is reached (8 per interior pixel) and all pairs are
    distinct: the sort runs on its largest input for the size."""
    h, w = 300, 517
    lab = np.arange(h * w, dtype=np.int32).reshape(h, w)[::-1].copy()
    src, tgt, keys, adj, _ = _run(cuda, lab)
    s2, t2 = oracle.segment_adjacency_edges(lab)
    k2, a2 = oracle.segment_adjacency(lab)
    assert src.size == 8 * h * w - 6 * (h + w) + 4
    assert np.array_equal(src, s2) and np.array_equal(tgt, t2)
    assert np.array_equal(keys, k2) and np.array_equal(adj, a2)


def test_4k_segments(cuda):
    """The benchmarked frame's segment labels (after merge and erosion)."""
    import torch
    import bench
    from split_gb300 import pipeline
    w, h = bench.W4K, bench.H4K
    rgb, c0 = bench.make_image(w, h)
    pipe = pipeline.Pipeline(w, h, pipeline.Params(), cuda)
    pipe.run(torch.from_numpy(rgb).to(cuda), torch.from_numpy(c0).to(cuda))
    torch.cuda.synchronize()
    lab = pipe.segment_labels.cpu().numpy().reshape(h, w)
    src, tgt, keys, adj, _ = _run(cuda, lab)
    s2, t2 = oracle.segment_adjacency_edges(lab)
    k2, a2 = oracle.segment_adjacency(lab)
    assert np.array_equal(src, s2) and np.array_equal(tgt, t2)
    assert np.array_equal(keys, k2) and np.array_equal(adj, a2)
