"""Self-consistency of the oracle restatement on small cases (CPU only):
labelling against a breadth-first search, erosion against a direct window
test, compression against numpy, merge invariants."""
from collections import deque

import numpy as np
import pytest

import oracle


def bfs_labels(lab, conn, conv):
    h, w = lab.shape
    out = np.full(lab.shape, -1, np.int64)
    nb = [(-1, 0), (1, 0), (0, -1), (0, 1)]
    if conn == 8:
        nb += [(-1, -1), (-1, 1), (1, -1), (1, 1)]
    for y in range(h):
        for x in range(w):
            if out[y, x] >= 0:
                continue
            comp = [(y, x)]
            q = deque(comp)
            out[y, x] = 0
            while q:
                cy, cx = q.popleft()
                for dy, dx in nb:
                    ny, nx = cy + dy, cx + dx
                    if 0 <= ny < h and 0 <= nx < w and out[ny, nx] < 0 and lab[ny, nx] == lab[y, x]:
                        out[ny, nx] = 0
                        comp.append((ny, nx))
                        q.append((ny, nx))
            idx = [a * w + b for a, b in comp]
            v = min(idx) if conv == 0 else max(idx)
            for a, b in comp:
                out[a, b] = v
    return out


@pytest.mark.parametrize("shape", [(1, 1), (1, 9), (7, 1), (13, 17), (24, 31)])
@pytest.mark.parametrize("conn", [4, 8])
@pytest.mark.parametrize("conv", [0, 1])
def test_ccl_matches_bfs(shape, conn, conv):
    rng = np.random.default_rng(shape[0] * 100 + shape[1] + conn)
    lab = rng.integers(0, 3, size=shape).astype(np.int32)
    assert np.array_equal(oracle.ccl(lab, conn, conv), bfs_labels(lab, conn, conv))


@pytest.mark.parametrize("r", [1, 2, 3])
def test_erode_window(r):
    rng = np.random.default_rng(r)
    lab = rng.integers(0, 2, size=(12, 15)).repeat(2, 0).repeat(2, 1).astype(np.int32)
    h, w = lab.shape
    want = np.full_like(lab, -1)
    for y in range(r, h - r):
        for x in range(r, w - r):
            win = lab[y - r:y + r + 1, x - r:x + r + 1]
            if (win == lab[y, x]).all():
                want[y, x] = lab[y, x]
    assert np.array_equal(oracle.erode(lab, r), want)


def test_compress_matches_numpy():
    rng = np.random.default_rng(3)
    lab = rng.integers(-1, 400, size=5000).astype(np.int32)
    out, n = oracle.compress_labels(lab)
    u, inv = np.unique(lab, return_inverse=True)
    assert n == len(u) and np.array_equal(out, inv)


@pytest.mark.parametrize("policy", [0, 1])
def test_merge_invariants(policy):
    rng = np.random.default_rng(policy + 5)
    lab = rng.integers(0, 3, size=(20, 25)).repeat(3, 0).repeat(3, 1).astype(np.int32)
    seg = oracle.ccl(lab, 8, 0)
    chroma = rng.random((2, seg.size), dtype=np.float32)
    P = 20
    out = oracle.merge_small(seg, P, policy, chroma)
    ids, sizes = np.unique(seg, return_counts=True)
    big = set(ids[sizes >= P])
    # large segments keep their pixels and id; every output id is an input id
    for s in big:
        assert (out[seg == s] == s).all()
    assert set(np.unique(out)) <= set(ids)
    # a segment moves as a whole
    for s in ids:
        assert len(np.unique(out[seg == s])) == 1


def test_merge_sorted_labels_quirk():
    # already non-decreasing labels: the reference rule applies no merge
    lab = np.repeat(np.arange(6, dtype=np.int32), 10).reshape(6, 10)
    lab = np.ascontiguousarray(lab)
    seg = oracle.compress_labels(oracle.ccl(lab, 4, 0))[0].reshape(lab.shape)
    assert np.array_equal(oracle.merge_small(seg, 100, 1, np.ones((2, seg.size), np.float32)), seg)
    assert not np.array_equal(oracle.merge_small(seg, 100, 0), seg)


def test_merge_smooth_rules():
    """Two halves with a long, smooth boundary merge into the larger id; a
    sharp boundary or a boundary of at most 15 edges keeps them apart."""
    h, w = 20, 16
    lab = np.zeros((h, w), np.int32)
    lab[:, w // 2:] = w // 2                   # ids: the first pixel of each half
    pts = np.zeros((3, h * w), np.float32)
    pts[0] = 0.5
    pts[0, lab.ravel() == w // 2] = 0.5005     # smooth: difference 5e-4
    pts[1] = 1.0
    out = oracle.merge_smooth(lab, pts, 0.01)
    assert (out == w // 2).all()
    sharp = pts.copy()
    sharp[0, lab.ravel() == w // 2] = 0.9      # difference 0.4 >= 0.01 * max
    assert np.array_equal(oracle.merge_smooth(lab, sharp, 0.01), lab)
    short = lab[:2].copy()                     # 2 rows: 4 edges each way, <= 15
    assert np.array_equal(oracle.merge_smooth(short, pts[:, : 2 * w], 0.01), short)
