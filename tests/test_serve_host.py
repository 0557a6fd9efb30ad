"""Host logic of the continuous-batching server (no GPU): the C++ server's
admission and batch-formation policy through split_server_admission_test
(arrival order, the byte budget, the pixel cap), the footprint query, and the
latency percentiles."""
import numpy as np
import pytest

from split_gb300 import pipeline
from split_gb300.serve import admission_plan, bytes_per_pixel, footprint, percentile, \
    poisson_arrivals


def test_footprint_rounds_to_arena_granule():
    assert footprint(64, 100) == 64 * 100
    assert footprint(65, 100) == 128 * 100
    bpp = bytes_per_pixel(pipeline.Params())
    # arenas (RGB8, two label planes, normals: 23 B) plus the workspace
    assert 23 + 16 < bpp < 512


def test_admission_is_fifo_under_budget():
    fp = [100] * 5
    batch, nb, peak = admission_plan(fp, [1] * 5, budget=200, max_batch_pixels=1 << 30, depth=2)
    # two fit at a time; each batch takes what was admitted, in order
    assert list(batch) == [0, 0, 1, 1, 2] and nb == 3 and peak <= 200
    # a large request at the head blocks the ones behind it (no overtaking):
    # 150 waits for the first batch to finish, and the small one behind it too
    batch, nb, _ = admission_plan([100, 150, 10], [1, 1, 1], budget=200,
                                  max_batch_pixels=1 << 30, depth=2)
    assert list(batch) == [0, 1, 1]


def test_in_flight_depth_bounds_batches():
    batch, nb, _ = admission_plan([1] * 6, [10] * 6, budget=1 << 40, max_batch_pixels=20,
                                  depth=1)
    assert list(batch) == [0, 0, 1, 1, 2, 2] and nb == 3


def test_oversized_request_rejected():
    from split_gb300 import _native
    with pytest.raises(_native.SplitError):
        admission_plan([1000], [1], budget=999, max_batch_pixels=1 << 30, depth=2)


def test_take_respects_pixel_cap_but_always_progresses():
    px = [10000, 10000, 90000, 100]
    batch, nb, _ = admission_plan([1] * 4, px, budget=1 << 40, max_batch_pixels=25000, depth=8)
    # the cap skips the large one and takes the small one behind it; the large
    # one then forms a batch alone
    assert list(batch) == [0, 0, 1, 0] and nb == 2


def test_percentile_matches_numpy_linear():
    rng = np.random.default_rng(3)
    v = rng.exponential(size=101).tolist()
    for q in (0, 50, 90, 99, 100):
        assert percentile(v, q) == pytest.approx(np.percentile(v, q))
    assert percentile([], 50) is None


def test_poisson_arrivals_rate():
    t = poisson_arrivals(1, 20000, 500.0)
    assert np.all(np.diff(t) > 0)
    assert t[-1] / len(t) == pytest.approx(1 / 500.0, rel=0.05)
