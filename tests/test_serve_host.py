"""Host logic of the continuous-batching server: admission order, the byte
budget, batch formation and the latency percentiles (no GPU)."""
import numpy as np
import pytest

from split_gb300.serve import Admission, Request, percentile, poisson_arrivals, BYTES_PER_PIXEL


def _req(rid, w, h, t=0.0):
    return Request(rid, np.zeros((h, w, 3), np.uint8), 8, 5, np.zeros((5, 8), np.float32), t)


def test_footprint_rounds_to_arena_granule():
    assert _req(0, 64, 1).footprint == 64 * BYTES_PER_PIXEL
    assert _req(0, 65, 1).footprint == 128 * BYTES_PER_PIXEL


def test_admission_is_fifo_under_budget():
    a = Admission(budget_bytes=_req(0, 64, 64).footprint * 2)
    reqs = [_req(i, 64, 64) for i in range(5)]
    for r in reqs:
        a.arrive(r)
    assert a.admit(1.0) == 2
    assert [r.rid for r in a.admitted] == [0, 1]
    assert a.admit(2.0) == 0
    batch = a.take()
    assert [r.rid for r in batch] == [0, 1] and a.admitted == []
    a.release(batch[:1])
    assert a.admit(3.0) == 1 and a.admitted[0].rid == 2 and a.admitted[0].admitted == 3.0
    a.release(batch[1:])
    a.release(a.take())
    assert a.in_use == 0
    # a large request at the head blocks the ones behind it (no overtaking)
    b = Admission(budget_bytes=_req(0, 64, 64).footprint * 2)
    b.arrive(_req(10, 64, 64))
    b.admit(0)
    b.arrive(_req(11, 64, 128))
    b.arrive(_req(12, 64, 32))
    assert b.admit(0) == 0


def test_oversized_request_rejected():
    a = Admission(budget_bytes=1000)
    with pytest.raises(ValueError):
        a.arrive(_req(0, 64, 64))


def test_take_respects_pixel_cap_but_always_progresses():
    a = Admission(budget_bytes=1 << 40)
    for i, (w, h) in enumerate([(100, 100), (100, 100), (300, 300), (10, 10)]):
        a.arrive(_req(i, w, h))
    a.admit(0)
    first = a.take(max_pixels=25000)
    assert [r.rid for r in first] == [0, 1, 3]
    second = a.take(max_pixels=25000)      # larger than the cap on its own
    assert [r.rid for r in second] == [2]


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
