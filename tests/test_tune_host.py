"""Tuning table through the C ABI (validation, round trip) and the
autotuner's host logic (class bounds, choice, cache) without a GPU."""
import pytest

from split_gb300 import _native, tune


@pytest.fixture
def restore_table():
    saved = tune.current()
    yield
    tune.apply(saved)


def test_table_round_trip(restore_table):
    es = [tune.Entry(1000, 16, 2), tune.Entry(5000, 32, 1), tune.Entry(10**9, 128, 0),
          tune.Entry(tune.INT64_MAX, 64, 1)]
    tune.apply(es)
    assert tune.current() == es
    tune.apply([])
    assert tune.current() == []


@pytest.mark.parametrize("bad", [
    [tune.Entry(100, 96, 0)],                              # unit rows not 16/32/64/128
    [tune.Entry(100, 8, 0)],
    [tune.Entry(100, 64, 9)],                              # blocks per SM out of range
    [tune.Entry(100, 64, -1)],
    [tune.Entry(0, 64, 0)],                                # empty class
    [tune.Entry(100, 64, 0), tune.Entry(100, 128, 0)],     # not ascending
])
def test_table_rejects_invalid(restore_table, bad):
    before = tune.current()
    with pytest.raises(_native.SplitError):
        tune.apply(bad)
    assert tune.current() == before


def test_table_too_long(restore_table):
    with pytest.raises(_native.SplitError):
        tune.apply([tune.Entry(i + 1, 64, 0) for i in range(_native.TUNE_MAX_ENTRIES + 1)])


def test_class_bounds_are_geometric_midpoints():
    b = tune.class_bounds(((100, 100), (400, 400), (1600, 1600)))
    assert b == [40000, 640000, tune.INT64_MAX]
    assert b == sorted(b)


def test_pick_fastest_with_stable_ties():
    t = {(64, 0): 2.0, (64, 2): 1.5, (64, 1): 1.5, (128, 0): 1.7, (128, 2): 3.0, (128, 1): 9.0}
    assert tune.pick(t) == (64, 2)          # tie 1.5: the earlier candidate
    assert tune.pick({(128, 1): 1.0}) == (128, 1)


def test_cache_round_trip(tmp_path, monkeypatch, restore_table):
    monkeypatch.setenv("SPLIT_GB300_TUNE_DIR", str(tmp_path))
    es = [tune.Entry(5000, 128, 2), tune.Entry(tune.INT64_MAX, 64, 0)]
    path = tune.save(es, "Some-GPU-sm152", {"512x512": {"chosen": "rows128_bps2"}})
    assert path.startswith(str(tmp_path))
    assert tune.load_cached("Some-GPU-sm152") == es
    assert tune.load_cached("Other-GPU-sm1") is None
    (tmp_path / "tune-Broken-sm1.json").write_text("{not json")
    assert tune.load_cached("Broken-sm1") is None
