"""The span-count autotuner: selection logic with host fakes (no GPU) and, on
a GPU, a tuned tree sequence whose statistics equal the default plan's."""
import numpy as np
import pytest

from tskit_gb300 import tune


class FakeTS:
    def __init__(self, n, num_trees=1000):
        self.num_spans = n if n > 0 else 297
        self.num_trees = num_trees
        self.num_edges = 4000
        self.num_samples = 100


def fake_timer(ms_of):
    calls = []

    def timer(step, steps, warmup):
        calls.append(step())
        return ms_of[calls[-1]]
    return timer, calls


def test_candidates_bounded_by_trees():
    assert tune.span_candidates(297, 10_000, 152) == [76, 152, 297, 304, 456, 608]
    assert tune.span_candidates(5, 40, 152) == [5, 40]


def test_picks_fastest_and_reports_every_count():
    ms = {297: 2.2, 76: 3.0, 152: 2.5, 304: 2.1, 456: 2.4, 608: 2.9}
    timer, calls = fake_timer(ms)
    ts, rep = tune.tune_num_spans(None, lambda t: (lambda: t.num_spans), build=FakeTS,
                                  timer=timer, num_sms=152)
    assert ts.num_spans == 304 and rep["num_spans"] == 304 and not rep["cached"]
    assert rep["ms"] == ms
    assert calls[0] == 297  # the default plan is timed first


def test_ties_go_to_fewer_spans_and_duplicates_timed_once():
    ms = {297: 2.0, 152: 2.0, 40: 9.0}
    timer, calls = fake_timer(ms)

    def build(n):
        return FakeTS(min(n, 40) if n not in (0, 152, 297) else n)
    ts, rep = tune.tune_num_spans(None, lambda t: (lambda: t.num_spans), build=build,
                                  timer=timer, candidates=[40, 80, 152, 297], num_sms=152)
    assert ts.num_spans == 152
    assert sorted(calls) == [40, 152, 297]


def test_cache_skips_measurement():
    cache = {}
    timer, calls = fake_timer({297: 2.0, 76: 1.0, 152: 3.0, 304: 3.0, 456: 3.0, 608: 3.0})
    ts, rep = tune.tune_num_spans(None, lambda t: (lambda: t.num_spans), key="w", cache=cache,
                                  build=FakeTS, timer=timer, num_sms=152)
    assert ts.num_spans == 76 and len(cache) == 1
    n = len(calls)
    ts2, rep2 = tune.tune_num_spans(None, lambda t: (lambda: t.num_spans), key="w",
                                    cache=cache, build=FakeTS, timer=timer, num_sms=152)
    assert ts2.num_spans == 76 and rep2["cached"] and len(calls) == n


@pytest.mark.gpu
def test_tuned_plan_same_statistics():
    import tskit_gb300
    from tskit_gb300 import sim

    tables = sim.simulate(300, 1e6, 600, 3000, 31)
    rng = np.random.default_rng(5)
    sets = [np.sort(p) for p in np.array_split(rng.permutation(tables.samples()), 3)]
    windows = np.linspace(0, tables.sequence_length, 7)

    def make_step(ts):
        return lambda: ts.diversity(sets, windows=windows, mode="branch")
    ts, rep = tune.tune_num_spans(tables, make_step, candidates=[1, 3, 17], steps=2, warmup=1)
    assert rep["num_spans"] in rep["ms"] and len(rep["ms"]) >= 3
    ref = tskit_gb300.TreeSequence(tables)
    for mode in ("branch", "site"):
        np.testing.assert_allclose(ts.diversity(sets, windows=windows, mode=mode),
                                   ref.diversity(sets, windows=windows, mode=mode),
                                   rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(
            ts.divergence(sets, indexes=[(0, 1), (1, 2)], windows=windows, mode=mode),
            ref.divergence(sets, indexes=[(0, 1), (1, 2)], windows=windows, mode=mode),
            rtol=1e-12, atol=1e-14)


class FakeCompactTS:
    """Host stand-in for a tree sequence with a compact plan."""

    def __init__(self, default=1000, num_trees=10_000, cap=None):
        self.num_compact_spans = default
        self.num_trees = num_trees
        self.num_edges = 4000
        self.num_samples = 100
        self.cap = cap
        self.built = []

    def set_compact_spans(self, n):
        self.built.append(n)
        if n < 0:
            n = 1000
        self.num_compact_spans = 0 if (self.cap and n > self.cap) else n
        return self.num_compact_spans


def test_compact_candidates():
    assert tune.compact_candidates(1000, 10_000) == [500, 750, 1000, 1250, 1500, 2000]
    assert tune.compact_candidates(1000, 1300) == [500, 750, 1000, 1250, 1300]


def test_tune_compact_picks_fastest_and_skips_unbuildable():
    ts = FakeCompactTS(cap=1800)
    ms = {1000: 2.0, 500: 2.5, 750: 2.2, 1250: 1.8, 1500: 1.7}
    timer, calls = fake_timer(ms)
    rep = tune.tune_compact_spans(ts, lambda t: (lambda: t.num_compact_spans), timer=timer)
    assert rep["num_spans"] == 1500 and ts.num_compact_spans == 1500
    assert rep["ms"] == ms          # 2000 spans could not be built: not timed
    assert calls[0] == 1000         # the default plan first
    cache = {}
    timer2, _ = fake_timer({**ms, 1125: 1.9})
    tune.tune_compact_spans(ts, lambda t: (lambda: t.num_compact_spans), timer=timer2,
                            cache=cache)
    ts2 = FakeCompactTS(cap=1800)
    rep2 = tune.tune_compact_spans(ts2, lambda t: (lambda: 0), cache=cache)
    assert rep2["cached"] and ts2.num_compact_spans == 1500


def test_tune_compact_without_plan():
    ts = FakeCompactTS(default=0)
    rep = tune.tune_compact_spans(ts, lambda t: (lambda: 0), timer=lambda *a: 1.0)
    assert rep == {"num_spans": 0, "ms": {}, "cached": False}


def test_cache_round_trip_and_key(tmp_path):
    cache = {}
    timer, _ = fake_timer({297: 2.0, 76: 1.0, 152: 3.0, 304: 3.0, 456: 3.0, 608: 3.0})
    tune.tune_num_spans(None, lambda t: (lambda: t.num_spans), key="diversity", cache=cache,
                        build=FakeTS, timer=timer, num_sms=152)
    (key, val), = cache.items()
    assert key.startswith("diversity|edges=4000|trees=1000|samples=100|sms=") and val == 76
    path = str(tmp_path / "tune.json")
    tune.save_cache(cache, path)
    assert tune.load_cache(path) == cache
    assert tune.load_cache(str(tmp_path / "missing.json")) == {}
