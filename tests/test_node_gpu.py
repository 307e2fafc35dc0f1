"""Node-mode statistics (one output row per node, trees.c:1788-1918) against
the reference's own values (tests/golden/make_node_golden.py): general_stat
with real-valued weights, sample_count_stat with a user summary and
genetic_relatedness_weighted, polarised or not, on simulated tree sequences
and on one with internal samples.  The built-in sample-set statistics in
node mode run through the golden cases of test_stats_gpu.py."""
import os

import numpy as np
import pytest

from weighted_summaries import COUNT_SUMMARIES, SUMMARIES

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TREES = {"a": "weighted_a.trees", "b": "weighted_b.trees", "internal": "node_internal.trees"}


def _check(got, exp):
    assert got.shape == exp.shape
    scale = np.max(np.abs(exp)) if exp.size else 1.0
    np.testing.assert_allclose(got, exp, rtol=1e-11, atol=1e-12 * scale)


def _load(name):
    import tskit_gb300

    return (tskit_gb300.load(os.path.join(GOLDEN, TREES[name])),
            np.load(os.path.join(GOLDEN, f"node_{name}.npz")))


@pytest.mark.parametrize("name", sorted(TREES))
@pytest.mark.parametrize("fname", sorted(SUMMARIES))
@pytest.mark.parametrize("polarised", [False, True])
def test_general_stat_node(name, fname, polarised, cuda_lib):
    ts, ref = _load(name)
    K, M, f = SUMMARIES[fname]
    got = ts.general_stat(ref[f"W{K}"], f, M, windows=ref["windows"], mode="node",
                          polarised=polarised, strict=False)
    _check(got, ref[f"general_{fname}_{int(polarised)}"])


@pytest.mark.parametrize("name", sorted(TREES))
@pytest.mark.parametrize("fname", sorted(COUNT_SUMMARIES))
@pytest.mark.parametrize("polarised", [False, True])
def test_sample_count_stat_node(name, fname, polarised, cuda_lib):
    ts, ref = _load(name)
    sizes, M, f = COUNT_SUMMARIES[fname]
    samples = ts.samples()
    sets, at = [], 0
    for s in sizes:
        sets.append(samples[at:at + s])
        at += s
    got = ts.sample_count_stat(sets, f, M, windows=ref["windows"], mode="node",
                               polarised=polarised, strict=False)
    _check(got, ref[f"count_{fname}_{int(polarised)}"])


@pytest.mark.parametrize("name", sorted(TREES))
@pytest.mark.parametrize("centre", [True, False])
@pytest.mark.parametrize("polarised", [False, True])
def test_relatedness_weighted_node(name, centre, polarised, cuda_lib):
    ts, ref = _load(name)
    got = ts.genetic_relatedness_weighted(ref["Wr"], indexes=[(0, 1), (2, 2)], mode="node",
                                          polarised=polarised, centre=centre)
    _check(got, ref[f"grw_{int(centre)}_{int(polarised)}"])


def test_node_mode_errors(cuda_lib):
    from tskit_gb300 import LibraryError
    from tskit_gb300 import _native as nat

    ts, _ = _load("a")
    s = list(ts.samples())
    # the allele frequency spectrum has no node mode (trees.c:3900-3903)
    with pytest.raises(LibraryError) as e:
        ts.allele_frequency_spectrum([s], mode="node")
    assert e.value.code == nat.ERR_UNSUPPORTED_STAT_MODE
    # real weights take at most 32 columns here
    ts_b, _ = _load("b")
    with pytest.raises(LibraryError) as e:
        ts_b.general_stat(np.random.default_rng(1).normal(size=(ts_b.num_samples, 33)),
                          lambda x: x[:1], 1, mode="node", strict=False)
    assert e.value.code == nat.ERR_TOO_MANY_SAMPLE_SETS


@pytest.mark.parametrize("mode", ["node", "branch", "site"])
def test_many_sets_weighted_paths(mode, cuda_lib):
    """More than 8 sets or weight columns: the weighted replay reads the
    child's state per component.  Node mode against the oracle; real
    weights in every mode against the same statistic from 0/1 weights
    scaled (general_stat is linear in a summary that is linear)."""
    import oracle as O

    ts, _ = _load("b")
    s = ts.samples()
    sets = [s[4 * k:4 * k + 4] for k in range(10)]
    if mode == "node":
        got = ts.diversity(sets, windows=[0, ts.sequence_length / 2, ts.sequence_length],
                           mode="node")
        exp = O.call(O.OracleTS(ts.tables), "diversity",
                     dict(sample_sets=sets, windows=[0, ts.sequence_length / 2,
                                                     ts.sequence_length], mode="node"))
        np.testing.assert_allclose(got, np.asarray(exp).reshape(got.shape), rtol=1e-12,
                                   atol=1e-13)
    rng = np.random.default_rng(3)
    W = rng.normal(size=(ts.num_samples, 12))

    def f(x):
        return np.array([np.sum(x), x[11] - 2 * x[0]])

    got = ts.general_stat(W, f, 2, mode=mode, polarised=True, strict=False)
    # f linear: the statistic of W equals that of its column sums' combination
    v = W.sum(axis=1, keepdims=True), (W[:, 11] - 2 * W[:, 0])[:, None]
    exp = np.concatenate([ts.general_stat(v[0], lambda x: x, 1, mode=mode, polarised=True,
                                          strict=False),
                          ts.general_stat(v[1], lambda x: x, 1, mode=mode, polarised=True,
                                          strict=False)], axis=-1)
    np.testing.assert_allclose(got, exp, rtol=1e-10, atol=1e-10 * np.max(np.abs(exp)))


def test_node_mode_deterministic(cuda_lib):
    ts, _ = _load("b")
    s = ts.samples()
    sets = [s[:20], s[20:]]
    a = ts.divergence(sets, windows=[0, ts.sequence_length / 2, ts.sequence_length], mode="node")
    b = ts.divergence(sets, windows=[0, ts.sequence_length / 2, ts.sequence_length], mode="node")
    assert np.array_equal(a, b)
