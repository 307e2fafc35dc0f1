"""GPU parity of general_stat / sample_count_stat with Python summary
functions: functions equal to the built-in statistics' summaries must give
the built-in statistics (oracle), and every call evaluates f only at count
vectors the tree sequence produces."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def medium(cuda_lib):
    import tskit_gb300
    from tskit_gb300 import sim

    tables = sim.simulate(120, 1e6, 800, 3000, 81)
    return tskit_gb300.TreeSequence(tables), O.OracleTS(tables), tables


def _sets(tables, k, seed=0):
    rng = np.random.default_rng(seed)
    perm = rng.permutation(tables.samples())
    return [np.sort(p) for p in np.array_split(perm, k)]


@pytest.mark.parametrize("mode", ["site", "branch"])
@pytest.mark.parametrize("polarised", [False, True])
def test_sample_count_stat_diversity_divergence(medium, mode, polarised):
    ts, ots, tables = medium
    sets = _sets(tables, 3)
    n = np.array([len(s) for s in sets], dtype=float)

    def f(x):
        return np.array([x[0] * (n[0] - x[0]) / (n[0] * (n[0] - 1)),
                         x[1] * (n[2] - x[2]) / (n[1] * n[2]),
                         x[0] * (n[1] - x[1]) * (n[2] - x[2]) / (n[0] * n[1] * n[2])])

    windows = np.linspace(0, tables.sequence_length, 6)
    got = ts.sample_count_stat(sets, f, 3, windows=windows, mode=mode, polarised=polarised,
                               strict=False)
    terms = [(O.DIVERSITY, (0,)), (O.DIVERGENCE, (1, 2)), (O.Y3, (0, 1, 2))]
    exp = O.sample_count_stat(ots, sets, terms, windows=windows, mode=mode, polarised=polarised)
    np.testing.assert_allclose(got, exp, rtol=1e-12, atol=1e-14)


def test_general_stat_weights_and_many_outputs(medium):
    ts, ots, tables = medium
    sets = _sets(tables, 2, seed=4)
    samples = tables.samples()
    W = np.stack([np.isin(samples, s) for s in sets], axis=1).astype(float)
    n = W.sum(axis=0)

    def f(x):
        # 40 outputs (two blocks of the device accumulators)
        base = x[0] * (n[0] - x[0]) / (n[0] * (n[0] - 1))
        return np.array([base * (j + 1) for j in range(40)])

    got = ts.general_stat(W, f, 40, mode="branch", windows=np.linspace(0, 1e6, 3))
    exp = O.sample_count_stat(ots, [sets[0]], [(O.DIVERSITY, (0,))], mode="branch",
                              windows=np.linspace(0, 1e6, 3))
    for j in range(40):
        np.testing.assert_allclose(got[:, j], exp[:, 0] * (j + 1), rtol=1e-12)


def test_general_stat_strict(medium):
    ts, _, tables = medium
    W = np.ones((tables.samples().size, 1))
    with pytest.raises(ValueError):
        ts.general_stat(W, lambda x: np.array([1.0]), 1)
