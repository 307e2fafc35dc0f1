"""GPU parity of the branch genetic relatedness matrix-vector product
(genetic_relatedness_vector) against the oracle (FP64, 1e-12 relative to the
output's scale per window)."""
import numpy as np
import pytest

import oracle as O
from ts_gaps import with_gaps

pytestmark = pytest.mark.gpu

RTOL = 1e-12


@pytest.fixture(scope="module")
def medium(cuda_lib):
    import tskit_gb300
    from tskit_gb300 import sim

    tables = sim.simulate(250, 1e6, 1500, 4000, 41)
    return tskit_gb300.TreeSequence(tables), O.OracleTS(tables), tables


def _check(ts, ots, W, **kw):
    got = ts.genetic_relatedness_vector(W, mode="branch", **kw)
    exp = O.genetic_relatedness_vector(ots, W, **kw)
    exp = exp.reshape(got.shape)
    # per window, relative to the window's largest output
    g = got.reshape(-1, *got.shape[-2:]) if got.ndim == 3 else got[None]
    e = exp.reshape(g.shape)
    for w in range(e.shape[0]):
        scale = max(np.abs(e[w]).max(), 1e-300)
        np.testing.assert_allclose(g[w], e[w], rtol=RTOL, atol=RTOL * scale)
    return got


@pytest.mark.parametrize("ncol", [1, 5, 32, 70])
@pytest.mark.parametrize("centre", [True, False])
def test_matvec_vs_oracle(medium, ncol, centre):
    ts, ots, tables = medium
    rng = np.random.default_rng(ncol)
    W = rng.normal(size=(tables.samples().size, ncol))
    L = tables.sequence_length
    for windows in (None, np.linspace(0, L, 7), [0.1 * L, 0.35 * L, 0.8 * L]):
        _check(ts, ots, W, windows=windows, centre=centre)
    _check(ts, ots, W, windows=np.linspace(0, L, 4), centre=centre, span_normalise=False)


def test_matvec_focal_nodes(medium):
    ts, ots, tables = medium
    rng = np.random.default_rng(2)
    W = rng.normal(size=(tables.samples().size, 3))
    samples = tables.samples()
    internal = np.arange(len(samples), tables.num_nodes, 97)
    nodes = np.concatenate([samples[::3], internal, samples[:4]])
    _check(ts, ots, W, windows=np.linspace(0, tables.sequence_length, 5), centre=False,
           nodes=nodes)


@pytest.mark.parametrize("num_spans", [1, 3, 40])
def test_matvec_span_counts_and_gaps(cuda_lib, num_spans):
    import tskit_gb300
    from tskit_gb300 import sim

    tables = with_gaps(sim.simulate(60, 1e5, 300, 600, 17), 3, frac=0.2)
    ts = tskit_gb300.TreeSequence(tables, num_spans=num_spans)
    ots = O.OracleTS(tables)
    W = np.random.default_rng(5).normal(size=(tables.samples().size, 4))
    for windows in (None, np.linspace(0, 1e5, 9), [2e4, 2.5e4, 9e4]):
        _check(ts, ots, W, windows=windows)
        _check(ts, ots, W, windows=windows, centre=False)


def test_matvec_large_n(cuda_lib):
    import tskit_gb300
    from tskit_gb300 import sim

    tables = sim.simulate(20000, 1e6, 300, 1000, 23)
    ts = tskit_gb300.TreeSequence(tables)
    ots = O.OracleTS(tables)
    W = np.random.default_rng(1).normal(size=(tables.samples().size, 40))
    _check(ts, ots, W, windows=np.linspace(0, 1e6, 3))


def test_matvec_repeatable(medium):
    ts, _, tables = medium
    W = np.random.default_rng(9).normal(size=(tables.samples().size, 8))
    a = ts.genetic_relatedness_vector(W, mode="branch", windows=np.linspace(0, 1e6, 4))
    b = ts.genetic_relatedness_vector(W, mode="branch", windows=np.linspace(0, 1e6, 4))
    np.testing.assert_array_equal(a, b)


def test_matvec_errors(medium):
    import tskit_gb300

    ts, _, tables = medium
    W = np.ones((tables.samples().size, 2))
    with pytest.raises(tskit_gb300.LibraryError) as e:
        ts.genetic_relatedness_vector(W, mode="site")
    assert e.value.code == -909
    with pytest.raises(tskit_gb300.LibraryError) as e:
        ts.genetic_relatedness_vector(W, mode="branch", windows=[0, 2e6])
    assert e.value.code == -901
    with pytest.raises(tskit_gb300.LibraryError) as e:
        ts.genetic_relatedness_vector(W, mode="branch", nodes=[tables.num_nodes], centre=False)
    assert e.value.code == -202
    with pytest.raises(ValueError):
        ts.genetic_relatedness_vector(W[:-1], mode="branch")
