"""GPU parity of the allele frequency spectrum against the oracle.

Site mode is exact (integer counts, sums of halves); branch mode sums its
areas exactly and rounds once per bin, so it agrees with the reference's
FP64 running sums to their own rounding (tests use 1e-12 relative)."""
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

    tables = sim.simulate(300, 1e6, 2000, 8000, 31)
    return tskit_gb300.TreeSequence(tables), O.OracleTS(tables), tables


def _sets(tables, k, size=None, seed=0):
    rng = np.random.default_rng(seed)
    perm = rng.permutation(tables.samples())
    if size is not None:
        perm = perm[: k * size]
    return [np.sort(p) for p in np.array_split(perm, k)]


def _check(ts, ots, sets, **kw):
    got = ts.allele_frequency_spectrum(sets, **kw)
    exp = O.allele_frequency_spectrum(ots, sets, **kw)
    exp = exp.reshape(got.shape)
    scale = np.abs(exp).max()
    np.testing.assert_allclose(got, exp, rtol=RTOL, atol=1e-14 * max(scale, 1e-300))
    return got


@pytest.mark.parametrize("mode", ["site", "branch"])
@pytest.mark.parametrize("polarised", [False, True])
@pytest.mark.parametrize("nsets", [1, 2, 3])
def test_afs_vs_oracle(medium, mode, polarised, nsets):
    ts, ots, tables = medium
    sets = [tables.samples()] if nsets == 1 else _sets(tables, nsets, size=12 if nsets == 3 else 40)
    windows = np.linspace(0, tables.sequence_length, 6)
    for w in (None, windows):
        _check(ts, ots, sets, windows=w, mode=mode, polarised=polarised)
    _check(ts, ots, sets, windows=windows, mode=mode, polarised=polarised, span_normalise=False)


def test_afs_time_windows(medium):
    ts, ots, tables = medium
    sets = _sets(tables, 2, size=30, seed=3)
    for tw in ([0, 0.05, np.inf], [0, 0.01, 0.1, 0.5, 2.0], [0, 1e-3]):
        _check(ts, ots, sets, windows=np.linspace(0, tables.sequence_length, 4),
               time_windows=tw, mode="branch")
        _check(ts, ots, [tables.samples()], time_windows=tw, mode="branch", polarised=True)


@pytest.mark.parametrize("mode", ["site", "branch"])
def test_afs_parentless_stretches(cuda_lib, mode):
    """Isolated leaves and temporary extra roots (split edges)."""
    import tskit_gb300
    from tskit_gb300 import sim

    tables = with_gaps(sim.simulate(80, 1e5, 300, 1200, 9), 5, frac=0.2)
    ts = tskit_gb300.TreeSequence(tables, num_spans=17)
    ots = O.OracleTS(tables)
    w = np.linspace(0, tables.sequence_length, 8)
    for sets in ([tables.samples()], _sets(tables, 2, seed=4)):
        for pol in (False, True):
            _check(ts, ots, sets, windows=w, mode=mode, polarised=pol)
            _check(ts, ots, sets, mode=mode, polarised=pol)


@pytest.mark.parametrize("n", [20000, 70000])
def test_afs_global_state_form(cuda_lib, n):
    """Node state in global memory (spans too large for shared memory, or
    sample counts above 16 bits)."""
    import tskit_gb300
    from tskit_gb300 import sim

    tables = sim.simulate(n, 1e6, 150 if n > 65535 else 400, 3000, 13)
    ts = tskit_gb300.TreeSequence(tables)
    ots = O.OracleTS(tables)
    w = np.linspace(0, tables.sequence_length, 4)
    for mode in ("site", "branch"):
        _check(ts, ots, [tables.samples()], windows=w, mode=mode)
        _check(ts, ots, _sets(tables, 2, size=50, seed=1), windows=w, mode=mode)


def test_afs_repeatable(medium):
    ts, _, tables = medium
    sets = _sets(tables, 2, size=60, seed=7)
    a = ts.allele_frequency_spectrum(sets, mode="branch", windows=np.linspace(0, 1e6, 5))
    b = ts.allele_frequency_spectrum(sets, mode="branch", windows=np.linspace(0, 1e6, 5))
    np.testing.assert_array_equal(a, b)


def test_afs_errors(medium):
    import tskit_gb300

    ts, _, tables = medium
    s = [tables.samples()[:10]]
    with pytest.raises(tskit_gb300.LibraryError) as e:
        ts.allele_frequency_spectrum(s, mode="site", time_windows=[0, 1, np.inf])
    assert e.value.code == -909  # TSK_ERR_UNSUPPORTED_STAT_MODE
    with pytest.raises(tskit_gb300.LibraryError) as e:
        ts.allele_frequency_spectrum(s, mode="branch", time_windows=[0.5, 1])
    assert e.value.code == -924  # TSK_ERR_BAD_TIME_WINDOWS
    with pytest.raises(tskit_gb300.LibraryError) as e:
        ts.allele_frequency_spectrum(s, mode="node")
    assert e.value.code == -909
