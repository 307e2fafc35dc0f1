"""tsg_treeseq_general_stat, the reference's C callback form of general_stat
(c/tskit/trees.h:1032-1036, c/tskit/trees.c:2035-2095), called through the C
ABI with a ctypes summary function: real-valued weights against the
reference's own values (tests/golden/make_weighted_golden.py), 0/1 weights
against the oracle, and the reference's argument errors."""
import ctypes
import os

import numpy as np
import pytest

import oracle as O
from weighted_summaries import SUMMARIES

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _callback(f, calls=None):
    from tskit_gb300 import _native as nat

    def cb(K, x, R, out, params):
        state = np.ctypeslib.as_array(x, shape=(K,)).copy()
        v = np.asarray(f(state), dtype=np.float64).reshape(-1)
        if v.shape[0] != R:
            return -100000
        for j in range(R):
            out[j] = v[j]
        if calls is not None:
            calls.append(state)
        return 0

    return nat.GENERAL_STAT_FUNC(cb)


def _general_stat(lib, ts, W, f, M, windows, options, calls=None):
    W = np.ascontiguousarray(W, dtype=np.float64)
    win = None if windows is None else np.ascontiguousarray(windows, dtype=np.float64)
    nw = 1 if win is None else len(win) - 1
    res = np.full((nw, M), np.nan)
    cb = _callback(f, calls)
    err = lib.tsg_treeseq_general_stat(
        ts._handle, W.shape[1], W.ctypes.data_as(ctypes.c_void_p), M,
        ctypes.cast(cb, ctypes.c_void_p), None, nw,
        None if win is None else win.ctypes.data_as(ctypes.c_void_p), options,
        res.ctypes.data_as(ctypes.c_void_p))
    return err, res


@pytest.mark.parametrize("name", ["a", "b"])
@pytest.mark.parametrize("fname", sorted(SUMMARIES))
@pytest.mark.parametrize("mode", ["site", "branch"])
@pytest.mark.parametrize("polarised", [False, True])
def test_callback_real_weights_golden(name, fname, mode, polarised, cuda_lib):
    import tskit_gb300
    from tskit_gb300 import _native as nat

    ts = tskit_gb300.load(os.path.join(GOLDEN, f"weighted_{name}.trees"))
    ref = np.load(os.path.join(GOLDEN, f"weighted_{name}.npz"))
    K, M, f = SUMMARIES[fname]
    options = (nat.STAT_SITE if mode == "site" else nat.STAT_BRANCH) | nat.STAT_SPAN_NORMALISE
    if polarised:
        options |= nat.STAT_POLARISED
    err, got = _general_stat(cuda_lib, ts, ref[f"W{K}"], f, M, ref["windows"], options)
    assert err == 0, err
    exp = ref[f"{fname}_{mode}_{int(polarised)}"]
    scale = np.max(np.abs(exp)) if exp.size else 1.0
    np.testing.assert_allclose(got, exp, rtol=1e-11, atol=1e-12 * scale)


@pytest.fixture(scope="module")
def medium(cuda_lib):
    import tskit_gb300
    from tskit_gb300 import sim

    tables = sim.simulate(120, 1e6, 800, 3000, 81)
    return tskit_gb300.TreeSequence(tables), O.OracleTS(tables), tables


@pytest.mark.parametrize("mode", ["site", "branch"])
@pytest.mark.parametrize("polarised", [False, True])
def test_callback_zero_one_weights(medium, mode, polarised, cuda_lib):
    from tskit_gb300 import _native as nat

    ts, ots, tables = medium
    rng = np.random.default_rng(3)
    perm = rng.permutation(tables.samples())
    sets = [np.sort(p) for p in np.array_split(perm, 2)]
    samples = tables.samples()
    W = np.stack([np.isin(samples, s) for s in sets], axis=1).astype(float)
    n = W.sum(axis=0)

    def f(x):
        return np.array([x[0] * (n[0] - x[0]) / (n[0] * (n[0] - 1)),
                         x[0] * (n[1] - x[1]) / (n[0] * n[1])])

    windows = np.linspace(0, tables.sequence_length, 5)
    options = (nat.STAT_SITE if mode == "site" else nat.STAT_BRANCH) | nat.STAT_SPAN_NORMALISE
    if polarised:
        options |= nat.STAT_POLARISED
    calls = []
    err, got = _general_stat(cuda_lib, ts, W, f, 2, windows, options, calls)
    assert err == 0, err
    exp = O.sample_count_stat(ots, sets, [(O.DIVERSITY, (0,)), (O.DIVERGENCE, (0, 1))],
                              windows=windows, mode=mode, polarised=polarised)
    np.testing.assert_allclose(got, exp, rtol=1e-12, atol=1e-14)
    # f sees count vectors only (each distinct one once, plus its complement
    # for the unpolarised branch sum)
    states = np.array(calls)
    assert np.all(states == np.round(states))
    assert np.all((states >= 0) & (states <= n))


def test_callback_default_mode_and_windows(medium, cuda_lib):
    ts, ots, tables = medium
    samples = tables.samples()
    W = np.ones((len(samples), 1))
    nn = float(len(samples))

    def f(x):
        return np.array([x[0] * (nn - x[0]) / (nn * (nn - 1))])

    err, got = _general_stat(cuda_lib, ts, W, f, 1, None, 0)
    assert err == 0, err
    # no mode bit: site mode; no windows: the whole genome, not normalised
    exp = O.sample_count_stat(ots, [samples], [(O.DIVERSITY, (0,))], mode="site",
                              span_normalise=False)
    np.testing.assert_allclose(got, exp, rtol=1e-12)


def test_callback_errors(medium, cuda_lib):
    from tskit_gb300 import _native as nat

    ts, _, tables = medium
    n = len(tables.samples())
    W = np.ones((n, 1))
    f = lambda x: np.array([0.0])  # noqa: E731
    err, _ = _general_stat(cuda_lib, ts, W, f, 1, None, nat.STAT_SITE | nat.STAT_BRANCH)
    assert err == nat.ERR_MULTIPLE_STAT_MODES
    err, _ = _general_stat(cuda_lib, ts, np.ones((n, 0)), f, 1, None, nat.STAT_SITE)
    assert err == -903  # TSK_ERR_BAD_STATE_DIMS
    err, _ = _general_stat(cuda_lib, ts, W, f, 0, None, nat.STAT_SITE)
    assert err == -904  # TSK_ERR_BAD_RESULT_DIMS
    err, _ = _general_stat(cuda_lib, ts, W, f, 1, np.array([0.0, 0.5 * tables.sequence_length]),
                           nat.STAT_SITE)
    assert err == nat.ERR_BAD_WINDOWS

    # a summary function that fails aborts the call with its own code
    def failing(K, x, R, out, params):
        return -7

    cb = nat.GENERAL_STAT_FUNC(failing)
    res = np.zeros((1, 1))
    err = cuda_lib.tsg_treeseq_general_stat(
        ts._handle, 1, W.ctypes.data_as(ctypes.c_void_p), 1, ctypes.cast(cb, ctypes.c_void_p),
        None, 1, None, nat.STAT_BRANCH, res.ctypes.data_as(ctypes.c_void_p))
    assert err == -7
