"""GPU parity: the CUDA path against the reference's golden outputs and the
oracle (FP64 form within 1e-12 relative; FP32-Kahan form within the stated
bound; integer-derived site statistics identical to the FP64 form)."""
import numpy as np
import pytest

import oracle as O
from golden_cases import all_cases, load, resolve

pytestmark = pytest.mark.gpu

GPU_METHODS = {
    "diversity", "segregating_sites", "Y1", "divergence", "Y2", "f2", "Y3", "f3", "f4",
    "genetic_relatedness", "Fst", "Tajimas_D", "allele_frequency_spectrum",
    "genetic_relatedness_vector", "genetic_relatedness_matrix", "divergence_matrix",
}
CASES = [(n, c) for n, c in all_cases() if c["method"] in GPU_METHODS]
_ts = {}

RTOL_F64 = 1e-12
# FP32 bulk evaluation: stated bound on relative error against the FP64
# oracle per window, relative to the statistic's scale (f2/f3/f4 are
# differences of products and lose the most; the others stay near 1e-7).
RTOL_F32 = 1e-5


def gpu_ts(name, cuda_lib):
    if name not in _ts:
        import tskit_gb300

        tables, data = load(name)
        _ts[name] = (tskit_gb300.TreeSequence(tables), data)
    return _ts[name]


@pytest.mark.parametrize("name,case", CASES, ids=[f"{n}-{c['key']}-{c['method']}" for n, c in CASES])
def test_golden(name, case, cuda_lib):
    ts, data = gpu_ts(name, cuda_lib)
    expected = data[case["key"]]
    got = np.asarray(getattr(ts, case["method"])(**resolve(case["kwargs"], data)))
    assert got.shape == expected.shape
    if case["method"] == "Tajimas_D":
        # D = (T - S/h) / sqrt(a S + b S (S-1)); for sets of 2-3 samples both
        # numerator and denominator vanish in exact arithmetic, so the sign
        # of the infinity depends on the last bit of T and S.  Where the
        # reference's value is not finite, require ours not finite too and
        # check T and S themselves.
        bad = ~np.isfinite(expected)
        assert np.all(~np.isfinite(got[bad]))
        got, expected = got[~bad], expected[~bad]
        kw = resolve(case["kwargs"], data)
        for m in ("diversity", "segregating_sites"):
            a = getattr(ts, m)(**dict(kw, span_normalise=False))
            b = O.call(O.OracleTS(ts.tables), m, dict(kw, span_normalise=False))
            np.testing.assert_allclose(np.ravel(a), np.ravel(b), rtol=RTOL_F64, atol=1e-13,
                                       equal_nan=True)
        # T - S/h cancels: D's relative error is that of T and S times
        # (|T| + |S/h|) / |T - S/h|, up to 1e4 on these fixtures
        np.testing.assert_allclose(got, expected, rtol=1e-8, atol=1e-13, equal_nan=True)
        return
    np.testing.assert_allclose(got, expected, rtol=RTOL_F64, atol=1e-13, equal_nan=True)


def test_known_answer_paper_ex(cuda_lib):
    """c/tests/test_stats.c:1718-1742"""
    ts, _ = gpu_ts("paper_ex", cuda_lib)
    assert abs(ts.diversity([0, 1, 2, 3], mode="site", span_normalise=False) - 1.5) < 1e-12
    assert np.isnan(ts.diversity([0], mode="site", span_normalise=False))


@pytest.fixture(scope="module")
def medium(cuda_lib):
    import tskit_gb300
    from tskit_gb300 import sim

    tables = sim.simulate(400, 1e6, 3000, 15000, 11)
    return tskit_gb300.TreeSequence(tables), O.OracleTS(tables), tables


def _sets(tables, k, seed=0):
    rng = np.random.default_rng(seed)
    perm = rng.permutation(tables.samples())
    return [np.sort(p) for p in np.array_split(perm, k)]


def _fused_terms(K):
    terms = [(O.DIVERSITY, (k,)) for k in range(K)]
    terms += [(O.SEGSITES, (k,)) for k in range(K)]
    terms += [(O.DIVERGENCE, (i, j)) for i in range(K) for j in range(i + 1, K)]
    terms += [(O.Y3, (0, 1, 2)), (O.Y3, (1, 2, 3)), (O.F4, (0, 1, 2, 3))]
    return terms


@pytest.mark.parametrize("precision,sweep", [("f64", "auto"), ("f32", "auto"),
                                             ("f64", "global"), ("f64", "global_state"),
                                             ("f32", "global_state")])
@pytest.mark.parametrize("polarised", [False, True])
def test_fused_both_modes_vs_oracle(medium, precision, sweep, polarised):
    import torch

    ts, ots, tables = medium
    sets = _sets(tables, 4)
    terms = _fused_terms(4)
    windows = np.linspace(0, tables.sequence_length, 17)
    q = ts.query(sets, terms, windows=windows, both_modes=True, polarised=polarised,
                 precision=precision, sweep=sweep)
    ws = __import__("tskit_gb300").Workspace()
    res = torch.zeros(q.result_size, dtype=torch.float64, device="cuda")
    q.launch(ws, res)
    torch.cuda.synchronize()
    q.check(ws)
    got = res.cpu().numpy().reshape(2, len(windows) - 1, len(terms))
    for m, mode in enumerate(["branch", "site"]):
        exp = O.sample_count_stat(ots, sets, terms, windows=windows, mode=mode,
                                  polarised=polarised)
        rtol = RTOL_F64 if (precision == "f64" or mode == "site") else RTOL_F32
        # per-window error relative to the statistic's magnitude (a term that
        # crosses zero inside the windows is measured against its scale)
        scale = np.maximum(np.abs(exp), np.abs(exp).max(axis=0, keepdims=True) * 1e-2)
        err = np.abs(got[m] - exp) / scale
        assert np.nanmax(err) < rtol, (mode, precision, np.nanmax(err))


def test_deterministic(medium):
    ts, _, tables = medium
    sets = _sets(tables, 3, seed=5)
    a = ts.divergence(sets, indexes=[(0, 1), (1, 2)], windows=np.linspace(0, 1e6, 9),
                      mode="branch")
    b = ts.divergence(sets, indexes=[(0, 1), (1, 2)], windows=np.linspace(0, 1e6, 9),
                      mode="branch")
    np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("num_spans", [1, 2, 7, 64, 1000])
def test_span_count_invariance(cuda_lib, num_spans):
    """The span decomposition changes only the summation order."""
    import tskit_gb300
    from tskit_gb300 import sim

    tables = sim.simulate(60, 1e5, 300, 1500, 4)
    ts = tskit_gb300.TreeSequence(tables, num_spans=num_spans)
    ots = O.OracleTS(tables)
    sets = _sets(tables, 2, seed=1)
    w = np.linspace(0, 1e5, 5)
    for mode in ("branch", "site"):
        got = ts.divergence(sets, windows=w, mode=mode)
        exp = O.k_way(ots, O.DIVERGENCE, sets, [(0, 1)], windows=w, mode=mode)[:, 0]
        np.testing.assert_allclose(got, exp, rtol=RTOL_F64)


def test_errors_match_reference_codes(medium):
    import tskit_gb300

    ts, _, tables = medium
    s = list(tables.samples()[:10])
    with pytest.raises(tskit_gb300.LibraryError) as e:
        ts.diversity([s + [s[0]]])
    assert e.value.code == -600  # TSK_ERR_DUPLICATE_SAMPLE
    with pytest.raises(tskit_gb300.LibraryError) as e:
        ts.diversity([s], windows=[0, 10, 5, tables.sequence_length])
    assert e.value.code == -901  # TSK_ERR_BAD_WINDOWS
    with pytest.raises(tskit_gb300.LibraryError) as e:
        ts.diversity([[tables.num_nodes - 1]])
    assert e.value.code == -601  # TSK_ERR_BAD_SAMPLES
    with pytest.raises(ValueError):
        ts.diversity([s], mode="nonsense")


def test_large_branch_only_repeatable(cuda_lib):
    """Spans with thousands of alive nodes: repeated single-mode launches are
    bit-identical and match the oracle (guards the ordering between the seek,
    the first-tree items and the replay)."""
    import torch

    import tskit_gb300
    from tskit_gb300 import sim

    tables = sim.simulate(3000, 1e7, 20000, 60000, 8)
    ts = tskit_gb300.TreeSequence(tables)
    ots = O.OracleTS(tables)
    sets = _sets(tables, 4, seed=2)
    windows = np.linspace(0, tables.sequence_length, 101)
    terms = [(O.DIVERSITY, (k,)) for k in range(4)]
    exp = O.sample_count_stat(ots, sets, terms, windows=windows, mode="branch")
    q = ts.query(sets, terms, windows=windows, mode="branch", precision="f64")
    ws = tskit_gb300.Workspace(q.workspace_bytes)
    outs = []
    for _ in range(3):
        r = torch.zeros(q.result_size, dtype=torch.float64, device="cuda")
        q.launch(ws, r)
        torch.cuda.synchronize()
        q.check(ws)
        outs.append(r.cpu().numpy().reshape(exp.shape))
    for o in outs[1:]:
        np.testing.assert_array_equal(o, outs[0])
    np.testing.assert_allclose(outs[0], exp, rtol=RTOL_F64)


@pytest.mark.parametrize("n,breaks", [(20000, 400), (70000, 60)])
def test_global_state_form_large_n(cuda_lib, n, breaks):
    """Spans whose node state exceeds shared memory (n = 20000), and sample
    sets above the 16-bit count range (n = 70000), run the item pipeline with
    node state in global memory and 32-bit counts."""
    import tskit_gb300
    from tskit_gb300 import sim

    tables = sim.simulate(n, 1e6, breaks, 3000, 12)
    ts = tskit_gb300.TreeSequence(tables)
    ots = O.OracleTS(tables)
    sets = [tables.samples()] if n > 65535 else _sets(tables, 3, seed=4)
    terms = [(O.DIVERSITY, (k,)) for k in range(len(sets))]
    terms += [(O.SEGSITES, (0,))]
    if len(sets) > 1:
        terms += [(O.DIVERGENCE, (0, 1)), (O.Y3, (0, 1, 2))]
    windows = np.linspace(0, tables.sequence_length, 5)
    for mode in ("branch", "site"):
        exp = O.sample_count_stat(ots, sets, terms, windows=windows, mode=mode)
        for precision in ("f64", "f32"):
            import torch

            q = ts.query(sets, terms, windows=windows, mode=mode, precision=precision)
            ws = tskit_gb300.Workspace(q.workspace_bytes)
            r = torch.zeros(q.result_size, dtype=torch.float64, device="cuda")
            q.launch(ws, r)
            torch.cuda.synchronize()
            q.check(ws)
            got = r.cpu().numpy().reshape(exp.shape)
            rtol = RTOL_F64 if (precision == "f64" or mode == "site") else RTOL_F32
            np.testing.assert_allclose(got, exp, rtol=rtol, err_msg=f"{mode} {precision}")


@pytest.mark.parametrize("mode", ["site", "branch"])
def test_many_sets_and_outputs_split(medium, mode):
    """More sets than one sweep holds (40 > 32) and more outputs (105 > 64):
    groups of outputs swept with just their sets, columns back in place;
    against the oracle.  The centred relatedness over more than 32 sets is
    refused (its mean runs over every set)."""
    import tskit_gb300

    ts, ots, tables = medium
    sets = _sets(tables, 40, seed=3)
    win = np.linspace(0, tables.sequence_length, 4)
    got = ts.diversity(sets, windows=win, mode=mode)
    exp = O.one_way(ots, O.DIVERSITY, sets, windows=win, mode=mode)
    np.testing.assert_allclose(got, exp, rtol=RTOL_F64, atol=1e-13)
    sets15 = sets[:15]
    pairs = [(i, j) for i in range(15) for j in range(i, 15)][:105]
    got = ts.divergence(sets15, indexes=pairs, windows=win, mode=mode)
    exp = O.k_way(ots, O.DIVERGENCE, sets15, pairs, windows=win, mode=mode)
    np.testing.assert_allclose(got, exp, rtol=RTOL_F64, atol=1e-13)
    triples = [(i, (i + 7) % 40, (i + 19) % 40) for i in range(40)]
    got = ts.Y3(sets, indexes=triples, windows=win, mode=mode)
    exp = O.k_way(ots, O.Y3, sets, triples, windows=win, mode=mode)
    np.testing.assert_allclose(got, exp, rtol=RTOL_F64, atol=1e-13)
    with pytest.raises(tskit_gb300.LibraryError):
        ts.genetic_relatedness(sets, indexes=[(0, 1)], mode=mode, proportion=False)
    # a duplicate sample in a set no output uses is still an error
    bad = [list(s) for s in sets[:33]]
    bad[32] = bad[32] + [bad[32][0]]
    with pytest.raises(tskit_gb300.LibraryError) as e:
        ts.divergence(bad, indexes=[(0, 1)], mode=mode)
    assert e.value.code == -600


def test_many_sets_node_mode(medium):
    ts, ots, tables = medium
    sets = _sets(tables, 36, seed=4)
    got = ts.diversity(sets, mode="node")
    exp = O.one_way(ots, O.DIVERSITY, sets, mode="node")
    np.testing.assert_allclose(got, np.asarray(exp).reshape(got.shape), rtol=RTOL_F64,
                               atol=1e-13)
