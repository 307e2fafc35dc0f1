"""The compact replay (short spans holding only the nodes their edge events
touch; tsg_cplan.cu, tsg_replay_compact.cuh) against the general replay and
the oracle.  Both replays emit the same items in the same order and value
them with the same arithmetic, so their results are bitwise equal whatever
the compact span count; the oracle pins both."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _run(ts, sets, terms, windows, precision, polarised=False, both=True):
    import torch

    import tskit_gb300

    q = ts.query(sets, terms, windows=windows, both_modes=both, mode="site",
                 span_normalise=False, precision=precision, polarised=polarised)
    ws = tskit_gb300.Workspace(q.workspace_bytes)
    res = torch.zeros(q.result_size, dtype=torch.float64, device="cuda")
    q.launch(ws, res)
    torch.cuda.synchronize()
    q.check(ws)
    return res.cpu().numpy()


CASES = [
    # n, L, breakpoints, sites, seed, sets
    (60, 1e5, 300, 600, 11, 2),
    (200, 1e6, 2000, 3000, 12, 4),
    (300, 1e6, 1500, 2000, 13, 8),
    (1000, 1e7, 5000, 6000, 14, 3),
]


@pytest.fixture(scope="module", params=CASES, ids=[f"n{c[0]}" for c in CASES])
def case(request, cuda_lib):
    import tskit_gb300
    from tskit_gb300 import sim

    n, L, b, s, seed, k = request.param
    tables = sim.simulate(n, L, b, s, seed)
    ts = tskit_gb300.TreeSequence(tables)
    rng = np.random.default_rng(seed)
    perm = rng.permutation(tables.samples())
    sets = [np.sort(p) for p in np.array_split(perm, k)]
    terms = [(O.DIVERSITY, (j,)) for j in range(k)] + [(O.SEGSITES, (0,))]
    terms += [(O.DIVERGENCE, (0, k - 1)), (O.Y3, (0, 1 % k, (k - 1))), (O.F4, (0, 1 % k, 0, k - 1))]
    windows = np.linspace(0, tables.sequence_length, 9)
    return ts, tables, sets, terms, windows


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("polarised", [False, True])
def test_compact_equals_general_replay(case, precision, polarised):
    ts, tables, sets, terms, windows = case
    assert ts.set_compact_spans(0) == 0
    general = _run(ts, sets, terms, windows, precision, polarised)
    built = []
    for num in (1, 5, 64, 10 ** 6):
        # a span count whose spans touch more nodes than a block's shared
        # memory holds leaves the general replay serving (0 compact spans)
        built.append(ts.set_compact_spans(num))
        got = _run(ts, sets, terms, windows, precision, polarised)
        np.testing.assert_array_equal(got, general)
    assert max(built) > 0
    ots = O.OracleTS(tables)
    res = general.reshape(2, len(windows) - 1, len(terms))
    for m, mode in enumerate(("branch", "site")):
        exp = O.sample_count_stat(ots, sets, terms, windows=windows, mode=mode,
                                  polarised=polarised, span_normalise=False)
        rtol = 1e-12 if precision == "f64" else 1e-5
        scale = np.max(np.abs(exp), axis=0)
        np.testing.assert_allclose(res[m], exp, rtol=rtol, atol=rtol * np.max(scale))


def test_compact_site_only_and_default_plan(case):
    ts, tables, sets, terms, windows = case
    ts.set_compact_spans(0)
    general = _run(ts, sets, terms, windows, "f64", both=False)
    assert ts.set_compact_spans(200) > 0
    got = _run(ts, sets, terms, windows, "f64", both=False)
    np.testing.assert_array_equal(got, general)


def test_query_prepared_before_a_larger_plan(case):
    """A query's workspace holds the compact replay's per-endpoint counts for
    the plan it was prepared against; after the plan is rebuilt with more
    spans the query still runs (on the general replay) with the same
    results, and a query prepared again uses the new plan."""
    import torch

    import tskit_gb300

    ts, tables, sets, terms, windows = case
    ts.set_compact_spans(0)
    general = _run(ts, sets, terms, windows, "f64")
    assert ts.set_compact_spans(2) > 0
    q = ts.query(sets, terms, windows=windows, both_modes=True, mode="site",
                 span_normalise=False, precision="f64")
    ws = tskit_gb300.Workspace(q.workspace_bytes)
    res = torch.zeros(q.result_size, dtype=torch.float64, device="cuda")
    built = ts.set_compact_spans(64)
    q.launch(ws, res)
    torch.cuda.synchronize()
    q.check(ws)
    np.testing.assert_array_equal(res.cpu().numpy(), general)
    if built > 0:
        np.testing.assert_array_equal(_run(ts, sets, terms, windows, "f64"), general)
    ts.set_compact_spans(-1)
