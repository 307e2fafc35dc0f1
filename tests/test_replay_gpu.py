"""GPU parity of the item replay on inputs that stress its bookkeeping:
transitions that replace whole trees (each touches far more nodes than one
touch list holds, so lists close mid-transition) and span counts from one
span to one span per tree (the spans' running sums are chained by a scan)."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

RTOL_F64 = 1e-12
RTOL_F32 = 1e-5


def reshuffled_tables(n, ntrees, sites_per_tree, seed):
    """ntrees independent random binary trees on samples 0..n-1, tree j on
    [j, j + 1): every transition removes all edges and inserts new ones."""
    from tskit_gb300.tables import Tables

    rng = np.random.default_rng(seed)
    node_time = [0.0] * n
    flags = [1] * n
    left, right, parent, child = [], [], [], []
    site_pos, mut_site, mut_node = [], [], []
    for j in range(ntrees):
        lineages = list(range(n))
        t = 0.0
        tree_nodes = []
        while len(lineages) > 1:
            k = len(lineages)
            t += rng.exponential(2.0 / (k * (k - 1)))
            a, b = rng.choice(k, size=2, replace=False)
            u = len(node_time)
            node_time.append(t)
            flags.append(0)
            for c in (lineages[a], lineages[b]):
                left.append(j)
                right.append(j + 1)
                parent.append(u)
                child.append(c)
            tree_nodes.extend([lineages[a], lineages[b]])
            lineages = [x for i, x in enumerate(lineages) if i not in (a, b)] + [u]
        for pos in np.sort(rng.uniform(j, j + 1, sites_per_tree)):
            site_pos.append(pos)
            mut_site.append(len(site_pos) - 1)
            mut_node.append(int(rng.choice(tree_nodes)))
    return Tables.from_columns(ntrees, np.array(node_time), np.array(flags, dtype=np.uint32),
                               left, right, parent, child, site_position=site_pos,
                               mutation_site=mut_site, mutation_node=mut_node)


def _terms(K):
    terms = [(O.DIVERSITY, (k,)) for k in range(K)]
    terms += [(O.SEGSITES, (k,)) for k in range(K)]
    terms += [(O.DIVERGENCE, (i, j)) for i in range(K) for j in range(i + 1, K)]
    terms += [(O.Y3, (0, 1, 2)), (O.F4, (0, 1, 2, 3))]
    return terms


def _run(ts, sets, terms, windows, precision, sweep, polarised=False):
    import torch
    import tskit_gb300

    q = ts.query(sets, terms, windows=windows, both_modes=True, polarised=polarised,
                 precision=precision, sweep=sweep)
    ws = tskit_gb300.Workspace()
    res = torch.zeros(q.result_size, dtype=torch.float64, device="cuda")
    q.launch(ws, res)
    torch.cuda.synchronize()
    q.check(ws)
    return res.cpu().numpy().reshape(2, len(windows) - 1, len(terms))


def _check(got, ots, sets, terms, windows, precision, polarised=False):
    for m, mode in enumerate(["branch", "site"]):
        exp = O.sample_count_stat(ots, sets, terms, windows=windows, mode=mode,
                                  polarised=polarised)
        rtol = RTOL_F64 if (precision == "f64" or mode == "site") else RTOL_F32
        scale = np.maximum(np.abs(exp), np.abs(exp).max(axis=0, keepdims=True) * 1e-2)
        err = np.abs(got[m] - exp) / scale
        assert np.nanmax(err) < rtol, (mode, precision, np.nanmax(err))


@pytest.fixture(scope="module")
def reshuffled(cuda_lib):
    tables = reshuffled_tables(600, 9, 40, 5)
    return tables, O.OracleTS(tables)


@pytest.mark.parametrize("precision,sweep", [("f64", "auto"), ("f32", "auto"),
                                             ("f64", "global_state"), ("f32", "global_state")])
@pytest.mark.parametrize("polarised", [False, True])
def test_whole_tree_transitions(reshuffled, precision, sweep, polarised):
    import tskit_gb300

    tables, ots = reshuffled
    rng = np.random.default_rng(1)
    perm = rng.permutation(tables.samples())
    sets = [np.sort(p) for p in np.array_split(perm, 4)]
    terms = _terms(4)
    windows = np.array([0, 0.5, 1.0, 2.25, 4.0, 4.5, 7.0, 9.0])
    ts = tskit_gb300.TreeSequence(tables)
    got = _run(ts, sets, terms, windows, precision, sweep, polarised)
    _check(got, ots, sets, terms, windows, precision, polarised)


@pytest.mark.parametrize("num_spans", [1, 2, 3, 5, 9])
def test_span_counts_agree(reshuffled, num_spans):
    """One span or one per tree: the same values (FP64, to rounding)."""
    import tskit_gb300

    tables, ots = reshuffled
    rng = np.random.default_rng(2)
    perm = rng.permutation(tables.samples())
    sets = [np.sort(p) for p in np.array_split(perm, 4)]
    terms = _terms(4)
    windows = np.linspace(0, 9, 7)
    ts = tskit_gb300.TreeSequence(tables, num_spans)
    # span boundaries split the edge events evenly, so a request can merge
    assert 1 <= ts.num_spans <= num_spans
    got = _run(ts, sets, terms, windows, "f64", "auto")
    _check(got, ots, sets, terms, windows, "f64")


def test_span_counts_medium(cuda_lib):
    """A seeded SMC tree sequence under several span counts, against the
    oracle and against each other."""
    import tskit_gb300
    from tskit_gb300 import sim

    tables = sim.simulate(300, 1e6, 2000, 4000, 17)
    ots = O.OracleTS(tables)
    rng = np.random.default_rng(3)
    perm = rng.permutation(tables.samples())
    sets = [np.sort(p) for p in np.array_split(perm, 4)]
    terms = _terms(4)
    windows = np.linspace(0, tables.sequence_length, 23)
    base = None
    for ns in (1, 7, 64, 0):
        ts = tskit_gb300.TreeSequence(tables, ns)
        got = _run(ts, sets, terms, windows, "f64", "auto")
        _check(got, ots, sets, terms, windows, "f64")
        if base is None:
            base = got
        np.testing.assert_allclose(got, base, rtol=1e-12, atol=1e-12)
