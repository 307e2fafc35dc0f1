"""The C oracle against the reference's golden outputs (CPU only).

Pins the oracle: every fixture of the reference's C test library
(c/tests/testlib.c) and the seeded SMC fixtures, for every statistics call in
tests/golden/cases.json, must match the reference's output.  Genotypes are
compared exactly, floating point at 1e-12 relative.
"""
import os

import numpy as np
import pytest

import oracle as O
from golden_cases import all_cases, load, resolve

CASES = all_cases()
_cache = {}


def ots_for(name):
    if name not in _cache:
        tables, data = load(name)
        _cache[name] = (O.OracleTS(tables), data)
    return _cache[name]


@pytest.mark.parametrize("name,case", CASES, ids=[f"{n}-{c['key']}-{c['method']}" for n, c in CASES])
def test_oracle_matches_reference(name, case):
    ots, data = ots_for(name)
    expected = data[case["key"]]
    got = O.call(ots, case["method"], resolve(case["kwargs"], data))
    got = np.asarray(got).reshape(expected.shape)
    if case["method"] == "genotype_matrix":
        np.testing.assert_array_equal(got, expected)
    else:
        np.testing.assert_allclose(got, expected, rtol=1e-12, atol=1e-13, equal_nan=True)


def test_paper_ex_known_answers():
    """Hand-derived values asserted by the reference's C tests
    (c/tests/test_stats.c:1718-1742): site diversity of paper_ex, not span
    normalised, is 1.5 and a
    sample set of size one gives NaN."""
    ots, _ = ots_for("paper_ex")
    pi = O.one_way(ots, O.DIVERSITY, [[0, 1, 2, 3]], mode="site", span_normalise=False)
    assert abs(pi[0, 0] - 1.5) < 1e-12
    pi1 = O.one_way(ots, O.DIVERSITY, [[0]], mode="site", span_normalise=False)
    assert np.isnan(pi1[0, 0])


@pytest.mark.parametrize("mode", ["site", "branch"])
def test_oracle_afs_parentless_stretches_vs_reference(mode):
    """The reference credits a child that regains a parent from its last
    update (c/tskit/trees.c:3639-3800); the oracle follows it on inputs with
    isolated leaves and temporary extra roots."""
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "oracle"))
    import ref_import

    if not ref_import.available():
        pytest.skip("reference not built here")
    tskit = ref_import.import_tskit()
    from tskit_gb300 import sim
    from ts_gaps import with_gaps

    g = with_gaps(sim.simulate(40, 1e5, 150, 500, 6), 2, frac=0.25)
    tc = tskit.TableCollection(g.sequence_length)
    for t, f in zip(g.node_time, g.node_flags):
        tc.nodes.add_row(flags=int(f), time=float(t))
    for l, r, p, c in zip(g.edge_left, g.edge_right, g.edge_parent, g.edge_child):
        tc.edges.add_row(l, r, p, c)
    for x in g.site_position:
        tc.sites.add_row(x, "0")
    for s, n in zip(g.mutation_site, g.mutation_node):
        tc.mutations.add_row(site=int(s), node=int(n), derived_state="1")
    tc.sort()
    tc.build_index()
    tc.compute_mutation_parents()
    ref = tc.tree_sequence()
    ots = O.OracleTS(g)
    rng = np.random.default_rng(0)
    perm = rng.permutation(g.samples())
    for sets in ([g.samples()], [np.sort(perm[:15]), np.sort(perm[15:])]):
        for pol in (False, True):
            kw = dict(windows=[0, 3e4, 7e4, 1e5], mode=mode, polarised=pol)
            a = ref.allele_frequency_spectrum([list(s) for s in sets], **kw)
            b = O.allele_frequency_spectrum(ots, sets, **kw).reshape(a.shape)
            np.testing.assert_allclose(b, a, rtol=1e-12, atol=1e-15)


_DD_METHODS = {"diversity", "segregating_sites", "Y1", "divergence", "Y2", "f2", "Y3", "f3",
               "f4"}
DD_CASES = [(n, c) for n, c in CASES
            if c["method"] in _DD_METHODS and c["kwargs"].get("mode") == "branch"]


@pytest.mark.parametrize("name,case", DD_CASES,
                         ids=[f"{n}-{c['key']}-{c['method']}" for n, c in DD_CASES])
def test_compensated_branch_oracle_matches_reference(name, case):
    """The double-double restatement of the branch sweep (the attribution
    oracle) agrees with the reference's FP64 values on every branch-mode
    sample-count golden case."""
    ots, data = ots_for(name)
    expected = data[case["key"]]
    kw = resolve(case["kwargs"], data)
    method = case["method"]
    sets = O._sets(ots, kw.get("sample_sets"))
    if method in O._ONE_WAY:
        outs = [(O._ONE_WAY[method], (k,)) for k in range(len(sets))]
    else:
        typ, k = O._K_WAY[method]
        outs = [(typ, tuple(t)) for t in O._tuples(kw.get("indexes"), k, len(sets))]
    if any(len(s) >= 1 << 15 for s in sets):
        pytest.skip("set too large for the integer numerators")
    got = O.branch_count_stat_dd(ots, sets, outs, windows=kw.get("windows"),
                                 span_normalise=kw.get("span_normalise", True))
    got = np.asarray(got).reshape(expected.shape)
    np.testing.assert_allclose(got, expected, rtol=1e-12, atol=1e-13, equal_nan=True)


def test_compensated_branch_oracle_vs_fp64_large():
    """On a seeded tree sequence with thousands of trees the FP64 sweep and the
    double-double sweep agree to well below 1e-12 normwise (the FP64 form's
    running-sum drift is the difference)."""
    from tskit_gb300 import sim

    t = sim.simulate(200, 1e6, 3000, 5000, 17)
    ots = O.OracleTS(t)
    rng = np.random.default_rng(2)
    perm = rng.permutation(t.samples())
    sets = [np.sort(p) for p in np.array_split(perm, 4)]
    terms = [(O.DIVERSITY, (0,)), (O.SEGSITES, (1,)), (O.DIVERGENCE, (0, 1)),
             (O.Y3, (0, 1, 2)), (O.F4, (0, 1, 2, 3)), (O.F2, (2, 3)), (O.Y2, (1, 3)),
             (O.Y1, (3,)), (O.F3, (0, 2, 3)), (O.RELATEDNESS_NC, (0, 3))]
    win = np.linspace(0, t.sequence_length, 41)
    for pol in (False, True):
        a = O.sample_count_stat(ots, sets, terms, windows=win, mode="branch", polarised=pol)
        b = O.branch_count_stat_dd(ots, sets, terms, windows=win, polarised=pol)
        err = np.max(np.abs(a - b), axis=0) / np.max(np.abs(b), axis=0)
        assert np.all(err < 1e-13), err


def test_site_range_oracles_vs_full_matrix():
    """The site-range genotype decode and the reference's pairwise site
    divergence loop agree with the whole-matrix oracle, and the exact
    full-size relatedness rows (path sums) equal the normalised divergence
    matrix's rows."""
    from tskit_gb300 import sim

    t = sim.simulate(150, 1e6, 400, 900, 23)
    ots = O.OracleTS(t)
    G = O.genotype_matrix(ots)
    S = t.num_sites
    np.testing.assert_array_equal(O.genotype_rows(ots, 100, 300), G[100:300])
    assert O.genotype_rows(ots, 5, 5).shape == (0, ots.num_samples)
    full = O.divergence_matrix_site(ots, span_normalise=False)[0]
    np.testing.assert_array_equal(O.divergence_counts_site_range(ots, 0, S), full)
    part = O.divergence_counts_site_range(ots, 0, 300) + O.divergence_counts_site_range(ots, 300, S)
    np.testing.assert_array_equal(part, full)
    # path sums: derived counts and shared-derived counts, exactly
    rows = [0, 7, 149, 60]
    Gi = G.astype(np.int64)
    sums = O.site_path_sums(ots, [ots.samples] + [[ots.samples[i]] for i in rows])
    np.testing.assert_array_equal(sums[:, 0], Gi.sum(axis=0))
    np.testing.assert_array_equal(sums[:, 1], Gi.T @ Gi.sum(axis=1))
    np.testing.assert_array_equal(sums[:, 2:].T, (Gi.T @ Gi)[rows])
    K, shared = O.relatedness_rows_site(ots, rows)
    exp = O.relatedness_from_divergence(O.divergence_matrix_site(ots)[0])[rows]
    np.testing.assert_array_equal(shared, (Gi.T @ Gi)[rows])
    assert np.max(np.abs(K - exp)) <= 1e-13 * np.max(np.abs(exp))
