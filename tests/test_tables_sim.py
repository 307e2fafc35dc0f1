"""Host-side tables, indexes, allele codes and the synthetic generator."""
import numpy as np

from tskit_gb300 import sim
from tskit_gb300.tables import Tables
from golden_cases import load, manifest


def test_generator_is_deterministic():
    a = sim.simulate(30, 1e5, 50, 200, 7)
    b = sim.simulate(30, 1e5, 50, 200, 7)
    for k, v in a.to_dict().items():
        if isinstance(v, np.ndarray):
            np.testing.assert_array_equal(v, getattr(b, k))


def test_generator_output_is_valid_and_binary():
    t = sim.simulate(50, 1e6, 200, 1000, 3)
    t.check()
    assert t.num_nodes == 50 + 49 + 200
    # every node but the samples is a parent; edges sorted by parent time
    tp = t.node_time[t.edge_parent]
    assert np.all(np.diff(tp) >= 0)
    assert np.all(t.node_time[t.edge_parent] > t.node_time[t.edge_child])
    # one biallelic mutation per site
    assert t.num_mutations == t.num_sites
    allele, alt, nall = t.allele_codes()
    assert np.all(allele == 1) and np.all(alt == 0) and np.all(nall == 2)


def test_index_matches_reference_fixtures():
    """Our index build equals the reference's on every golden fixture."""
    for name in manifest():
        tables, _ = load(name)
        ins, rem = tables.edge_insertion_order.copy(), tables.edge_removal_order.copy()
        tables.build_index()
        np.testing.assert_array_equal(ins, tables.edge_insertion_order)
        np.testing.assert_array_equal(rem, tables.edge_removal_order)


def test_allele_codes_back_mutation():
    """single_tree_ex has a back mutation and recurrent mutations
    (c/tests/testlib.c); codes follow get_allele_weights' numbering."""
    tables, _ = load("single_tree_ex")
    allele, alt, nall = tables.allele_codes()
    # site 1: mutation to "1" then a back mutation (derived "0") with parent
    ms = tables.mutation_site
    s1 = np.flatnonzero(ms == 1)
    assert list(allele[s1]) == [1, 0]
    assert list(alt[s1]) == [0, 1]
    s2 = np.flatnonzero(ms == 2)
    assert list(allele[s2]) == [1, 1, 1, 1]
    assert nall[1] == 2 and nall[2] == 2
