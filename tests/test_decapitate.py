"""The topology of decapitate (used by pca's time windows) against the
reference's own decapitate (tests/golden/make_pca_golden.py).  Host code
only."""
import os

import numpy as np
import pytest

from tskit_gb300.tables import Tables

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("label", ["mid", "zero"])
def test_decapitated_topology_matches_reference(label, cuda_lib_cpu):
    ref = np.load(os.path.join(GOLDEN, "pca.npz"))
    t = Tables.load(os.path.join(GOLDEN, "weighted_b.trees"))
    time = float(ref["t_mid"]) if label == "mid" else 0.0
    d = t.decapitated_topology(time)
    d.check()
    assert d.num_nodes == int(ref[f"decap_{label}_num_nodes"])
    got = np.column_stack([d.edge_left, d.edge_right, d.edge_child,
                           d.node_time[d.edge_parent]])
    exp = ref[f"decap_{label}_edges"]
    key = lambda a: a[np.lexsort(a.T[::-1])]  # noqa: E731
    np.testing.assert_array_equal(key(got), key(exp))
    assert np.all(d.node_time[d.edge_parent] <= time)
