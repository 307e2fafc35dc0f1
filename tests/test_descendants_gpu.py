"""mean_descendants against the reference's own values
(tests/golden/make_descendants_golden.py): reference sets of samples, of
internal nodes and of arbitrary nodes, on tree sequences the reference
wrote (one with internal samples)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FILES = {"a": "weighted_a.trees", "b": "weighted_b.trees", "internal": "node_internal.trees"}


@pytest.mark.parametrize("name", sorted(FILES))
def test_mean_descendants_matches_reference(name, cuda_lib):
    import tskit_gb300

    ts = tskit_gb300.load(os.path.join(GOLDEN, FILES[name]))
    ref = np.load(os.path.join(GOLDEN, f"descendants_{name}.npz"))
    sets = np.split(ref["flat"], np.cumsum(ref["sizes"])[:-1])
    got = ts.mean_descendants([list(x) for x in sets])
    np.testing.assert_allclose(got, ref["result"], rtol=1e-12, atol=1e-13)


def test_mean_descendants_errors(cuda_lib):
    import tskit_gb300
    from tskit_gb300 import LibraryError
    from tskit_gb300 import _native as nat

    ts = tskit_gb300.load(os.path.join(GOLDEN, "weighted_a.trees"))
    with pytest.raises(LibraryError) as e:
        ts.mean_descendants([[ts.num_nodes]])
    assert e.value.code == nat.ERR_NODE_OUT_OF_BOUNDS
    with pytest.raises(LibraryError) as e:
        ts.mean_descendants([])
    assert e.value.code == nat.ERR_BAD_PARAM_VALUE


@pytest.mark.parametrize("name", sorted(FILES))
def test_gnn_matches_reference(name, cuda_lib):
    """genealogical_nearest_neighbours: focal samples and internal nodes,
    reference sets of samples and of internal nodes."""
    import tskit_gb300

    ts = tskit_gb300.load(os.path.join(GOLDEN, FILES[name]))
    ref = np.load(os.path.join(GOLDEN, f"descendants_{name}.npz"))
    sets = np.split(ref["gnn_flat"], np.cumsum(ref["gnn_sizes"])[:-1])
    got = ts.genealogical_nearest_neighbours(ref["gnn_focal"], [list(x) for x in sets])
    np.testing.assert_allclose(got, ref["gnn_result"], rtol=1e-12, atol=1e-13)


def test_gnn_errors(cuda_lib):
    import tskit_gb300
    from tskit_gb300 import LibraryError
    from tskit_gb300 import _native as nat

    ts = tskit_gb300.load(os.path.join(GOLDEN, "weighted_a.trees"))
    s = list(ts.samples())
    with pytest.raises(LibraryError) as e:
        ts.genealogical_nearest_neighbours(s, [s[:3], s[2:5]])
    assert e.value.code == nat.ERR_DUPLICATE_SAMPLE
    with pytest.raises(LibraryError) as e:
        ts.genealogical_nearest_neighbours([ts.num_nodes], [s])
    assert e.value.code == nat.ERR_NODE_OUT_OF_BOUNDS
    assert ts.genealogical_nearest_neighbours([], [s]).shape == (0, 1)
