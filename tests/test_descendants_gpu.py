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
