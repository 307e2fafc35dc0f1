"""genetic_relatedness_weighted against the reference's own values
(tests/golden/make_relatedness_weighted_golden.py) on tree sequences the
reference wrote: both modes, polarised or not, centred or not, default and
explicit index pairs, a single pair (dimension dropped), no windows, and
unnormalised spans; then the reference's argument errors."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = {
    "two": (None, True, True),
    "pairs": ([(0, 1), (1, 2), (2, 2), (0, 0), (2, 0)], True, True),
    "single": ([0, 2], True, False),
    "nowin": ([(3, 1), (0, 3)], False, True),
}


@pytest.mark.parametrize("name", ["a", "b"])
@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("mode", ["site", "branch"])
@pytest.mark.parametrize("polarised", [False, True])
@pytest.mark.parametrize("centre", [True, False])
def test_matches_reference(name, case, mode, polarised, centre, cuda_lib):
    import tskit_gb300

    ts = tskit_gb300.load(os.path.join(GOLDEN, f"weighted_{name}.trees"))
    ref = np.load(os.path.join(GOLDEN, f"relatedness_weighted_{name}.npz"))
    indexes, with_win, span_norm = CASES[case]
    got = ts.genetic_relatedness_weighted(
        ref[f"W_{case}"], indexes=indexes, windows=ref["windows"] if with_win else None,
        mode=mode, span_normalise=span_norm, polarised=polarised, centre=centre)
    exp = ref[f"{case}_{mode}_{int(polarised)}_{int(centre)}"]
    assert got.shape == exp.shape
    scale = np.max(np.abs(exp)) if exp.size else 1.0
    np.testing.assert_allclose(got, exp, rtol=1e-10, atol=1e-11 * scale)


def test_argument_errors(cuda_lib):
    import tskit_gb300
    from tskit_gb300 import LibraryError
    from tskit_gb300 import _native as nat

    ts = tskit_gb300.load(os.path.join(GOLDEN, "weighted_a.trees"))
    n = ts.num_samples
    W3 = np.ones((n, 3))
    with pytest.raises(ValueError):
        ts.genetic_relatedness_weighted(np.ones((n - 1, 2)))
    with pytest.raises(ValueError):
        ts.genetic_relatedness_weighted(W3)  # indexes needed unless 2 columns
    with pytest.raises(ValueError):
        ts.genetic_relatedness_weighted(W3, indexes=[(0, 1, 2)])
    with pytest.raises(LibraryError) as e:
        ts.genetic_relatedness_weighted(np.ones((n, 0)), indexes=[(0, 0)])
    assert e.value.code == nat.ERR_INSUFFICIENT_WEIGHTS
    with pytest.raises(LibraryError) as e:
        ts.genetic_relatedness_weighted(W3, indexes=[(0, 3)])
    assert e.value.code == nat.ERR_BAD_SAMPLE_SET_INDEX
    with pytest.raises(ValueError):
        ts.genetic_relatedness_weighted(W3, indexes=[(0, 1)], mode="nonsense")
