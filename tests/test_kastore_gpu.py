"""Statistics of tree sequences read from .trees files written by the
reference, against the values the reference computes on the same files
(tests/golden/make_trees_files.py); uncalibrated times refuse branch mode
as the reference does (c/tskit/trees.c:1383, 3723)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("name", ["sim_n40", "multiallelic_n30", "uncalibrated_n20"])
def test_stats_of_loaded_files(name, cuda_lib):
    import tskit_gb300
    from tskit_gb300 import _native as nat

    ts = tskit_gb300.load(os.path.join(GOLDEN, name + ".trees"))
    ref = np.load(os.path.join(GOLDEN, name + "_trees.npz"))
    sets = [ref["set0"], ref["set1"]]
    windows = ref["windows"]
    for mode in ("site", "branch"):
        key = f"diversity_{mode}"
        if key not in ref.files:
            with pytest.raises(tskit_gb300.LibraryError) as e:
                ts.diversity(sets, windows=windows, mode=mode)
            assert e.value.code == nat.ERR_TIME_UNCALIBRATED
            with pytest.raises(tskit_gb300.LibraryError):
                ts.allele_frequency_spectrum([sets[0]], windows=windows, mode=mode)
            continue
        np.testing.assert_allclose(ts.diversity(sets, windows=windows, mode=mode), ref[key],
                                   rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(ts.divergence(sets, windows=windows, mode=mode),
                                   ref[f"divergence_{mode}"], rtol=1e-12, atol=1e-14)
