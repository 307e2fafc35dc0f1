"""general_stat with real-valued weights against the reference's own values
(tests/golden/make_weighted_golden.py) on tree sequences the reference wrote,
for both modes, polarised or not, several summary functions and windows."""
import os

import numpy as np
import pytest

from weighted_summaries import SUMMARIES

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("name", ["a", "b"])
@pytest.mark.parametrize("fname", sorted(SUMMARIES))
@pytest.mark.parametrize("mode", ["site", "branch"])
@pytest.mark.parametrize("polarised", [False, True])
def test_general_stat_real_weights(name, fname, mode, polarised, cuda_lib):
    import tskit_gb300

    ts = tskit_gb300.load(os.path.join(GOLDEN, f"weighted_{name}.trees"))
    ref = np.load(os.path.join(GOLDEN, f"weighted_{name}.npz"))
    K, M, f = SUMMARIES[fname]
    got = ts.general_stat(ref[f"W{K}"], f, M, windows=ref["windows"], mode=mode,
                          polarised=polarised, strict=False)
    exp = ref[f"{fname}_{mode}_{int(polarised)}"]
    scale = np.max(np.abs(exp)) if exp.size else 1.0
    np.testing.assert_allclose(got, exp, rtol=1e-11, atol=1e-12 * scale)
