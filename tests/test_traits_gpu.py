"""trait_covariance, trait_correlation and trait_linear_model (with and
without covariates) against the reference's own values
(tests/golden/make_trait_golden.py) in site, branch and node mode, with and
without windows, on tree sequences the reference wrote (one with internal
samples)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FILES = {"a": "weighted_a.trees", "b": "weighted_b.trees", "internal": "node_internal.trees"}


def _check(got, exp):
    got = np.asarray(got)
    assert got.shape == np.shape(exp)
    scale = np.max(np.abs(exp)) if np.size(exp) else 1.0
    np.testing.assert_allclose(got, exp, rtol=1e-10, atol=1e-12 * scale)


@pytest.mark.parametrize("name", sorted(FILES))
@pytest.mark.parametrize("stat", ["cov", "cor", "lm", "lmz"])
@pytest.mark.parametrize("mode", ["site", "branch", "node"])
@pytest.mark.parametrize("windowed", ["w", "n"])
def test_traits_match_reference(name, stat, mode, windowed, cuda_lib):
    import tskit_gb300

    ts = tskit_gb300.load(os.path.join(GOLDEN, FILES[name]))
    ref = np.load(os.path.join(GOLDEN, f"traits_{name}.npz"))
    W, Z = ref["W"], ref["Z"]
    win = ref["windows"] if windowed == "w" else None
    if stat == "cov":
        got = ts.trait_covariance(W, windows=win, mode=mode)
    elif stat == "cor":
        got = ts.trait_correlation(W, windows=win, mode=mode)
    elif stat == "lm":
        got = ts.trait_linear_model(W, windows=win, mode=mode)
    else:
        got = ts.trait_linear_model(W, Z, windows=win, mode=mode)
    _check(got, ref[f"{stat}_{mode}_{windowed}"])


def test_trait_arguments(cuda_lib):
    import tskit_gb300

    ts = tskit_gb300.load(os.path.join(GOLDEN, "weighted_a.trees"))
    ref = np.load(os.path.join(GOLDEN, "traits_a.npz"))
    W = ref["W"]
    _check(ts.trait_covariance(W, windows=ref["windows"], span_normalise=False),
           ref["cov_site_unnorm"])
    with pytest.raises(ValueError):
        ts.trait_covariance(W[:-1])
    with pytest.raises(ValueError):
        ts.trait_correlation(np.ones_like(W))
    with pytest.raises(ValueError):
        ts.trait_linear_model(W, np.ones((ts.num_samples, 2)))
    with pytest.warns(FutureWarning):
        got = ts.trait_regression(W, windows=ref["windows"])
    _check(got, ref["lm_site_w"])
