"""TreeSequence.pca against the reference's own results
(tests/golden/make_pca_golden.py): the same range sketches give the same
factors, eigenvalues, final sketches and error bounds, for all samples, a
subset, windows, individuals, time windows and without centring; then the
reference's argument errors."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _cases(ts, ref):
    L = ts.sequence_length
    s = ts.samples()
    t_mid = float(ref["t_mid"])
    t_max = float(np.max(ts.tables.node_time)) + 1.0
    return {
        "default": dict(num_components=3),
        "windows": dict(num_components=4, windows=[0, L / 2, L], centre=False),
        "subset": dict(num_components=3, samples=s[:25], num_iterations=3),
        "individuals": dict(num_components=2, individuals=np.arange(20)),
        "time": dict(num_components=3, time_windows=[0.0, t_mid]),
        "time_high": dict(num_components=2, time_windows=[t_mid, t_max], windows=[0, L / 3, L]),
    }


def _aligned(got, exp):
    """Columns of got with the signs of exp (singular vectors are defined up
    to sign; the same sketch gives the same signs unless nearly degenerate)."""
    sign = np.sign(np.sum(got * exp, axis=-2, keepdims=True))
    return got * np.where(sign == 0, 1, sign)


@pytest.mark.parametrize("case", ["default", "windows", "subset", "individuals", "time",
                                  "time_high"])
def test_pca_matches_reference(case, cuda_lib):
    import tskit_gb300

    ref = np.load(os.path.join(GOLDEN, "pca.npz"))
    name = "pca_individuals.trees" if case == "individuals" else "weighted_b.trees"
    ts = tskit_gb300.load(os.path.join(GOLDEN, name))
    kw = _cases(ts, ref)[case]
    res = ts.pca(range_sketch=ref[f"{case}_sketch"], **kw)
    ev = ref[f"{case}_eigenvalues"]
    np.testing.assert_allclose(res.eigenvalues, ev, rtol=1e-9)
    np.testing.assert_allclose(res.error_bound, ref[f"{case}_error_bound"], rtol=1e-9)
    np.testing.assert_allclose(_aligned(res.factors, ref[f"{case}_factors"]),
                               ref[f"{case}_factors"], atol=1e-7)
    np.testing.assert_allclose(_aligned(res.range_sketch, ref[f"{case}_range_sketch"]),
                               ref[f"{case}_range_sketch"], atol=1e-7)


def test_pca_seed_draws_the_sketch(cuda_lib):
    import tskit_gb300

    ts = tskit_gb300.load(os.path.join(GOLDEN, "weighted_b.trees"))
    a = ts.pca(3, random_seed=17)
    sketch = np.random.default_rng(17).normal(size=(1, ts.num_samples, 13))
    b = ts.pca(3, range_sketch=sketch[0])
    np.testing.assert_array_equal(a.factors, b.factors)
    assert a.factors.shape == (ts.num_samples, 3) and a.eigenvalues.shape == (3,)
    # further power iterations from the returned sketch barely move the result
    c = ts.pca(3, range_sketch=a.range_sketch)
    np.testing.assert_allclose(c.eigenvalues, a.eigenvalues, rtol=1e-3)


def test_pca_errors(cuda_lib):
    import tskit_gb300
    from tskit_gb300 import LibraryError
    from tskit_gb300 import _native as nat

    ts = tskit_gb300.load(os.path.join(GOLDEN, "weighted_b.trees"))
    n = ts.num_samples
    with pytest.raises(ValueError):
        ts.pca(2, num_iterations=0)
    with pytest.raises(ValueError):
        ts.pca(n + 1)
    with pytest.raises(ValueError):
        ts.pca(2, samples=ts.samples(), individuals=[0])
    with pytest.raises(ValueError):
        ts.pca(2, num_oversamples=3, range_sketch=np.zeros((n, 5)))
    with pytest.raises(ValueError):
        ts.pca(4, range_sketch=np.zeros((n, 3)))
    with pytest.raises(ValueError):
        ts.pca(2, range_sketch=np.zeros((n - 1, 5)))
    with pytest.raises(LibraryError) as e:
        ts.pca(2, time_windows=[0, np.inf])
    assert e.value.code == nat.ERR_TIME_NONFINITE
