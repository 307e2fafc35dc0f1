"""The C oracle against the reference's golden outputs (CPU only).

Pins the oracle: every fixture of the reference's C test library
(c/tests/testlib.c) and the seeded SMC fixtures, for every statistics call in
tests/golden/cases.json, must match the reference's output.  Genotypes are
compared exactly, floating point at 1e-12 relative.
"""
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
