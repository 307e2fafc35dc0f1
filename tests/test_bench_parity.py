"""The full-size parity checker of the relatedness-matrix benchmark
(bench.grm_parity) on the CPU, at a size the whole-matrix oracle handles:
given a correct operand, Gram (entries below the diagonal band garbage, as
the kernel leaves them) and relatedness matrix it passes; a wrong Gram
entry, operand byte or relatedness entry makes it fail."""
import os
import sys

import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")
sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


@pytest.fixture(scope="module")
def case():
    from tskit_gb300 import sim

    t = sim.simulate(2048, 1e6, 300, 3000, 5)
    ots = O.OracleTS(t)
    n, S = 2048, t.num_sites
    kp = (S + 127) // 128 * 128
    geno = O.genotype_matrix(ots)
    G = torch.zeros((n, kp), dtype=torch.uint8)
    G[:, :S] = torch.from_numpy((geno.T != 0).astype(np.uint8) * 0x38)
    # the exact integer product through FP64 BLAS (exact below 2^53), and the
    # biallelic identity: differing sites = a_i + a_j - 2 G_ij
    X = (geno.T != 0).astype(np.float64)
    full = np.rint(X @ X.T).astype(np.int64)
    a = np.diag(full)
    D = (a[:, None] + a[None, :] - 2 * full) / t.sequence_length
    r = np.arange(n)[:, None] // 256
    c = np.arange(n)[None, :] // 256
    P = torch.from_numpy(np.where(c >= r, full, -7).astype(np.int32))
    K = O.relatedness_from_divergence(D)
    return ots, G, P, K, n, S, kp


def test_parity_passes_on_correct_results(case):
    ots, G, P, K, n, S, kp = case
    out = bench.grm_parity(O, ots, G, P, K, n, S, kp)
    assert out["pass"], out
    assert out["tiles"]["mismatches"] == 0 and out["rows"]["product_mismatches"] == 0
    assert out["rows"]["relatedness_max_rel_err"] < 1e-13


def test_parity_catches_errors(case):
    ots, G, P, K, n, S, kp = case
    out = bench.grm_parity(O, ots, G, P, K, n, S, kp)
    rows = out["rows"]["samples"]
    # a wrong product entry in a checked row (the upper part the kernel writes)
    P2 = P.clone()
    i = rows[0]
    P2[i, n - 1] += 1
    assert not bench.grm_parity(O, ots, G, P2, K, n, S, kp)["pass"]
    # a stray operand byte
    G2 = G.clone()
    G2[3, 5] = 0x40
    assert not bench.grm_parity(O, ots, G2, P, K, n, S, kp)["pass"]
    # a relatedness entry off by far more than the bound
    K2 = K.copy()
    K2[rows[1], 7] += 1e-6 * np.max(np.abs(K))
    assert not bench.grm_parity(O, ots, G, P, K2, n, S, kp)["pass"]
