"""GPU parity of the tensor-core Gram matrix, the site-mode divergence matrix
and the site-mode genetic relatedness matrix.

The Gram matrix of 0/1 operands is exact: it must equal a CPU integer
product bit for bit.  Divergence counts are integers divided by window spans
(identical to the oracle's); the relatedness normalisation is FP64 (1e-12)."""
import ctypes

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _gram(lib, G01):
    """Device Gram of a 0/1 matrix (rows = samples) through tsg_gram_e4m3."""
    import torch

    n, k = G01.shape
    kp = (k + 127) // 128 * 128
    host = np.zeros((n, kp), dtype=np.uint8)
    host[:, :k] = np.where(G01 != 0, 0x38, 0)
    G = torch.from_numpy(host).cuda()
    P = torch.zeros((n, n), dtype=torch.int32, device="cuda")
    err = lib.tsg_gram_e4m3(ctypes.c_void_p(G.data_ptr()), n, kp, kp,
                            ctypes.c_void_p(P.data_ptr()), n,
                            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert err == 0, err
    torch.cuda.synchronize()
    return P.cpu().numpy()


def _upper_tiles_mask(n):
    """Entries the kernel writes: 256 x 256 tiles with row block <= column
    block (every entry of the upper triangle and the diagonal)."""
    m = np.zeros((n, n), dtype=bool)
    for r in range(0, n, 256):
        m[r:r + 256, r:] = True
    assert m[np.triu_indices(n)].all()
    return m


@pytest.mark.parametrize("n,k,p", [(128, 128, 0.5), (300, 1024, 0.3), (777, 128 * 37, 0.05),
                                   (1000, 4096, 0.9), (256, 128 * 300, 0.5), (1100, 512, 0.2)])
def test_gram_exact(cuda_lib, n, k, p):
    rng = np.random.default_rng(n + k)
    G01 = (rng.random((n, k)) < p).astype(np.int64)
    got = _gram(cuda_lib, G01)
    exp = G01 @ G01.T
    m = _upper_tiles_mask(n)
    np.testing.assert_array_equal(got[m], exp[m])


@pytest.fixture(scope="module")
def small(cuda_lib):
    import tskit_gb300
    from tskit_gb300 import sim

    tables = sim.simulate(150, 1e5, 300, 2500, 61)
    return tskit_gb300.TreeSequence(tables), O.OracleTS(tables), tables


def test_divergence_matrix_vs_oracle(small):
    ts, ots, tables = small
    L = tables.sequence_length
    for windows in (None, np.linspace(0, L, 5), [0.2 * L, 0.5 * L, 0.7 * L]):
        for sn in (True, False):
            got = ts.divergence_matrix(windows=windows, span_normalise=sn)
            exp = O.divergence_matrix_site(ots, windows=windows, span_normalise=sn)
            exp = exp.reshape(got.shape)
            np.testing.assert_array_equal(got, exp)


def test_divergence_matrix_sample_sets(small):
    ts, ots, tables = small
    rng = np.random.default_rng(3)
    perm = rng.permutation(tables.samples())
    sets = [np.sort(perm[:10]), np.sort(perm[10:11]), np.sort(perm[11:40])]
    windows = np.linspace(0, tables.sequence_length, 3)
    got = ts.divergence_matrix(sets, windows=windows)
    D = O.divergence_matrix_site(ots, windows=windows)  # per sample, span normalised
    idx = [np.searchsorted(tables.samples(), s) for s in sets]
    exp = np.zeros_like(got)
    for w in range(D.shape[0]):
        for i, a in enumerate(idx):
            for j, b in enumerate(idx):
                tot = D[w][np.ix_(a, b)].sum()
                den = len(a) * (len(a) - 1) if i == j else len(a) * len(b)
                exp[w, i, j] = tot / den if den else tot
    np.testing.assert_allclose(got, exp, rtol=1e-12, atol=0)


def test_genetic_relatedness_matrix_vs_oracle(small):
    ts, ots, tables = small
    windows = np.linspace(0, tables.sequence_length, 4)
    got = ts.genetic_relatedness_matrix(windows=windows)
    D = O.divergence_matrix_site(ots, windows=windows)
    for w in range(D.shape[0]):
        exp = O.relatedness_from_divergence(D[w])
        scale = np.abs(exp).max()
        np.testing.assert_allclose(got[w], exp, rtol=1e-12, atol=1e-12 * scale)


def test_divergence_matrix_multiallelic(cuda_lib):
    """Sites with several derived alleles: the extra indicator rows."""
    import tskit_gb300
    from tskit_gb300 import sim
    from tskit_gb300.tables import Tables

    base = sim.simulate(90, 1e5, 200, 800, 71)
    rng = np.random.default_rng(8)
    # add a second mutation, to a new state, below the first at some sites
    msite, mnode, mparent, mder = [], [], [], []
    for m in range(base.num_mutations):
        s, u = int(base.mutation_site[m]), int(base.mutation_node[m])
        msite.append(s)
        mnode.append(u)
        mparent.append(-1)
        mder.append(b"1")
        if rng.random() < 0.3:
            kids = base.edge_child[(base.edge_parent == u)
                                   & (base.edge_left <= base.site_position[s])
                                   & (base.edge_right > base.site_position[s])]
            if len(kids):
                msite.append(s)
                mnode.append(int(kids[0]))
                mparent.append(len(msite) - 2)
                mder.append(b"2" if rng.random() < 0.7 else b"0")
    anc = [b"0"] * base.num_sites
    tables = Tables.from_columns(base.sequence_length, base.node_time, base.node_flags,
                                 base.edge_left, base.edge_right, base.edge_parent,
                                 base.edge_child, site_position=base.site_position,
                                 site_ancestral_state=anc, mutation_site=msite,
                                 mutation_node=mnode, mutation_parent=mparent,
                                 mutation_derived_state=mder)
    ts = tskit_gb300.TreeSequence(tables)
    ots = O.OracleTS(tables)
    windows = np.linspace(0, tables.sequence_length, 3)
    got = ts.divergence_matrix(windows=windows)
    exp = O.divergence_matrix_site(ots, windows=windows)
    np.testing.assert_array_equal(got, exp)


def test_divergence_matrix_errors(small):
    import tskit_gb300

    ts, _, tables = small
    with pytest.raises(tskit_gb300.LibraryError) as e:
        ts.divergence_matrix(mode="node")
    assert e.value.code == -909
    with pytest.raises(tskit_gb300.LibraryError) as e:
        ts.divergence_matrix([tables.samples()[0], tables.samples()[0]])
    assert e.value.code == -600


def _set_means(D, sets, index):
    """Mean pairwise entries between sets (distinct samples within a set),
    as fill_lower_triangle_count_normalise (trees.c:8876-8899)."""
    K = len(sets)
    out = np.zeros((D.shape[0], K, K))
    for a in range(K):
        for b in range(K):
            ia, ib = index[sets[a]], index[sets[b]]
            block = D[:, ia][:, :, ib]
            if a == b:
                denom = len(ia) * (len(ia) - 1)
                out[:, a, b] = block.sum(axis=(1, 2)) / denom if denom else block.sum(axis=(1, 2))
            else:
                out[:, a, b] = block.sum(axis=(1, 2)) / (len(ia) * len(ib))
    return out


def test_branch_divergence_matrix_sets_partial_windows(small):
    """Branch mode through the relatedness sweep: sample sets of several
    samples and windows that leave parts of the sequence out, against the
    oracle's per-tree path lengths (FP64 within 1e-12 of the scale)."""
    ts, ots, tables = small
    L = tables.sequence_length
    s = tables.samples()
    rng = np.random.default_rng(5)
    perm = rng.permutation(s)
    sets = [np.sort(perm[:7]), np.sort(perm[7:8]), np.sort(perm[8:40]), np.sort(perm[40:41])]
    windows = [L / 5, L / 3, 0.7 * L]
    got = ts.divergence_matrix(sets, windows=windows, mode="branch")
    D = O.divergence_matrix_branch(ots, windows=windows)
    index = np.full(tables.num_nodes, -1)
    index[s] = np.arange(len(s))
    exp = _set_means(D, sets, index)
    np.testing.assert_allclose(got, exp, rtol=1e-12, atol=1e-12 * np.max(np.abs(exp)))
    # every sample alone, the whole sequence, not normalised by span
    got = ts.divergence_matrix(mode="branch", span_normalise=False)
    exp = O.divergence_matrix_branch(ots, span_normalise=False)[0]
    np.testing.assert_allclose(got, exp, rtol=1e-12, atol=1e-12 * np.max(np.abs(exp)))
    assert np.all(np.diag(got) == 0)
