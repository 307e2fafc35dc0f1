"""Batched launches across resident tree sequences (tsg_batch_*): prepared
queries on tree sequences of uneven size -- sample-count statistics in both
modes, both arithmetics, polarised or not, 1 to 8 sample sets, different
windows, an allele frequency spectrum and a relatedness-vector product --
run as one launch per pipeline stage, and every result equals the result of
the query's own launch bit for bit.  The oracle pins the fused results."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

SEQS = [
    # n, L, breakpoints, sites, seed
    (40, 1e5, 150, 300, 31),
    (700, 1e6, 3000, 4000, 32),
    (3000, 1e7, 8000, 9000, 33),
    (250, 5e5, 900, 1500, 34),
]


@pytest.fixture(scope="module")
def resident(cuda_lib):
    import tskit_gb300
    from tskit_gb300 import sim

    out = []
    for n, L, b, s, seed in SEQS:
        tables = sim.simulate(n, L, b, s, seed)
        out.append((tskit_gb300.TreeSequence(tables), tables))
    return out


def _queries(resident):
    """(query, description) pairs: several per tree sequence."""
    from tskit_gb300 import _native as nat
    from tskit_gb300.trees import AfsQuery, RelatednessVectorQuery

    qs = []
    for i, (ts, tables) in enumerate(resident):
        rng = np.random.default_rng(100 + i)
        samples = tables.samples()
        L = tables.sequence_length
        for j, (k, nwin, prec, pol, both) in enumerate([
                (1, 1, "f64", False, True), (4, 7, "f64", True, True),
                (8, 13, "f32", False, False), (3, 1, "f32", True, True),
                (6, 40, "f64", False, False)]):
            perm = rng.permutation(samples)
            sets = [np.sort(p) for p in np.array_split(perm[: max(k, len(perm) * 3 // 4)], k)]
            terms = [(O.DIVERSITY, (a,)) for a in range(k)] + [(O.SEGSITES, (0,))]
            if k > 1:
                terms += [(O.DIVERGENCE, (0, k - 1)), (O.F2, (0, k - 1))]
            if k > 2:
                terms += [(O.Y3, (0, 1, 2)), (O.F3, (2, 0, 1))]
            windows = None if nwin == 1 else np.sort(np.concatenate(
                [[0, L], rng.uniform(0, L, nwin - 1)]))
            mode = ("branch", "site")[j % 2]
            sn = bool(j % 2)
            q = ts.query(sets, terms, windows=windows, both_modes=both, mode=mode,
                         span_normalise=sn, precision=prec, polarised=pol)
            qs.append((q, dict(ts=i, kind="counts", nwin=nwin, prec=prec, pol=pol, both=both,
                               mode=mode, sets=sets, terms=terms, windows=windows, sn=sn)))
        afs_sets = [np.sort(rng.permutation(samples)[: min(30, len(samples))])]
        qs.append((AfsQuery(ts, afs_sets, None, None, nat.STAT_SITE | nat.STAT_SPAN_NORMALISE),
                   dict(ts=i, kind="afs")))
    return qs


def _own(q):
    import torch

    import tskit_gb300

    ws = tskit_gb300.Workspace(q.workspace_bytes)
    res = torch.full((q.result_size,), -7.0, dtype=torch.float64, device="cuda")
    q.launch(ws, res)
    torch.cuda.synchronize()
    q.check(ws)
    return res.cpu().numpy()


def _bits(a):
    return np.asarray(a, dtype=np.float64).view(np.int64)


def test_batch_equals_own_launches(resident):
    import torch

    import tskit_gb300
    from tskit_gb300 import _native as nat
    from tskit_gb300.trees import RelatednessVectorQuery

    qs = _queries(resident)
    # a relatedness-vector product (runs on its own inside the batch)
    ts0 = resident[1][0]
    rv = RelatednessVectorQuery(ts0, 3, None, None, nat.STAT_BRANCH)
    W = torch.from_numpy(np.random.default_rng(5).normal(size=(ts0.num_samples, 3))).cuda()
    rv.set_weights(W)
    qs.append((rv, dict(ts=1, kind="rv")))
    own = [_own(q) for q, _ in qs]
    ws = tskit_gb300.Workspace()
    results = [torch.full((q.result_size,), -7.0, dtype=torch.float64, device="cuda")
               for q, _ in qs]
    batch = tskit_gb300.QueryBatch([q for q, _ in qs], results, ws)
    # sample-count queries on tree sequences with a compact plan are fused
    fused = sum(1 for _, d in qs if d["kind"] == "counts"
                and resident[d["ts"]][0].num_compact_spans > 0)
    assert fused >= 10 and batch.num_fused == fused
    for rep in range(2):
        for r in results:
            r.fill_(-7.0)
        batch.launch()
        torch.cuda.synchronize()
        batch.check()
        for (q, d), mine, r in zip(qs, own, results):
            np.testing.assert_array_equal(_bits(r.cpu().numpy()), _bits(mine),
                                          err_msg=str({k: v for k, v in d.items()
                                                       if k not in ("sets", "terms", "windows")}))


def test_batch_matches_oracle(resident):
    import torch

    import tskit_gb300

    qs = [(q, d) for q, d in _queries(resident) if d["kind"] == "counts" and d["prec"] == "f64"]
    ws = tskit_gb300.Workspace()
    results = [torch.zeros(q.result_size, dtype=torch.float64, device="cuda") for q, _ in qs]
    batch = tskit_gb300.QueryBatch([q for q, _ in qs], results, ws)
    batch.launch()
    torch.cuda.synchronize()
    batch.check()
    for (q, d), r in zip(qs, results):
        ots = O.OracleTS(resident[d["ts"]][1])
        got = r.cpu().numpy().reshape((2 if d["both"] else 1), d["nwin"], len(d["terms"]))
        modes = ("branch", "site") if d["both"] else (d["mode"],)
        for m, md in enumerate(modes):
            exp = O.sample_count_stat(ots, d["sets"], d["terms"], windows=d["windows"], mode=md,
                                      polarised=d["pol"], span_normalise=d["sn"])
            scale = np.max(np.abs(exp), axis=0)
            np.testing.assert_allclose(got[m], exp, rtol=1e-12,
                                       atol=1e-12 * max(1.0, float(np.max(scale))))


def test_batch_in_cuda_graph(resident):
    """A batch of fused queries replays from a captured CUDA graph with the
    same results."""
    import torch

    import tskit_gb300

    qs = [q for q, d in _queries(resident) if d["kind"] == "counts"
          and resident[d["ts"]][0].num_compact_spans > 0]
    own = [_own(q) for q in qs]
    ws = tskit_gb300.Workspace()
    results = [torch.zeros(q.result_size, dtype=torch.float64, device="cuda") for q in qs]
    batch = tskit_gb300.QueryBatch(qs, results, ws)
    assert batch.num_fused == len(qs)
    st = torch.cuda.Stream()
    with torch.cuda.stream(st):
        batch.launch(st)  # warm-up outside the capture
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=st):
        batch.launch(st)
    for r in results:
        r.zero_()
    g.replay()
    torch.cuda.synchronize()
    batch.check()
    for mine, r in zip(own, results):
        np.testing.assert_array_equal(_bits(r.cpu().numpy()), _bits(mine))


def test_query_launch_in_cuda_graph(resident):
    """A single query's launch -- its independent stages forked onto the
    workspace's side streams and joined by events -- replays from a captured
    CUDA graph with the eager launch's results."""
    import torch

    import tskit_gb300

    qs = [(q, d) for q, d in _queries(resident) if d["kind"] == "counts"
          and resident[d["ts"]][0].num_compact_spans > 0 and d["both"]][:3]
    assert qs
    st = torch.cuda.Stream()
    for q, _ in qs:
        ws = tskit_gb300.Workspace(q.workspace_bytes)
        eager = _own(q)
        res = torch.zeros(q.result_size, dtype=torch.float64, device="cuda")
        with torch.cuda.stream(st):
            q.launch(ws, res, st)  # warm-up outside the capture
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=st):
            q.launch(ws, res, st)
        res.zero_()
        g.replay()
        g.replay()
        torch.cuda.synchronize()
        q.check(ws)
        np.testing.assert_array_equal(_bits(res.cpu().numpy()), _bits(eager))
