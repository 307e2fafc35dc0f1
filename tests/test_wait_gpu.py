"""Bounded device waits (failure detection without a GPU fault): the general
replay's evaluating warps wait for the replay with a bounded number of
polls; TSG_TEST_WAIT_EXPIRES makes every such wait expire at its first
check.  The launch must return normally with TSG_ERR_DEVICE_CHECK in its
check word, and the next ordinary launch on the same workspace must be clean
and give the same result as before.  (The expired launch reads items of the
same query on the same workspace, written by its earlier launch: every
access stays in bounds.)"""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def test_expired_wait_reports_and_next_launch_is_clean(cuda_lib):
    import torch

    import tskit_gb300
    from tskit_gb300 import _native as nat, sim
    from tskit_gb300.trees import Query

    tables = sim.simulate(200, 1e6, 3000, 3000, 31)
    ts = tskit_gb300.TreeSequence(tables)
    ts.set_compact_spans(0)  # the general replay, whose warps wait on one another
    rng = np.random.default_rng(1)
    perm = rng.permutation(tables.samples())
    sets = [np.sort(p) for p in np.array_split(perm, 2)]
    terms = [(O.DIVERSITY, (0,)), (O.DIVERGENCE, (0, 1)), (O.SEGSITES, (1,))]
    windows = np.linspace(0, tables.sequence_length, 5)
    base = nat.STAT_BRANCH | nat.STAT_SPAN_NORMALISE
    q = Query(ts, sets, terms, windows, base)
    q_exp = Query(ts, sets, terms, windows, base | nat.TEST_WAIT_EXPIRES)
    ws = tskit_gb300.Workspace(max(q.workspace_bytes, q_exp.workspace_bytes))
    res = torch.zeros(q.result_size, dtype=torch.float64, device="cuda")

    q.launch(ws, res)
    torch.cuda.synchronize()
    q.check(ws)
    ref = res.cpu().numpy().copy()
    exp = O.sample_count_stat(O.OracleTS(tables), sets, terms, windows=windows, mode="branch")
    np.testing.assert_allclose(ref.reshape(exp.shape), exp, rtol=1e-12)

    q_exp.launch(ws, res)
    torch.cuda.synchronize()
    assert cuda_lib.tsg_workspace_check(ws.handle, q_exp.handle) == nat.ERR_DEVICE_CHECK

    res.zero_()
    q.launch(ws, res)
    torch.cuda.synchronize()
    q.check(ws)
    np.testing.assert_array_equal(res.cpu().numpy(), ref)
