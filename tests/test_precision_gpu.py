"""Stated error bounds of the fused sweep's two arithmetic forms, on a reduced
windowed workload (n=2,000, 4 sets of 500, 200 windows; diversity,
segregating sites, divergence, Y3 and the derived Fst and Tajima's D, branch
and site).  Errors are normwise per statistic, scaled by each statistic's
componentwise condition in its raw terms (bench.cond_err), so that Fst near
0 -- random subsets of one population -- is not read as a failure:

* FP64 form: <= 1e-12 against the compensated (double-double) branch oracle
  and against the FP64 oracle in site mode (the GPU's site sums are exact
  integers rounded once);
* FP32-compensated form: <= 1e-5 against the same.

The FP64 oracle itself (the reference's arithmetic) is checked against the
compensated oracle at the same 1e-12, which attributes any FP64 disagreement.
"""
import numpy as np
import pytest

import bench
import oracle as O

pytestmark = pytest.mark.gpu

NUM_WINDOWS = 200


@pytest.fixture(scope="module")
def workload(cuda_lib):
    import tskit_gb300
    from tskit_gb300 import sim

    tables = sim.simulate(2000, 2e7, 20000, 40000, 4242)
    rng = np.random.default_rng(7)
    perm = rng.permutation(tables.samples())
    sets = [np.sort(perm[j * 500:(j + 1) * 500]).astype(np.int32) for j in range(4)]
    windows = np.linspace(0, tables.sequence_length, NUM_WINDOWS + 1)
    terms, pairs, triples = bench.term_list()
    ts = tskit_gb300.TreeSequence(tables)
    ots = O.OracleTS(tables)
    raw_o = np.zeros((2, NUM_WINDOWS, len(terms)))
    for m, mode in enumerate(bench.MODES):
        raw_o[m] = O.sample_count_stat(ots, sets, terms, windows=windows, mode=mode,
                                       span_normalise=False)
    raw_dd = raw_o.copy()
    raw_dd[0] = O.branch_count_stat_dd(ots, sets, terms, windows=windows, span_normalise=False)
    return ts, sets, windows, terms, pairs, raw_o, raw_dd


def _gpu_raw(ts, sets, windows, terms, precision):
    import torch

    import tskit_gb300

    q = ts.query(sets, terms, windows=windows, both_modes=True, span_normalise=False,
                 precision=precision)
    ws = tskit_gb300.Workspace(q.workspace_bytes)
    res = torch.zeros(q.result_size, dtype=torch.float64, device="cuda")
    q.launch(ws, res)
    torch.cuda.synchronize()
    q.check(ws)
    return res.cpu().numpy().reshape(2, len(windows) - 1, len(terms))


def _finish(raw, windows, sets, pairs):
    saved = bench.NUM_WINDOWS
    bench.NUM_WINDOWS = len(windows) - 1
    try:
        return bench.finish(raw, windows, sets, pairs)
    finally:
        bench.NUM_WINDOWS = saved


def _errors(raw, ref, windows, sets, pairs):
    fin = _finish(raw, windows, sets, pairs)
    fref = _finish(ref, windows, sets, pairs)
    out = {}
    for mode in bench.MODES:
        for stat in ("diversity", "divergence", "Fst", "Tajimas_D", "Y3"):
            out[f"{mode}.{stat}"] = bench.cond_err(fin[mode], fref[mode], stat, pairs, sets)
    return out


@pytest.mark.parametrize("precision,bound", [("f64", bench.ERROR_BOUNDS["f64"]),
                                             ("f32", bench.ERROR_BOUNDS["f32k"])])
def test_fused_sweep_error_bounds(workload, precision, bound):
    ts, sets, windows, terms, pairs, raw_o, raw_dd = workload
    raw = _gpu_raw(ts, sets, windows, terms, precision)
    # branch against the compensated oracle, site against the FP64 oracle
    truth = raw_o.copy()
    truth[0] = raw_dd[0]
    errs = _errors(raw, truth, windows, sets, pairs)
    bad = {k: v for k, v in errs.items() if not v <= bound}
    assert not bad, bad
    if precision == "f64":
        # the FP64 form's raw terms are at least about as close to the
        # compensated values as the reference's own FP64 arithmetic
        ref_errs = _errors(raw_o, truth, windows, sets, pairs)
        for k in ("branch.diversity", "branch.divergence", "branch.Y3"):
            assert errs[k] <= max(8 * ref_errs[k], 1e-14), (k, errs[k], ref_errs[k])


def test_fp64_oracle_within_bound_of_compensated(workload):
    ts, sets, windows, terms, pairs, raw_o, raw_dd = workload
    truth = raw_o.copy()
    truth[0] = raw_dd[0]
    errs = _errors(raw_o, truth, windows, sets, pairs)
    assert max(errs.values()) <= bench.ERROR_BOUNDS["f64"], errs
