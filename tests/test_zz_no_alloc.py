"""The launch that allocates nothing (tsg_query_launch_noalloc), on a GPU.

Callers that cannot allocate device memory while a query runs -- a host that
owns a fixed device-memory budget, or a latency-critical serving path -- run
a prepared query with the scratch taken from a fixed 32 MiB array compiled
into the library.  This file is collected last so that a failure here does not
hide the other GPU tests.  It calls the C ABI directly and compares with the
ordinary workspace launch, twice in a row (the array keeps the previous
call's contents, which must not leak into the next result).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _query(lib, ts, sets, terms, windows, flags):
    from tskit_gb300 import _native as nat

    sizes = np.array([len(s) for s in sets], dtype=np.uint64)
    flat = np.concatenate(sets).astype(np.int32)
    outs = (nat.Output_t * len(terms))()
    for r, (typ, idx) in enumerate(terms):
        outs[r].type = typ
        for j, v in enumerate(list(idx) + [0] * (4 - len(idx))):
            outs[r].idx[j] = v
    win = np.ascontiguousarray(windows, dtype=np.float64)
    h = ctypes.c_void_p()
    err = lib.tsg_query_create(
        ctypes.byref(h), ts._handle, len(sizes), sizes.ctypes.data_as(ctypes.c_void_p),
        flat.ctypes.data_as(ctypes.c_void_p), len(terms), ctypes.cast(outs, ctypes.c_void_p),
        len(win) - 1, win.ctypes.data_as(ctypes.c_void_p), flags)
    assert err == 0, err
    return h


def test_noalloc_matches_workspace_launch(cuda_lib):
    import torch

    import tskit_gb300
    from tskit_gb300 import _native as nat, sim

    lib = cuda_lib
    tables = sim.simulate(200, 1e6, 400, 2000, 21)
    ts = tskit_gb300.TreeSequence(tables)
    rng = np.random.default_rng(3)
    perm = rng.permutation(tables.samples())
    sets = [np.sort(p) for p in np.array_split(perm, 3)]
    terms = [(nat.DIVERSITY, (0,)), (nat.DIVERSITY, (2,)), (nat.DIVERGENCE, (0, 1)),
             (nat.Y3, (0, 1, 2)), (nat.SEGREGATING_SITES, (1,))]
    windows = np.linspace(0, tables.sequence_length, 9)
    for precision in (0, nat.PRECISION_F32_KAHAN):
        q = _query(lib, ts, sets, terms, windows, nat.STAT_BOTH_MODES | precision)
        try:
            nbytes = lib.tsg_query_workspace_bytes(q)
            assert 0 < nbytes <= nat.NOALLOC_SCRATCH_BYTES
            size = lib.tsg_query_result_size(q)
            stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
            ws = ctypes.c_void_p()
            assert lib.tsg_workspace_create(ctypes.byref(ws)) == 0
            assert lib.tsg_workspace_reserve(ws, nbytes) == 0
            ref = torch.zeros(size, dtype=torch.float64, device="cuda")
            assert lib.tsg_query_launch(q, ws, ctypes.c_void_p(ref.data_ptr()), stream) == 0
            torch.cuda.synchronize()
            assert lib.tsg_workspace_check(ws, q) == 0
            lib.tsg_workspace_free(ws)
            for _ in range(2):
                out = torch.full((size,), np.nan, dtype=torch.float64, device="cuda")
                err = lib.tsg_query_launch_noalloc(q, ctypes.c_void_p(out.data_ptr()), stream)
                assert err == 0, err
                torch.cuda.synchronize()
                assert lib.tsg_noalloc_check(q) == 0
                np.testing.assert_allclose(out.cpu().numpy(), ref.cpu().numpy(), rtol=RTOL,
                                           atol=1e-14)
        finally:
            lib.tsg_query_free(q)


def test_noalloc_refuses_oversized_query(cuda_lib):
    import torch

    import tskit_gb300
    from tskit_gb300 import _native as nat, sim

    lib = cuda_lib
    tables = sim.simulate(50, 1e6, 100, 500, 5)
    ts = tskit_gb300.TreeSequence(tables)
    sets = [tables.samples()[:25], tables.samples()[25:]]
    # enough windows that the per-window accumulators exceed the array
    windows = np.linspace(0, tables.sequence_length, 400_001)
    terms = [(nat.DIVERSITY, (0,))] * 16
    q = _query(lib, ts, sets, terms, windows, nat.STAT_BOTH_MODES)
    try:
        assert lib.tsg_query_workspace_bytes(q) > nat.NOALLOC_SCRATCH_BYTES
        out = torch.zeros(lib.tsg_query_result_size(q), dtype=torch.float64, device="cuda")
        err = lib.tsg_query_launch_noalloc(q, ctypes.c_void_p(out.data_ptr()),
                                           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert err == nat.ERR_NOALLOC_TOO_LARGE
    finally:
        lib.tsg_query_free(q)
