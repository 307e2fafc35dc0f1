"""Edge orders sorted on the device (tsg_edge_orders) against the host
lexicographic sorts of the reference's keys (c/tskit/tables.c:11393-11450;
the edge order of tsk_table_collection_sort), ties in edge-table order."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def host_orders(left, right, parent, child, time):
    tp = time[parent]
    sort = np.lexsort((left, child, parent, tp), axis=0)
    ins = np.lexsort((child, parent, tp, left))
    rem = np.lexsort((-child, -parent, -tp, right))
    return sort, ins, rem


def device_orders(lib, left, right, parent, child, time):
    import torch

    dev = torch.device("cuda")
    E = len(left)
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in
         dict(left=left, right=right, parent=parent.astype(np.int32),
              child=child.astype(np.int32), time=time).items()}
    outs = [torch.full((max(E, 1),), -1, dtype=torch.int32, device=dev) for _ in range(3)]
    code = lib.tsg_edge_orders(E, t["left"].data_ptr(), t["right"].data_ptr(),
                               t["parent"].data_ptr(), t["child"].data_ptr(),
                               t["time"].data_ptr(), outs[0].data_ptr(), outs[1].data_ptr(),
                               outs[2].data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert code == 0
    return [o.cpu().numpy()[:E] for o in outs]


def _shuffled(seed):
    from tskit_gb300 import sim

    t = sim.simulate(200, 1e5, 400, 0, seed)
    rng = np.random.default_rng(seed)
    perm = rng.permutation(t.num_edges)
    return (t.edge_left[perm], t.edge_right[perm], t.edge_parent[perm], t.edge_child[perm],
            t.node_time)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_orders_match_host(seed, cuda_lib):
    cols = _shuffled(seed)
    for d, h in zip(device_orders(cuda_lib, *cols), host_orders(*cols)):
        np.testing.assert_array_equal(d, h)


def test_ties_and_negative_coordinates(cuda_lib):
    """Equal keys keep table order; negative times and ids order correctly."""
    rng = np.random.default_rng(9)
    E = 5000
    left = rng.integers(-3, 3, E).astype(np.float64)
    right = left + rng.integers(1, 3, E)
    time = np.concatenate([[-1.5, -0.0, 0.0], rng.normal(size=60)])
    parent = rng.integers(0, len(time), E).astype(np.int32)
    child = rng.integers(0, len(time), E).astype(np.int32)
    for d, h in zip(device_orders(cuda_lib, left, right, parent, child, time),
                    host_orders(left, right, parent, child, time)):
        np.testing.assert_array_equal(d, h)


def test_tree_sequence_uses_device_index(cuda_lib):
    """A tree sequence built from tables gives the reference's statistics
    with its indexes sorted on the device."""
    import tskit_gb300
    from tskit_gb300 import sim

    import oracle as O

    t = sim.simulate(100, 1e5, 300, 500, 5)
    ts = tskit_gb300.TreeSequence(t)
    ots = O.OracleTS(t)
    s = [t.samples()[:50], t.samples()[50:]]
    for mode in ("branch", "site"):
        np.testing.assert_allclose(ts.divergence(s, mode=mode),
                                   O.call(ots, "divergence", dict(sample_sets=s, mode=mode)),
                                   rtol=1e-12)
