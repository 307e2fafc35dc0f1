"""The multi-process path of bench.py on CPU: two ranks over gloo (the
replicas of bench.py --gpus N share nothing but the timing reduction and the
barrier).  The job's time is the slowest rank's; the reference arm runs on
rank 0 only."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        got = bench.max_over_ranks(1.5 + rank, world, device="cpu")
        # the reference arm returns at once on ranks other than 0
        ran = rank != 0 and bench.run_reference(None) is None
        dist.barrier()
        out.put((rank, got, ran))
    finally:
        dist.destroy_process_group()


def test_two_ranks_gloo():
    ctx = torch.multiprocessing.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(out.get(timeout=10) for _ in range(2))
    assert [r[1] for r in res] == [2.5, 2.5]
    assert res[1][2] is True


def test_one_rank_is_identity():
    import bench

    assert bench.max_over_ranks(3.25, 1) == 3.25
