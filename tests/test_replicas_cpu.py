"""The multi-GPU form is replicas only (no exchange step): each rank runs the whole workload and the job
value is all ranks' samples over the slowest rank's time.  The cross-rank part, checked with two gloo
ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench

    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert bench.dist_env() == (rank, world, rank)
        slowest = bench.max_over_ranks(10.0 + 5.0 * rank, world, "cpu")
        q.put((rank, slowest))
    finally:
        torch.distributed.destroy_process_group()


def test_max_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 15.0), (1, 15.0)]


def test_single_rank_passthrough():
    import bench

    assert bench.max_over_ranks(3.5, 1, "cpu") == 3.5
