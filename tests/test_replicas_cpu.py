"""bench.py's multi-GPU path is N independent replicas (searches and crystal steps do not exchange data):
every rank runs the workload, timing is the maximum over ranks and the whole-job value counts all
ranks' units. This runs that aggregation with two gloo ranks on the CPU (127.0.0.1)."""
import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q) -> None:
    import torch.distributed as dist

    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 10.0 + 5.0 * rank  # rank 1 is the slowest
    m = bench.reduce_max(ms)
    v = bench.replica_value(1000, world, 7, m)
    dist.barrier()
    q.put((rank, m, v))
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [15.0, 15.0]
    assert out[0][2] == out[1][2] == pytest.approx(1000 * 2 * 7 / 15e-3)


def test_single_process_is_its_own_maximum():
    import bench

    assert bench.reduce_max(3.5) == 3.5
    assert bench.replica_value(10, 1, 2, 1000.0) == pytest.approx(20.0)
