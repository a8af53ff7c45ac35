"""The N > 1 path of bench.py: N independent replicas, one per rank, timed by
the slowest rank.  Runs as two gloo ranks on the CPU (no GPU needed)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    import torch.distributed as dist
    os.environ.update({"WORLD_SIZE": str(ws), "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    ms, value = bench.replica_value(10.0 + 5.0 * rank, 1000, 4)
    q.put((rank, ms, value))
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=10) for _ in range(2))
    for rank, ms, value in out:
        assert ms == 15.0                         # max over ranks
        assert value == pytest.approx(2 * 1000 * 2 * 4 / 0.015)


def test_single_replica_value():
    import bench
    os.environ.pop("WORLD_SIZE", None)
    ms, value = bench.replica_value(20.0, 500, 3)
    assert ms == 20.0 and value == pytest.approx(500 * 2 * 3 / 0.02)
