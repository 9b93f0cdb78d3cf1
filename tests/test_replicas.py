"""The multi-GPU path (replicas, one process per GPU) reduces units and
times over ranks: world_size 2 over gloo on the CPU."""
import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from snapatac2_gb300._replicas import replica_throughput
    q.put((rank, replica_throughput(100.0 * (rank + 1), 10.0 + 5 * rank)))
    dist.destroy_process_group()


def test_replica_throughput_single_process():
    from snapatac2_gb300._replicas import replica_throughput
    assert replica_throughput(7, 3.5) == (7.0, 3.5)


@pytest.mark.timeout(120)
def test_replica_throughput_two_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=90) for _ in procs)
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    assert out[0] == out[1] == (300.0, 15.0)
