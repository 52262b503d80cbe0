"""The multi-rank path of bench.py on CPU: two gloo ranks, each a replica of the workload,
reduce to the slowest rank's time and the sum of agent-steps (no GPU involved)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    local_ms = 100.0 * (rank + 1)
    local_work = 1000 * (rank + 1)
    q.put((rank, bench.replica_throughput(dist, local_ms, local_work)))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for r in (0, 1):
        t_max, total, value = out[r]
        assert t_max == 200.0 and total == 3000.0
        assert value == pytest.approx(3000.0 / 0.2)


def test_replica_throughput_single_process():
    import bench

    assert bench.replica_throughput(None, 250.0, 500) == (250.0, 500.0, 2000.0)
