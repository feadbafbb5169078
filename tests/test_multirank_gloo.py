"""The N>1 path of bench.py (independent replicas per rank, one reduction of
the timing and the walker-step count) on CPU with the gloo backend."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms, ws = bench.reduce_over_ranks(10.0 + rank, 1000.0 * (rank + 1), dist, torch.device("cpu"))
    q.put((rank, ms, ws))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_reduce_over_ranks_gloo(world):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for rank, ms, ws in res:
        assert ms == 10.0 + (world - 1)          # slowest rank
        assert ws == sum(1000.0 * (r + 1) for r in range(world))  # all ranks' walker-steps
