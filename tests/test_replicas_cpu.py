"""The multi-GPU replica path of bench.py on two gloo ranks on the CPU: each rank reports its
own time, the job rate uses the slowest rank (no data-path collective exists; the solve is
replicated per GPU)."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    rate, tmax = bench.replica_rate(100.0 * (rank + 1), 5, world, "cpu")
    out[rank] = (rate, tmax)
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_rate_uses_the_slowest_rank():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        rate, tmax = res[rank]
        assert tmax == pytest.approx(200.0)            # the slower rank's 200 ms
        assert rate == pytest.approx(2 * 5 / 0.2)      # 10 steps in total over 0.2 s
