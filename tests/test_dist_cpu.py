"""Two gloo ranks on CPU exercising the replica helpers bench.py uses for
--gpus N > 1 (the translation path shards without any collective; ranks only
meet at a barrier and a max-reduction of their step times)."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.barrier(world)
    v = bench.allmax(world, 1.5 + rank, torch.device("cpu"))
    out[rank] = v
    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_rank_barrier_and_max():
    world = 2
    port = _free_port()
    out = mp.Manager().dict()
    mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
    assert out[0] == out[1] == 2.5
