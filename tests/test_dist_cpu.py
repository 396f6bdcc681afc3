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


def _shard_worker(rank, world, port, out):
    """Each rank translates its target shard of one batch (the oracle's FP64
    rotation restatement stands in for the GPU kernel); the owned ranges,
    summed across ranks, must equal the one-rank result bit for bit."""
    import sys

    import numpy as np

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "oracle"))
    sys.path.insert(0, root)
    import pyoracle

    from solidfmm_gb300.shard import shard_by_target, target_range

    dist.init_process_group("gloo", rank=rank, world_size=world)
    P, n, nsrc, ntgt = 6, 300, 40, 37
    rng = np.random.default_rng(11)
    S = P * (P + 1)
    src = rng.normal(size=(nsrc, S))
    sidx = rng.integers(0, nsrc, n).astype(np.uint32)
    tidx = rng.integers(0, ntgt, n).astype(np.uint32)  # targets repeat
    pin = rng.integers(1, P + 1, n).astype(np.uint32)
    pout = rng.integers(1, P + 1, n).astype(np.uint32)
    d = rng.normal(size=(n, 3))
    xyz = d / np.linalg.norm(d, axis=1, keepdims=True) * 3.0
    full = np.zeros((ntgt, S))
    pyoracle.rot("m2l", src, pin, full, pout, xyz, sidx=sidx, tidx=tidx)
    pos = shard_by_target(tidx, ntgt, world, rank)
    mine = np.zeros((ntgt, S))
    pyoracle.rot("m2l", src, pin[pos], mine, pout[pos], xyz[pos], sidx=sidx[pos], tidx=tidx[pos])
    lo, hi = target_range(ntgt, world, rank)
    untouched = bool(np.all(mine[:lo] == 0) and np.all(mine[hi:] == 0))
    t = torch.from_numpy(mine)
    dist.all_reduce(t)  # owned ranges are disjoint: the sum assembles them
    out[rank] = (untouched, bool(np.array_equal(t.numpy(), full)), len(pos))
    dist.destroy_process_group()


@pytest.mark.timeout(180)
def test_two_rank_target_shards_reassemble_the_batch():
    world = 2
    port = _free_port()
    out = mp.Manager().dict()
    mp.spawn(_shard_worker, args=(world, port, out), nprocs=world, join=True)
    assert all(out[r][0] for r in range(world))  # no rank wrote outside its targets
    assert all(out[r][1] for r in range(world))  # bit-identical to one rank
    assert out[0][2] + out[1][2] == 300  # every entry ran exactly once


def test_target_ranges_cover_and_split_evenly():
    from solidfmm_gb300.shard import shard_by_target, target_range

    import numpy as np

    for n, w in ((10, 3), (7, 7), (5, 8), (0, 2), (1000, 4)):
        ranges = [target_range(n, w, r) for r in range(w)]
        assert ranges[0][0] == 0 and ranges[-1][1] == n
        assert all(a[1] == b[0] for a, b in zip(ranges, ranges[1:]))
        sizes = [hi - lo for lo, hi in ranges]
        assert max(sizes) - min(sizes) <= 1
    tidx = np.array([4, 0, 9, 4, 2, 7, 7, 1])
    parts = [shard_by_target(tidx, 10, 3, r) for r in range(3)]
    assert sorted(np.concatenate(parts).tolist()) == list(range(len(tidx)))
    assert all(np.all(np.diff(p) > 0) for p in parts if len(p))  # batch order kept
    assert shard_by_target(None, 10, 3, 1).tolist() == [4, 5, 6]
    t = torch.tensor([3, 8, 0])
    assert shard_by_target(t, 10, 2, 1).tolist() == [1]
    with pytest.raises(ValueError):
        target_range(4, 2, 2)
