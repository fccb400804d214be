"""Sharding of independent units across ranks, with world_size 2 gloo
process groups on the CPU (the multi-GPU runs use the same host logic)."""
import os
import socket

import numpy as np
import pytest

from gimic_gb300 import shard


def test_shards_partition_and_balance():
    rng = np.random.default_rng(0)
    costs = rng.uniform(1, 100, 57)
    for world in (1, 2, 3, 8):
        parts = [shard.shard_indices(costs, r, world) for r in range(world)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        loads = [costs[p].sum() for p in parts]
        assert max(loads) - min(loads) <= costs.max() + 1e-9
    assert shard.shard_indices([], 0, 2) == []
    with pytest.raises(ValueError):
        shard.shard_indices(costs, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, costs, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = shard.shard_indices(costs, rank, world)
    # per-rank "work": the sum of its units; the timing reduction is a max
    done = shard.reduce_scalar(len(mine), "sum", dist)
    slowest = shard.reduce_scalar(float(np.sum(np.asarray(costs)[mine])), "max", dist)
    dist.destroy_process_group()
    q.put((rank, mine, done, slowest))


@pytest.mark.timeout(120)
def test_two_gloo_ranks_cover_every_unit_once():
    import torch.multiprocessing as mp

    costs = list(np.random.default_rng(1).uniform(1, 10, 23))
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, costs, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=100) for _ in range(2))
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    units = sorted(out[0][1] + out[1][1])
    assert units == list(range(len(costs)))
    assert out[0][2] == out[1][2] == len(costs)
    loads = [sum(costs[i] for i in o[1]) for o in out]
    assert out[0][3] == out[1][3] == pytest.approx(max(loads))
