"""Work sharding across ranks for the multi-GPU runs.

The path has no exchange step: molecules, planes and point batches are
independent, so N GPUs run as N processes that each take a share of the
units and need no collective on the data path (weak scaling).  Only the
timing and the unit counts are reduced, for reporting.
"""
import numpy as np


def shard_indices(costs, rank, world):
    """Indices of the units that ``rank`` of ``world`` processes: largest
    cost first to the least-loaded rank (ties to the lower rank), which is
    deterministic and keeps the ranks within one unit's cost of each other.
    Returned in ascending order."""
    costs = np.asarray(costs, dtype=np.float64)
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank %r of world %r" % (rank, world))
    load = np.zeros(world)
    owner = np.empty(len(costs), dtype=np.int64)
    for i in sorted(range(len(costs)), key=lambda k: (-costs[k], k)):
        r = int(np.argmin(load))
        owner[i] = r
        load[r] += costs[i]
    return [int(i) for i in np.nonzero(owner == rank)[0]]


def reduce_scalar(value, op="max", dist=None, device=None):
    """value reduced over the ranks of the default process group (the value
    itself without one)."""
    if dist is None or not dist.is_available() or not dist.is_initialized():
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op={"max": dist.ReduceOp.MAX, "sum": dist.ReduceOp.SUM}[op])
    return float(t.item())
