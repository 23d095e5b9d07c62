"""One ensemble over the GPUs of a node: one process per GPU, each advancing a
contiguous shard of the tracers, then one host gather.

Tracers are independent (no exchange step during integration), so an ensemble
shards with no collective on the data path. The shards are contiguous index
ranges balanced by an estimate of each tracer's cost, in right-hand-side field
evaluations over the requested advance:

  particle:       delta / T_c            x  K_PARTICLE
  guiding centre: delta * v / |x|        x  K_GC

T_c is the cyclotron period at the start (utils.cyclotron_period,
rapt/utils.py:62-66): the DOP853 controller resolves the gyration, about 14
right-hand sides per period at rtol 1e-8, each one field evaluation. A guiding
centre's steps follow its transit along the field line, v / |x|; DOPRI5 takes
about 150 right-hand sides per transit at rtol 1e-8 (the 1M config-2 ensemble:
~930 per tracer-second), each seven field evaluations. The constants only set
the relative weight of the two modes (an Adaptive ensemble is weighted by each
tracer's mode at the start). After the advance, ``gather`` brings every shard's
final state to rank 0 in index order and ``sum_counters`` adds the step
counters: the host-side collective the sharded path needs (gloo or any
torch.distributed backend with object collectives).
"""
import numpy as np

C_LIGHT = 299792458.0
K_PARTICLE = 14.0 * 1.0
K_GC = 150.0 * 7.0


def cost_estimate(mode, pos, speed, mass, charge, magB, delta):
    """Estimated field evaluations per tracer. mode: 0 particle, 1 guiding
    centre (arrays or scalars broadcast to the tracer count)."""
    pos = np.atleast_2d(np.asarray(pos, float))
    n = pos.shape[0]
    mode, speed, mass, charge, magB, delta = (np.broadcast_to(np.asarray(a, float), (n,))
                                              for a in (mode, speed, mass, charge, magB, delta))
    gamma = 1.0 / np.sqrt(1.0 - (speed / C_LIGHT) ** 2)
    fc = np.abs(charge) * magB / (2 * np.pi * gamma * mass)  # 1 / T_c
    r = np.linalg.norm(pos, axis=1)
    return np.where(mode == 0, delta * fc * K_PARTICLE, delta * speed / np.maximum(r, 1.0) * K_GC)


def partition(costs, world):
    """Contiguous [start, stop) ranges, one per rank, with the cumulative cost
    split as evenly as contiguity allows (each boundary at the first index where
    the running cost reaches rank / world of the total). Every rank gets at
    least one tracer when there are at least `world` tracers."""
    costs = np.asarray(costs, float)
    n = len(costs)
    if world <= 1 or n == 0:
        return [(0, n)]
    cum = np.cumsum(np.maximum(costs, 0.0))
    total = cum[-1]
    bounds = [0]
    for r in range(1, world):
        b = int(np.searchsorted(cum, total * r / world, side="left")) + 1 if total > 0 else (n * r) // world
        lo = bounds[-1] + (1 if n >= world else 0)
        hi = n - (world - r) if n >= world else n
        bounds.append(min(max(b, lo), hi))
    bounds.append(n)
    return [(bounds[r], bounds[r + 1]) for r in range(world)]


def shard(costs, rank, world):
    """This rank's [start, stop)."""
    return partition(costs, world)[rank]


def gather(dist, arrays, dst=0):
    """Gather a dict of numpy arrays (first axis = this rank's tracers) to rank
    `dst`, concatenated in rank order; other ranks get None. Without a process
    group the arrays are returned as they are."""
    if dist is None:
        return arrays
    world = dist.get_world_size()
    out = [None] * world if dist.get_rank() == dst else None
    dist.gather_object({k: np.asarray(v) for k, v in arrays.items()}, out, dst=dst)
    if dist.get_rank() != dst:
        return None
    return {k: np.concatenate([o[k] for o in out], axis=0) for k in arrays}


def sum_counters(dist, counters):
    """Sum a dict of integer counters over the ranks (every rank gets the sums)."""
    if dist is None:
        return dict(counters)
    import torch
    keys = sorted(counters)
    t = torch.tensor([int(counters[k]) for k in keys], dtype=torch.int64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return {k: int(v) for k, v in zip(keys, t.tolist())}
