"""Sharding of independent cables over the ranks of one node (one process per GPU).

Cables, fibres and gradient lanes of a population are independent (the
reference steps each ``Population`` cable with its own tridiagonal system,
integrators/implicit.py:569-664), so a multi-GPU run partitions them and each
rank advances its own shard with no collective on the data path.  The only
exchanges are host-side: after the run, the slowest rank's time and the total
work over all ranks, or a gather of results.

``balanced_shards`` partitions cables by compartment count so that every rank
gets nearly the same number of compartment-steps; ``gather_cables`` puts the
ranks' per-cable results (spike counts, thresholds, gradients) back in
population order; ``reduce_timing`` turns each rank's timed region into the
whole-job figure (max time over ranks, summed work).  The collectives work on
any ``torch.distributed`` backend: NCCL on a GPU node (each rank's device set
current first), gloo on CPU.
"""

from __future__ import annotations

import heapq

import numpy as np
import torch


def balanced_shards(sizes, world: int) -> list[np.ndarray]:
    """Partition item indices into ``world`` shards of nearly equal total size.

    ``sizes[i]`` is item i's work (compartments of cable i).  Items go, largest
    first (ties by index), to the shard with the smallest total so far (ties by
    rank), so every shard total lies within ``max(sizes)`` of every other.  Each
    shard's indices are returned in ascending order; the result depends only on
    ``sizes`` and ``world``, so every rank computes the same partition.
    """
    if world < 1:
        raise ValueError(f"world must be >= 1 (got {world})")
    sizes = np.asarray(sizes)
    if sizes.ndim != 1:
        raise ValueError("sizes must be one-dimensional")
    if sizes.size and int(sizes.min()) < 0:
        raise ValueError("sizes must be non-negative")
    order = np.lexsort((np.arange(sizes.size), -sizes.astype(np.int64)))
    heap = [(0, r) for r in range(world)]
    owner = np.empty(sizes.size, dtype=np.int64)
    for i in order:
        load, r = heapq.heappop(heap)
        owner[i] = r
        heapq.heappush(heap, (load + int(sizes[i]), r))
    return [np.flatnonzero(owner == r) for r in range(world)]


def shard_of(sizes, world: int, rank: int) -> np.ndarray:
    """Indices of the items that ``rank`` owns under ``balanced_shards``."""
    if not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside [0, {world})")
    return balanced_shards(sizes, world)[rank]


def gather_cables(local: torch.Tensor, shard, n_total: int, group=None) -> torch.Tensor:
    """Reassemble per-cable results of every rank in population order.

    ``local`` holds this rank's results, one leading-dimension entry per cable
    of ``shard`` (in the shard's order); the result, on every rank, is a CPU
    tensor with ``n_total`` entries where entry ``shard[j]`` of each rank is
    that rank's ``local[j]``.  Results travel once, at the end of a run, so
    they go through the host (``all_gather_object``) on any backend.  Without
    an initialised process group, ``shard`` must cover the whole population.
    """
    import torch.distributed as dist

    shard = np.asarray(shard, dtype=np.int64)
    local = local.detach().cpu()
    if local.shape[0] != shard.size:
        raise ValueError(f"local has {local.shape[0]} entries for a shard of {shard.size}")
    if dist.is_available() and dist.is_initialized():
        parts = [None] * dist.get_world_size(group)
        dist.all_gather_object(parts, (shard, local), group=group)
    else:
        parts = [(shard, local)]
    out = torch.empty((n_total, *local.shape[1:]), dtype=local.dtype)
    seen = np.zeros(n_total, dtype=bool)
    for idx, vals in parts:
        if idx.size and (idx.min() < 0 or idx.max() >= n_total or seen[idx].any()
                         or np.unique(idx).size != idx.size):
            raise ValueError("shards overlap or fall outside the population")
        seen[idx] = True
        out[torch.as_tensor(idx)] = vals
    if not seen.all():
        raise ValueError(f"{int((~seen).sum())} cables are in no shard")
    return out


def reduce_timing(ms: float, units: float, group=None, device=None) -> tuple[float, float]:
    """Whole-job ``(max ms over ranks, summed work units)`` of one timed region.

    Each rank passes its own region time and the units it processed; the job's
    throughput is ``units_total / max_ms``.  Without an initialised process
    group the rank's own figures come back unchanged.  ``device`` holds the
    reduction tensors: a CUDA device for NCCL, CPU (the default) for gloo.
    """
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return float(ms), float(units)
    dev = torch.device("cpu") if device is None else torch.device(device)
    t = torch.tensor([float(ms)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    n = torch.tensor([float(units)], dtype=torch.float64, device=dev)
    dist.all_reduce(n, op=dist.ReduceOp.SUM, group=group)
    return float(t.item()), float(n.item())
