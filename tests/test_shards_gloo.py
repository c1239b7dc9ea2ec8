"""Multi-rank host logic on CPU: two gloo ranks partition a ragged
population by compartment count, gather per-cable results back in population
order, and reduce their timings the way a ``torchrun --nproc-per-node N
bench.py`` run does on GPUs.

Each rank builds its own shard's population on the host (geometry, workspace,
extracellular field) and checks that the shards are disjoint, cover every
cable, carry nearly equal compartment counts, and that ``reduce_timing``
returns the slowest rank's time and the summed work.
"""

import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from dendra_gb300.shards import balanced_shards, gather_cables, reduce_timing, shard_of
from dendra_gb300.workloads import c2_spec

N_CABLES = 512
SEED = 7
WORLD = 2


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from dendra_gb300.workloads import cable_population_c2

        ks = c2_spec(N_CABLES, SEED)["ks"]
        mine = shard_of(ks, world, rank)
        pop = cable_population_c2(n_cables=N_CABLES, seed=SEED, dtype=torch.float64,
                                  device="cpu", subset=mine)
        assert pop.B == len(mine)
        assert pop.N == int(ks[mine].sum())

        shards = [None] * world
        dist.all_gather_object(shards, mine.tolist())
        flat = np.concatenate([np.asarray(s, dtype=np.int64) for s in shards])
        assert np.array_equal(np.sort(flat), np.arange(N_CABLES))  # disjoint and complete
        loads = [int(ks[np.asarray(s, dtype=np.int64)].sum()) for s in shards]
        assert max(loads) - min(loads) <= int(ks.max())

        # per-cable results back in population order on every rank
        local = torch.as_tensor(ks[mine] * 10.0 + rank, dtype=torch.float64)[:, None]
        full = gather_cables(local, mine, N_CABLES)
        owner = np.empty(N_CABLES)
        for r, s in enumerate(shards):
            owner[np.asarray(s, dtype=np.int64)] = r
        assert full.shape == (N_CABLES, 1)
        assert np.array_equal(full[:, 0].numpy(), ks * 10.0 + owner)

        steps = 2000
        ms, units = reduce_timing(10.0 + 5.0 * rank, pop.N * steps)
        assert ms == 10.0 + 5.0 * (world - 1)
        assert units == float(ks.sum()) * steps
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_reduce():
    mp.spawn(_rank_main, args=(WORLD, _free_port()), nprocs=WORLD, join=True)


def test_balanced_shards_properties():
    rng = np.random.default_rng(3)
    for world in (1, 2, 3, 4, 8):
        sizes = rng.integers(0, 400, 1000)
        shards = balanced_shards(sizes, world)
        assert len(shards) == world
        flat = np.concatenate(shards)
        assert np.array_equal(np.sort(flat), np.arange(sizes.size))
        for s in shards:
            assert np.all(np.diff(s) > 0)
        loads = [int(sizes[s].sum()) for s in shards]
        assert max(loads) - min(loads) <= int(sizes.max())
        assert all(np.array_equal(a, b) for a, b in zip(shards, balanced_shards(sizes, world)))


def test_balanced_shards_edges():
    assert [s.tolist() for s in balanced_shards([], 3)] == [[], [], []]
    # more ranks than cables: the extra ranks own nothing
    assert [s.tolist() for s in balanced_shards([5, 9], 4)] == [[1], [0], [], []]
    with pytest.raises(ValueError):
        balanced_shards([1, 2], 0)
    with pytest.raises(ValueError):
        balanced_shards([1, -2], 2)
    with pytest.raises(ValueError):
        shard_of([1, 2], 2, 2)


def test_reduce_timing_without_group():
    assert reduce_timing(3.5, 7) == (3.5, 7.0)


def test_gather_cables_without_group_checks_coverage():
    vals = torch.arange(4.0)
    out = gather_cables(vals, [2, 0, 3, 1], 4)
    assert out.tolist() == [1.0, 3.0, 0.0, 2.0]
    with pytest.raises(ValueError, match="in no shard"):
        gather_cables(vals[:3], [0, 1, 2], 4)
    with pytest.raises(ValueError, match="overlap"):
        gather_cables(vals, [0, 0, 1, 2], 4)
    with pytest.raises(ValueError, match="entries for a shard"):
        gather_cables(vals, [0, 1], 4)
