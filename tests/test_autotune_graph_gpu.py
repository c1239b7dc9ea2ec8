"""Autotuner choices and CUDA-graph capture: launch shapes change, results do not."""

import pytest
import torch

from dendra_gb300.autotune import tune_cable_run, tune_network, tune_tridiag_lanes
from dendra_gb300.network import random_network
from dendra_gb300.solvers import tridiag_solve_lanes
from tests._cases import synthetic_population

pytestmark = pytest.mark.gpu


def test_cable_run_tuning_picks_a_candidate_and_cta_size_is_result_neutral(cuda):
    """The tuner picks one of its (cables per CTA, lane split) candidates; the
    CTA size alone never changes a result (the lane split changes rounding
    only, within the oracle tolerances tested in test_full_traces_gpu.py)."""
    from dendra_gb300.autotune import CABLE_RUN_CANDIDATES

    pop = synthetic_population(3, 300, 1, 401, torch.float32, cuda, fast_math=True)
    state = tuple(t.clone() for t in (pop.v, pop.m, pop.h, pop.n))
    best, timings = tune_cable_run(pop, n_steps=20, force=True)
    assert best in CABLE_RUN_CANDIDATES and pop.warps_per_block == max(best[0], 0)
    assert pop.split_gates == (best[0] < 0)
    assert set(timings) == set(CABLE_RUN_CANDIDATES)
    for split in (None, (128, 64)):
        outs = []
        # cables per CTA 1, 2, 4 and (32 lanes only) the split-gate run
        for wpb in (1, 2, 4) + ((-1,) if split is None else ()):
            for dst, src in zip((pop.v, pop.m, pop.h, pop.n), state):
                dst.copy_(src)
            pop.step_index = 0
            pop.warps_per_block = max(wpb, 0)
            pop.split_gates = wpb < 0
            pop.lanes_split = split
            res = pop.run(100, rec_idx=0, spk_idx=0)
            pop.check_status()
            outs.append((pop.v.clone(), res.trace.clone(), res.spk_count.clone()))
        for other in outs[1:]:
            for a, b in zip(outs[0], other):
                assert torch.equal(a, b)


def test_tridiag_lane_split_tuning(cuda):
    best, timings = tune_tridiag_lanes(512, 201, torch.float64, cuda, force=True)
    assert best in timings and all(-(-201 // n) <= 32 for n in timings)
    g = torch.Generator().manual_seed(1)
    a = -torch.rand(16, 200, generator=g, dtype=torch.float64).to(cuda)
    c = -torch.rand(16, 200, generator=g, dtype=torch.float64).to(cuda)
    b = 3 + torch.rand(16, 201, generator=g, dtype=torch.float64).to(cuda)
    d = torch.randn(16, 201, generator=g, dtype=torch.float64).to(cuda)
    x = tridiag_solve_lanes(a, b, c, d, lanes=best)
    M = torch.diag_embed(b) + torch.diag_embed(a, -1) + torch.diag_embed(c, 1)
    torch.testing.assert_close(x, torch.linalg.solve(M, d), rtol=1e-10, atol=1e-12)


def _net(cuda):
    net, n = random_network(48, k_range=(50, 400), syn_per_cell=20, seed=8,
                            dtype=torch.float32, device=cuda, t_stop_ms=30.0, rate_hz=40.0)
    return net, n


def test_network_graph_replay_matches_the_eager_run(cuda):
    net, n = _net(cuda)
    eager = net.run(n)
    ref = [t.clone() for t in (net.v, net.A, net.B, net.ring, net.spike_count)]
    assert int(eager.sum()) > 0
    net.reset()
    cap = net.capture(n)
    assert (net.step, net.slot) == (0, 0) and cap.launches >= 2
    for _ in range(2):  # replay twice from the same start
        net.reset()
        raster = cap.replay()
        assert torch.equal(raster, eager)
        for a, b in zip(ref, (net.v, net.A, net.B, net.ring, net.spike_count)):
            assert torch.equal(a, b)
    with pytest.raises(RuntimeError):
        cap.replay()  # not at the captured start


def test_network_tiling_choice_is_result_neutral(cuda):
    net, n = _net(cuda)
    best, timings = tune_network(net, force=True)
    assert best in timings and len(timings) == 5
    rasters = []
    for tpc, wpb in ((32, 1), (32, 4), (64, 2), (64, 4), (128, 4), (128, 2), (256, 8), (512, 8)):
        net.threads_per_cell, net.warps_per_block = tpc, wpb
        net.reset()
        rasters.append((net.run(n), net.v.clone(), net.A.clone(), net.ring.clone()))
    for other in rasters[1:]:
        for a, b in zip(rasters[0], other):
            assert torch.equal(a, b)
