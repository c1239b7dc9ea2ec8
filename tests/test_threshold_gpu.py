"""Batched bisection thresholds on the GPU against the oracle's bisection."""

import numpy as np
import pytest
import torch

from dendra_gb300.threshold import (K_FIBRE, Thresholder, fibre_params, fibre_population,
                                    horizon_steps, node_compartment)
from tests._cases import oracle_thresholds

pytestmark = pytest.mark.gpu


def test_fibre_layout():
    assert K_FIBRE == 241
    assert node_compartment(5) == 60 and node_compartment(-5) == 192


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_thresholds_match_oracle_bisection(cuda, dtype):
    p = fibre_params(12, seed=4)
    p["pw"] = np.minimum(p["pw"], 0.3)
    pop = fibre_population(p, dtype=dtype, device=cuda)
    n = horizon_steps(p["pw"].max())
    th = Thresholder(pop, lb=0.0, ub=0.05, rtol=0.01)
    ub, lb = th.calculate_thresholds(n)
    ub_ref, lb_ref = oracle_thresholds(fibre_population(p, dtype=dtype, device="cpu"), 0.0, 0.05, n)
    np.testing.assert_array_equal(np.isnan(ub.cpu().numpy()), np.isnan(ub_ref))
    assert np.isfinite(ub_ref).sum() >= 6
    # identical decisions give identical brackets
    np.testing.assert_array_equal(ub.cpu().numpy(), ub_ref)
    np.testing.assert_array_equal(lb.cpu().numpy(), lb_ref)
    assert bool(((ub - lb) / ub)[torch.isfinite(ub)].max() < 0.01)
