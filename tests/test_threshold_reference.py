"""Threshold search pinned to the reference's own Thresholder.

thresholds.npz records the reference Thresholder (bound fixing by doubling,
bisection to rtol 1 %, activity = a 0 mV rising edge at compartment 5 or -5)
on twelve unbranched HH cables under a cathodic point-source pulse, float64.
The same decisions give the same brackets bit for bit, including the lanes
whose bound fixing gave up (NaN): the oracle's bisection on the CPU and the
GPU Thresholder must reproduce them exactly.
"""

import numpy as np
import pytest
import torch

from dendra_gb300.cable import CablePopulation
from tests._cases import oracle_thresholds


def cables(g, device):
    B, K = int(g["B"]), int(g["K"])
    pop = CablePopulation([K] * B, torch.as_tensor(g["diam"]), float(g["dx"]), rhoa=100.0,
                          celsius=6.3, v_init=-65.0, dtype=torch.float64, device=device)
    pop.set_extracellular(torch.as_tensor(g["field"]).reshape(-1),
                          torch.zeros(B, dtype=torch.float64), 0.0, float(g["pw"]))
    return pop.initialize(float(g["dt"]))


def _steps(g):
    return int(round(float(g["tstop"]) / float(g["dt"])))


def test_oracle_bisection_matches_reference(golden):
    g = golden("thresholds.npz")
    K = int(g["K"])
    ub, lb = oracle_thresholds(cables(g, "cpu"), float(g["lb0"]), float(g["ub0"]), _steps(g),
                               rtol=float(g["rtol"]), spk=(5, K - 5))
    assert np.isfinite(g["ub"]).sum() >= 8 and np.isnan(g["ub"]).sum() >= 1
    np.testing.assert_array_equal(ub, g["ub"])
    np.testing.assert_array_equal(lb, g["lb"])


@pytest.mark.gpu
def test_gpu_thresholder_matches_reference(cuda, golden):
    from dendra_gb300.threshold import Thresholder

    g = golden("thresholds.npz")
    th = Thresholder(cables(g, cuda), lb=float(g["lb0"]), ub=float(g["ub0"]),
                     rtol=float(g["rtol"]), compartments=(5, -5))
    ub, lb = th.calculate_thresholds(_steps(g))
    np.testing.assert_array_equal(ub.cpu().numpy(), g["ub"])
    np.testing.assert_array_equal(lb.cpu().numpy(), g["lb"])
