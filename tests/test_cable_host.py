"""Host-side checks of CablePopulation.run on CPU: bad compartment indices and
raster settings are refused before any device work."""

import pytest
import torch

from dendra_gb300.cable import CablePopulation


def _pop():
    return CablePopulation([11, 21], 1.0, 10.0, dtype=torch.float64,
                           device="cpu").initialize(0.025)


def test_run_rejects_bad_indices_before_any_device_work():
    pop = _pop()
    with pytest.raises(ValueError, match="rec_idx out of range"):
        pop.run(5, rec_idx=11)
    with pytest.raises(ValueError, match="spk_idx out of range"):
        pop.run(5, spk_idx=[0, 21])
    with pytest.raises(ValueError, match="spk_idx2 out of range"):
        pop.run(5, spk_idx=0, spk_idx2=-2)
    with pytest.raises(ValueError, match="raster compartment out of range"):
        pop.run(5, raster=[0, 15])
    with pytest.raises(ValueError, match="1 to 4"):
        pop.run(5, raster=[0, 1, 2, 3, 4])
    with pytest.raises(ValueError, match="raster_cap"):
        pop.run(5, raster=[0], raster_cap=-1)
    assert pop.step_index == 0 and pop.t == 0.0  # nothing advanced


def test_run_needs_initialize():
    pop = CablePopulation([11], 1.0, 10.0, dtype=torch.float64, device="cpu")
    with pytest.raises(RuntimeError, match="initialized"):
        pop.run(5)
