"""The 64-cable float64 workload at its stated size and with its stated outputs.

64 unbranched HH cables x 101 compartments (L = 1000 um, dx = 10 um, diam
1 um, Ra 100 ohm cm), float64, backward Euler + cnexp at dt 0.025 ms for
2000 steps, a 1 ms somatic current clamp at 5 ms of U[0.05, 0.5] nA per cable.
Outputs, as the reference's Recorder(("v",)) (callbacks.py:522) and Raster /
threshold_crossing (callbacks.py:2114, _threshold_callbacks.py:50-53) give
them: the full (2001, 64, 101) voltage trace and every step of an upward
0 mV crossing.  Both come out of one persistent launch (dgb_cable_run with
trace_all and the raster) and are compared with the float64 oracle:
traces within 1e-7 mV, spike steps identical.
"""

import numpy as np
import pytest
import torch

import oracle
from dendra_gb300.workloads import C1_STEPS, cable_population_c1
from tests._cases import golden_cable_population

pytestmark = pytest.mark.gpu

F64_MV = 1e-7
CHECKS = [0, 5, 50, -5]  # soma, Raster's default node_check [5, -5], the middle


def _oracle_c1(pop, steps, checks):
    p = pop.problem_dict()
    kk = np.asarray(pop.n_comp)
    idx = np.array([[c % k for c in checks] for k in kk], dtype=np.int32)
    _, _, _, _, extra = oracle.cable_run(p, steps, record_all=True, raster=idx,
                                         raster_cap=256)
    return extra


def test_64_cable_run_full_traces_and_every_spike_step(cuda):
    pop = cable_population_c1(device=cuda)
    assert pop.B == 64 and set(pop.n_comp) == {101} and pop.dtype == torch.float64
    ref = _oracle_c1(cable_population_c1(device="cpu"), C1_STEPS, CHECKS)
    res = pop.run(C1_STEPS, record_all=True, raster=CHECKS, raster_cap=256, spk_thr=0.0)
    pop.check_status()
    tr = res.trace_all.cpu().numpy()
    assert tr.shape == (C1_STEPS + 1, 64 * 101)
    assert np.isfinite(tr).all()
    err = np.abs(tr - ref["trace_all"]).max()
    print(f"64 cables: max |dV| GPU vs float64 oracle over all compartments and steps {err:.3e}")
    assert err <= F64_MV
    rs = res.raster
    assert not rs.overflow
    np.testing.assert_array_equal(rs.count.cpu().numpy(), ref["rast_count"])
    np.testing.assert_array_equal(rs.steps.cpu().numpy(), ref["rast_steps"])
    np.testing.assert_array_equal(rs.below.cpu().numpy(), ref["rast_below"])
    # the raster agrees with the crossings read off the recorded traces
    v = tr.reshape(C1_STEPS + 1, 64, 101)
    for c in range(64):
        for q, node in enumerate(CHECKS):
            above = v[:, c, node] >= 0.0
            steps = np.nonzero(above[1:] & ~above[:-1])[0] + 1
            np.testing.assert_array_equal(rs.spike_steps(c, q), steps)
    # the stimulus drives most cables to fire, several of them repeatedly
    counts = rs.count.cpu().numpy()[:, 0]
    assert (counts > 0).sum() >= 32


def test_raster_and_trace_continue_across_runs(cuda):
    """Two runs with the raster state carried over equal one long run."""
    a = cable_population_c1(device=cuda, n_cables=16)
    b = cable_population_c1(device=cuda, n_cables=16)
    ra = a.run(1200, record_all=True, raster=CHECKS, raster_cap=64)
    rb1 = b.run(600, record_all=True, raster=CHECKS, raster_cap=64)
    rb2 = b.run(600, record_all=True, raster_state=rb1.raster)
    assert torch.equal(ra.trace_all[:601], rb1.trace_all)
    assert torch.equal(ra.trace_all[600:], rb2.trace_all)
    assert torch.equal(ra.raster.count, rb2.raster.count)
    assert torch.equal(ra.raster.steps, rb2.raster.steps)


def test_raster_overflow_is_reported(cuda):
    pop = cable_population_c1(device=cuda, n_cables=8)
    res = pop.run(C1_STEPS, raster=[0], raster_cap=0)
    counts = res.raster.count.cpu().numpy()
    assert counts.max() > 0
    assert res.raster.overflow


def test_full_trace_matches_reference_recording(cuda, golden):
    """The reference's own Recorder run (hh_cable_f64.npz, 3 cables x 101
    compartments, 800 steps) against the full trace at its recorded
    compartments."""
    g = golden("hh_cable_f64.npz")
    pop = golden_cable_population(g, torch.float64, cuda)
    res = pop.run(int(g["steps"]), record_all=True)
    B, K = int(g["B"]), int(g["K"])
    tr = res.trace_all.cpu().numpy().reshape(-1, B, K)[:, :, g["trace_comps"]]
    assert np.abs(tr - g["v_trace"]).max() < F64_MV
    np.testing.assert_allclose(pop.v.cpu().numpy().reshape(B, K), g["v_final"], rtol=0,
                               atol=F64_MV)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("split", [None, (128, 64), (128, 0), (0, 0)])
def test_lane_split_matches_oracle(cuda, dtype, split):
    """Every Thomas/PCR split (8, 16 or 32 lanes per cable) on a ragged
    population with the full trace and a raster, against the oracle."""
    from tests._cases import as_f64, synthetic_population

    pop = synthetic_population(31, 96, 1, 301, dtype, cuda, intra=True)
    pop.lanes_split = split
    p = pop.problem_dict()
    ref64 = as_f64(p)
    steps = 400
    kk = np.asarray(pop.n_comp)
    checks = [0, -1]
    idx = np.array([[c % k for c in checks] for k in kk], dtype=np.int32)
    _, _, _, _, ref = oracle.cable_run(ref64, steps, gate_f32=dtype == torch.float32,
                                       record_all=True, raster=idx, raster_cap=32)
    res = pop.run(steps, record_all=True, raster=checks, raster_cap=32)
    pop.check_status()
    tr = res.trace_all.double().cpu().numpy()
    err = np.abs(tr - ref["trace_all"]).max()
    tol = 1e-8 if dtype == torch.float64 else 1e-3
    print(f"split {split} {dtype}: {err:.3e} mV")
    assert err <= tol
    np.testing.assert_array_equal(res.raster.count.cpu().numpy(), ref["rast_count"])
    np.testing.assert_array_equal(res.raster.steps.cpu().numpy(), ref["rast_steps"])
