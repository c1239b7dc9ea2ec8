"""Interpolated delay transport: the oracle against the reference's own outputs,
the column plans and the host-side checks (CPU only).

The fixtures ``delay_{f64,f32}.npz`` hold outputs of the reference's ordered
two-tap CPU operators (networks/_two_tap_enqueue_cpu.cpp) and of its pure-torch
dense_interpolated_delay_transition with autograd (networks/_event_delivery.py:229-308).
"""

import numpy as np
import pytest
import torch

import oracle
from dendra_gb300 import delays

TAGS = [("f64", np.float64), ("f32", np.float32)]


def _fraction(z, dt):
    pos = np.maximum(z["r_delays"].astype(dt) / dt(z["dt"]), dt(1))
    lo = np.floor(pos)
    return lo.astype(np.int64), (pos - lo).astype(dt)


@pytest.mark.parametrize("tag,dt", TAGS)
def test_oracle_two_tap_enqueue_matches_reference_op(golden, tag, dt):
    z = golden(f"delay_{tag}.npz")
    q, f, w = z["queue"].astype(dt), z["fraction"].astype(dt), z["w"].astype(dt)
    got, pay = oracle.two_tap_enqueue(q, z["slot"], w, z["g"].astype(dt), f, z["lower"],
                                      z["upper"])
    np.testing.assert_array_equal(got, z["op_edge"])
    np.testing.assert_array_equal(pay, q[int(z["slot"])])
    got, _ = oracle.two_tap_enqueue(q, z["slot"], w, z["g_src"].astype(dt), f, z["lower"],
                                    z["upper"], pre_idx=z["pre"])
    np.testing.assert_array_equal(got, z["op_src"])
    got, _ = oracle.two_tap_enqueue(q, z["slot"], w, z["g"].astype(dt), f, z["lower"],
                                    z["general_upper"])
    np.testing.assert_array_equal(got, z["op_general"])


@pytest.mark.parametrize("tag,dt", TAGS)
def test_oracle_two_tap_vjp_matches_reference_op(golden, tag, dt):
    z = golden(f"delay_{tag}.npz")
    cot, f, w = z["cot"].astype(dt), z["fraction"].astype(dt), z["w"].astype(dt)
    off = int(z["slot"]) * int(z["width"])
    for name, g, pre in (("edge", z["g"], None), ("src", z["g_src"], z["pre"])):
        dw, dg, df = oracle.two_tap_vjp(cot, off, w, g.astype(dt), f, z["lower"], z["upper"], pre)
        np.testing.assert_array_equal(dw, z[f"vjp_{name}_dw"])
        np.testing.assert_array_equal(dg, z[f"vjp_{name}_dg"])
        np.testing.assert_array_equal(df, z[f"vjp_{name}_df"])


@pytest.mark.parametrize("tag,dt", TAGS)
def test_oracle_three_tap_matches_reference_transition(golden, tag, dt):
    z = golden(f"delay_{tag}.npz")
    got, _ = oracle.three_tap_enqueue(z["queue"].astype(dt), z["slot"], z["w"].astype(dt),
                                      z["g"].astype(dt), z["coeff3"].astype(dt), z["offsets3"],
                                      z["post"])
    np.testing.assert_array_equal(got, z["three_tap"])


@pytest.mark.parametrize("tag,dt", TAGS)
def test_oracle_rollout_matches_reference_autograd(golden, tag, dt):
    """40 steps: payloads, final ring and the reverse sweep's gradients equal the
    reference's autograd through its per-step transition, bit for bit."""
    z = golden(f"delay_{tag}.npz")
    D, W = int(z["r_depth"]), int(z["r_width"])
    lo, frac = _fraction(z, dt)
    lower = (lo % D) * W + z["r_post"]
    upper = (lower + W) % (D * W)
    args = (z["r_w"].astype(dt), z["r_gates"].astype(dt), frac, lower, upper)
    fin, pay = oracle.two_tap_rollout(z["r_queue0"].astype(dt), z["r_slot0"], *args,
                                      pre_idx=z["r_pre"])
    np.testing.assert_array_equal(pay, z["r_payload"])
    np.testing.assert_array_equal(fin, z["r_final"])
    R0, dw, dg, df = oracle.two_tap_rollout_vjp(z["r_cfin"].astype(dt), z["r_slot0"], *args,
                                                z["r_cpay"].astype(dt), pre_idx=z["r_pre"])
    np.testing.assert_array_equal(R0, z["r_dqueue0"])
    np.testing.assert_array_equal(dw, z["r_dw"])
    np.testing.assert_array_equal(dg, z["r_dgates"])
    # d fraction / d delay = 1/dt: the reference divides every step's share,
    # the rollout divides the sum once (a rounding-order difference only)
    ddel = df / dt(z["dt"])
    tol = 1e-12 if tag == "f64" else 2e-5
    np.testing.assert_allclose(ddel, z["r_ddelays"], rtol=tol, atol=tol * np.abs(ddel).max())


def test_plan_lists_each_column_in_ascending_edge_order():
    rng = np.random.default_rng(3)
    depth, width, E = 6, 11, 300
    post = torch.as_tensor(rng.integers(0, width, E))
    off = torch.as_tensor(rng.integers(1, depth + 2, E))
    lower, upper = delays.transition_addresses(off, post, depth, width)
    plan = delays.TapPlan(depth, width, lower, upper)
    assert plan.consistent
    ptr, edge = plan.col_ptr.numpy(), plan.col_edge.numpy()
    for c in range(width):
        members = edge[ptr[c]:ptr[c + 1]]
        np.testing.assert_array_equal(members, np.flatnonzero(post.numpy() == c))
    general = torch.as_tensor(rng.integers(0, depth * width, E))
    plan = delays.TapPlan(depth, width, lower, general)
    assert not plan.consistent
    for c in range(width):
        got = plan.upper_edge.numpy()[plan.upper_ptr[c]:plan.upper_ptr[c + 1]]
        np.testing.assert_array_equal(got, np.flatnonzero(general.numpy() % width == c))
    pre = torch.as_tensor(rng.integers(0, 7, E))
    plan = delays.TapPlan(depth, width, lower, upper, pre, 7)
    for s in range(7):
        got = plan.src_edge.numpy()[plan.src_ptr[s]:plan.src_ptr[s + 1]]
        np.testing.assert_array_equal(got, np.flatnonzero(pre.numpy() == s))


def test_rollout_plan_rows_and_source_positions():
    rng = np.random.default_rng(4)
    depth, width, E = 9, 40, 120
    post = torch.as_tensor(rng.integers(0, width - 3, E))  # three empty columns
    off = torch.as_tensor(rng.integers(1, depth + 1, E))
    pre = torch.as_tensor(rng.integers(0, 5, E))
    lower, upper = delays.transition_addresses(off, post, depth, width)
    plan = delays.TapPlan(depth, width, lower, upper, pre, 5)
    rp = delays.RolloutPlan(plan, lower, upper)
    edge = plan.col_edge.numpy()
    np.testing.assert_array_equal(rp.lo_row.numpy(), lower.numpy()[edge] // width)
    np.testing.assert_array_equal(rp.hi_row.numpy(), upper.numpy()[edge] // width)
    np.testing.assert_array_equal(rp.hi_row.numpy(), (rp.lo_row.numpy() + 1) % depth)
    assert rp.flags == 0  # several edges per column
    pos = np.empty(E, np.int64)
    pos[edge] = np.arange(E)
    for s_ in range(5):
        got = rp.src_pos.numpy()[rp.src_ptr[s_]:rp.src_ptr[s_ + 1]]
        np.testing.assert_array_equal(got, pos[np.flatnonzero(pre.numpy() == s_)])
    one = torch.as_tensor(rng.permutation(width))
    lo1, up1 = delays.transition_addresses(off[:width], one, depth, width)
    assert delays.RolloutPlan(delays.TapPlan(depth, width, lo1, up1), lo1, up1).flags == \
        delays.ONE_EDGE


def test_plan_rejects_addresses_and_sources_out_of_range():
    lower = torch.tensor([0, 5, 12])
    with pytest.raises(RuntimeError, match="outside the delivery ring"):
        delays.TapPlan(3, 4, lower, torch.tensor([1, 2, 3]))
    ok = torch.tensor([0, 5, 11])
    with pytest.raises(IndexError, match="source index is out of range"):
        delays.TapPlan(3, 4, ok, ok, torch.tensor([0, 2, 3]), 3)


def test_host_checks_reject_non_cuda_inputs():
    q = torch.zeros(4, 3, dtype=torch.float64)
    v = torch.zeros(2, dtype=torch.float64)
    i = torch.zeros(2, dtype=torch.int64)
    with pytest.raises(RuntimeError, match="CUDA float32 or float64 matrix"):
        delays.ordered_two_tap_enqueue(q, 0, v, v, v, i, i)


def test_delay_interpolation_positions():
    d = torch.tensor([0.01, 0.025, 0.0375, 0.1], dtype=torch.float64)
    dt = torch.tensor([0.025], dtype=torch.float64)
    off, frac = delays.delay_interpolation(d, dt, dtype=torch.float64, taps=2, sigma=0.0)
    np.testing.assert_array_equal(off.numpy(), [1, 1, 1, 4])
    np.testing.assert_allclose(frac.numpy(), [0.0, 0.0, 0.5, 0.0], atol=1e-15)
    off3, c3 = delays.delay_interpolation(d, dt, dtype=torch.float64, taps=3, sigma=0.5)
    np.testing.assert_array_equal(off3[:, 1].numpy(), off.numpy())
    np.testing.assert_allclose(c3.sum(-1).numpy(), 1.0, rtol=1e-15)
