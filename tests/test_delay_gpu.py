"""Interpolated delay transport on the GPU, through the C ABI.

Bit-exact against the reference's own outputs (``delay_{f64,f32}.npz``: the
ordered two-tap CPU op, its VJP and gather, the pure-torch transition with two
and three taps, and a 40-step rollout with autograd) and against the oracle on
larger rings with heavy collisions.
"""

import numpy as np
import pytest
import torch

import oracle
from dendra_gb300 import delays

pytestmark = pytest.mark.gpu

TAGS = [("f64", np.float64, torch.float64), ("f32", np.float32, torch.float32)]


def _t(a, dev, dt=None):
    t = torch.as_tensor(np.ascontiguousarray(a))
    return (t.to(dt) if dt is not None else t).to(dev)


@pytest.mark.parametrize("tag,npt,tdt", TAGS)
def test_ordered_enqueue_matches_reference_op(cuda, golden, tag, npt, tdt):
    z = golden(f"delay_{tag}.npz")
    q, w, g, gs, f = (_t(z[k], cuda, tdt) for k in ("queue", "w", "g", "g_src", "fraction"))
    lower, upper, gen, pre = (_t(z[k], cuda) for k in ("lower", "upper", "general_upper", "pre"))
    slot = int(z["slot"])
    out = delays.ordered_two_tap_enqueue(q, slot, w, g, f, lower, upper)
    np.testing.assert_array_equal(out.cpu().numpy(), z["op_edge"])
    out = delays.ordered_two_tap_enqueue_from_source(q, slot, w, gs, f, lower, upper, pre)
    np.testing.assert_array_equal(out.cpu().numpy(), z["op_src"])
    out = delays.ordered_two_tap_enqueue(q, slot, w, g, f, lower, gen)  # taps in two columns
    np.testing.assert_array_equal(out.cpu().numpy(), z["op_general"])
    ring = q.clone()
    payload = torch.empty(q.shape[1], dtype=tdt, device=cuda)
    delays.ordered_two_tap_enqueue_(ring, torch.tensor([slot], device=cuda), w, g, f, lower,
                                    upper, payload=payload)
    np.testing.assert_array_equal(ring.cpu().numpy(), z["op_edge"])
    np.testing.assert_array_equal(payload.cpu().numpy(), z["queue"][slot].astype(npt))
    assert delays.delay_status() == 0


@pytest.mark.parametrize("tag,npt,tdt", TAGS)
def test_vjp_and_gather_match_reference_op(cuda, golden, tag, npt, tdt):
    z = golden(f"delay_{tag}.npz")
    cot, w, g, gs, f = (_t(z[k], cuda, tdt) for k in ("cot", "w", "g", "g_src", "fraction"))
    lower, upper, pre = (_t(z[k], cuda) for k in ("lower", "upper", "pre"))
    off = int(z["slot"]) * int(z["width"])
    for name, gates, src in (("edge", g, None), ("src", gs, pre)):
        dw, dg, df = delays.delay_ring_two_tap_vjp(cot, off, w, gates, f, lower, upper, src)
        np.testing.assert_array_equal(dw.cpu().numpy(), z[f"vjp_{name}_dw"])
        np.testing.assert_array_equal(dg.cpu().numpy(), z[f"vjp_{name}_dg"])
        np.testing.assert_array_equal(df.cpu().numpy(), z[f"vjp_{name}_df"])
    lo, hi = delays.delay_ring_gather_two_tap(cot, off, lower, upper)
    np.testing.assert_array_equal(lo.cpu().numpy(), z["gather_lo"])
    np.testing.assert_array_equal(hi.cpu().numpy(), z["gather_hi"])


@pytest.mark.parametrize("tag,npt,tdt", TAGS)
def test_autograd_of_enqueue_equals_reference_adjoint(cuda, golden, tag, npt, tdt):
    z = golden(f"delay_{tag}.npz")
    q = _t(z["queue"], cuda, tdt).requires_grad_()
    w, gs, f = (_t(z[k], cuda, tdt).requires_grad_() for k in ("w", "g_src", "fraction"))
    lower, upper, pre = (_t(z[k], cuda) for k in ("lower", "upper", "pre"))
    slot = int(z["slot"])
    out = delays.ordered_two_tap_enqueue_from_source(q, slot, w, gs, f, lower, upper, pre)
    cot = _t(z["cot"], cuda, tdt)
    (out * cot).sum().backward()
    np.testing.assert_array_equal(w.grad.cpu().numpy(), z["vjp_src_dw"])
    np.testing.assert_array_equal(gs.grad.cpu().numpy(), z["vjp_src_dg"])
    np.testing.assert_array_equal(f.grad.cpu().numpy(), z["vjp_src_df"])
    expect = z["cot"].astype(npt).copy()
    expect[slot] = 0
    np.testing.assert_array_equal(q.grad.cpu().numpy(), expect)


@pytest.mark.parametrize("tag,npt,tdt", TAGS)
def test_three_tap_transition_and_gradients_match_reference(cuda, golden, tag, npt, tdt):
    z = golden(f"delay_{tag}.npz")
    q = _t(z["queue"], cuda, tdt)
    w, g, c = (_t(z[k], cuda, tdt).requires_grad_() for k in ("w", "g", "coeff3"))
    off3, post = _t(z["offsets3"], cuda), _t(z["post"], cuda)
    D, W = int(z["depth"]), int(z["width"])
    tr = delays.dense_interpolated_delay_transition(
        q, torch.tensor([int(z["slot"])], device=cuda), torch.zeros(1, dtype=torch.int64,
                                                                    device=cuda),
        w, g, None, None, post_idx=post, depth=D, width=W, taps=3, sigma=float(z["sigma"]),
        delay_taps=(off3, c))
    np.testing.assert_array_equal(tr.queue.detach().cpu().numpy(), z["three_tap"])
    assert int(tr.slot.item()) == (int(z["slot"]) + 1) % D
    (tr.queue * _t(z["cot"], cuda, tdt)).sum().backward()
    np.testing.assert_array_equal(w.grad.cpu().numpy(), z["three_dw"])
    np.testing.assert_array_equal(g.grad.cpu().numpy(), z["three_dg"])
    np.testing.assert_array_equal(c.grad.cpu().numpy(), z["three_dc"])


def _rollout_inputs(z, cuda, tdt, requires_grad):
    w = _t(z["r_w"], cuda, tdt).requires_grad_(requires_grad)
    gates = _t(z["r_gates"], cuda, tdt).requires_grad_(requires_grad)
    dl = _t(z["r_delays"], cuda, tdt).requires_grad_(requires_grad)
    q0 = _t(z["r_queue0"], cuda, tdt).requires_grad_(requires_grad)
    return w, gates, dl, q0


@pytest.mark.parametrize("tag,npt,tdt", TAGS)
def test_per_step_transitions_match_reference_rollout(cuda, golden, tag, npt, tdt):
    """The reference's 40-step loop, step by step through the transition with
    autograd: payloads, final ring and every gradient bit for bit (delays
    within rounding of the reference's per-step division by dt)."""
    z = golden(f"delay_{tag}.npz")
    D, W = int(z["r_depth"]), int(z["r_width"])
    w, gates, dl, q0 = _rollout_inputs(z, cuda, tdt, True)
    post, pre = _t(z["r_post"], cuda), _t(z["r_pre"], cuda)
    dt = torch.tensor([float(z["dt"])], dtype=tdt, device=cuda)
    queue, slot = q0, torch.tensor([int(z["r_slot0"])], device=cuda)
    gs = torch.zeros(1, dtype=torch.int64, device=cuda)
    pays = []
    for k in range(gates.shape[0]):
        pays.append(queue.index_select(0, slot).squeeze(0))
        queue, slot, gs, _ = delays.dense_interpolated_delay_transition(
            queue, slot, gs, w, gates[k].index_select(0, pre), dl, dt, post_idx=post,
            depth=D, width=W, taps=2, sigma=0.0)
    pay = torch.stack(pays)
    np.testing.assert_array_equal(pay.detach().cpu().numpy(), z["r_payload"])
    np.testing.assert_array_equal(queue.detach().cpu().numpy(), z["r_final"])
    loss = (pay * _t(z["r_cpay"], cuda, tdt)).sum() + (queue * _t(z["r_cfin"], cuda, tdt)).sum()
    loss.backward()
    np.testing.assert_array_equal(w.grad.cpu().numpy(), z["r_dw"])
    np.testing.assert_array_equal(gates.grad.cpu().numpy(), z["r_dgates"])
    np.testing.assert_array_equal(q0.grad.cpu().numpy(), z["r_dqueue0"])
    tol = 1e-12 if tag == "f64" else 2e-5
    ref = z["r_ddelays"]
    np.testing.assert_allclose(dl.grad.cpu().numpy(), ref, rtol=tol, atol=tol * np.abs(ref).max())


@pytest.mark.parametrize("tag,npt,tdt", TAGS)
def test_rollout_in_one_launch_matches_reference(cuda, golden, tag, npt, tdt):
    z = golden(f"delay_{tag}.npz")
    D, W = int(z["r_depth"]), int(z["r_width"])
    w, gates, dl, q0 = _rollout_inputs(z, cuda, tdt, True)
    post, pre = _t(z["r_post"], cuda), _t(z["r_pre"], cuda)
    dt = torch.tensor([float(z["dt"])], dtype=tdt, device=cuda)
    off, frac = delays.delay_interpolation(dl, dt, dtype=tdt, taps=2, sigma=0.0)
    lower, upper = delays.transition_addresses(off, post, D, W)
    pay, fin = delays.two_tap_rollout(q0, int(z["r_slot0"]), w, gates, frac, lower, upper, pre)
    np.testing.assert_array_equal(pay.detach().cpu().numpy(), z["r_payload"])
    np.testing.assert_array_equal(fin.detach().cpu().numpy(), z["r_final"])
    loss = (pay * _t(z["r_cpay"], cuda, tdt)).sum() + (fin * _t(z["r_cfin"], cuda, tdt)).sum()
    loss.backward()
    np.testing.assert_array_equal(w.grad.cpu().numpy(), z["r_dw"])
    np.testing.assert_array_equal(gates.grad.cpu().numpy(), z["r_dgates"])
    np.testing.assert_array_equal(q0.grad.cpu().numpy(), z["r_dqueue0"])
    tol = 1e-12 if tag == "f64" else 2e-5
    ref = z["r_ddelays"]
    np.testing.assert_allclose(dl.grad.cpu().numpy(), ref, rtol=tol, atol=tol * np.abs(ref).max())


def _network_case(seed, depth, width, E, n_src, steps, npt, chained=False):
    """Connections into few targets (heavy collisions) with delays wrapping the
    ring; width == E: one connection per target slot (the register path);
    chained: one per slot with both taps clear of the delivered row (the
    direct kernels)."""
    rng = np.random.default_rng(seed)
    post = rng.permutation(E) if width == E else rng.integers(0, width, E)
    pre = rng.integers(0, n_src, E)
    pos = rng.uniform(1.0, depth - 1.0 if chained else depth + 0.9, E)
    off = np.floor(pos).astype(np.int64)
    frac = (pos - off).astype(npt)
    lower = (off % depth) * width + post
    upper = (lower + width) % (depth * width)
    w = rng.standard_normal(E).astype(npt)
    gates = rng.random((steps, n_src)).astype(npt)
    gates[rng.random((steps, n_src)) < 0.7] = 0
    q0 = rng.standard_normal((depth, width)).astype(npt)
    return post, pre, frac, lower, upper, w, gates, q0


@pytest.mark.parametrize("depth,width,chained", [(33, 700, False), (33, 5000, False),
                                                (600, 700, False), (33, 5000, True),
                                                (600, 5000, True)])
@pytest.mark.parametrize("tag,npt,tdt", TAGS)
def test_window_equals_single_steps_and_oracle(cuda, tag, npt, tdt, depth, width, chained):
    """Shared-memory ring (depth 33), the ring in place in HBM (depth 600) and
    the direct kernels (chained)."""
    E, n_src, steps = 5000, 97, 70
    post, pre, frac, lower, upper, w, gates, q0 = _network_case(5, depth, width, E, n_src,
                                                                steps, npt, chained)
    T = lambda a, dt=tdt: _t(a, cuda, dt)  # noqa: E731
    tl, tu, tp = T(lower, None), T(upper, None), T(pre, None)
    pay, fin = delays.two_tap_rollout(T(q0), 4, T(w), T(gates), T(frac), tl, tu, tp)
    ring = T(q0).clone()
    one = torch.empty(steps, width, dtype=tdt, device=cuda)
    for k in range(steps):
        delays.ordered_two_tap_enqueue_(ring, (4 + k) % depth, T(w), T(gates[k]), T(frac), tl,
                                        tu, tp, payload=one[k])
    torch.testing.assert_close(fin, ring, rtol=0, atol=0)
    torch.testing.assert_close(pay, one, rtol=0, atol=0)
    ofin, opay = oracle.two_tap_rollout(q0, 4, w, gates, frac, lower, upper, pre_idx=pre)
    np.testing.assert_array_equal(fin.cpu().numpy(), ofin)
    np.testing.assert_array_equal(pay.cpu().numpy(), opay)
    assert delays.delay_status() == 0
    assert bool(delays.two_tap_plan(depth, width, tl, tu, tp, n_src).rollout.flags
                & delays.CHAINED) == chained


@pytest.mark.parametrize("width,chained", [(300, False), (2000, False), (2000, True)])
@pytest.mark.parametrize("with_pre", [True, False])
@pytest.mark.parametrize("tag,npt,tdt", TAGS)
def test_rollout_adjoint_matches_oracle(cuda, tag, npt, tdt, with_pre, width, chained,
                                        monkeypatch):
    depth, E, n_src, steps = 21, 2000, 41, 50
    post, pre, frac, lower, upper, w, gates, q0 = _network_case(9, depth, width, E, n_src,
                                                                steps, npt, chained)
    if not with_pre:
        gates = np.ascontiguousarray(gates[:, pre])
    rng = np.random.default_rng(10)
    cpay = rng.standard_normal((steps, width)).astype(npt)
    cfin = rng.standard_normal((depth, width)).astype(npt)
    T = lambda a, dt=tdt: _t(a, cuda, dt)  # noqa: E731
    # small chunks: the reverse sweep is carried across several launches
    monkeypatch.setattr(delays, "_SCRATCH_BYTES", 7 * E * np.dtype(npt).itemsize)
    tw, tg, tf, tq = (T(a).requires_grad_() for a in (w, gates, frac, q0))
    pay, fin = delays.two_tap_rollout(tq, 3, tw, tg, tf, T(lower, None), T(upper, None),
                                      T(pre, None) if with_pre else None)
    ((pay * T(cpay)).sum() + (fin * T(cfin)).sum()).backward()
    R0, dw, dg, df = oracle.two_tap_rollout_vjp(cfin, 3, w, gates, frac, lower, upper, cpay,
                                                pre_idx=pre if with_pre else None)
    np.testing.assert_array_equal(tq.grad.cpu().numpy(), R0)
    np.testing.assert_array_equal(tw.grad.cpu().numpy(), dw)
    np.testing.assert_array_equal(tg.grad.cpu().numpy(), dg)
    np.testing.assert_array_equal(tf.grad.cpu().numpy(), df)


@pytest.mark.parametrize("chained", [False, True])
@pytest.mark.parametrize("tag,npt,tdt", TAGS)
def test_rollout_from_an_empty_ring(cuda, tag, npt, tdt, chained):
    depth, width, E, n_src, steps = 40, 3000, 3000, 50, 90
    post, pre, frac, lower, upper, w, gates, _ = _network_case(13, depth, width, E, n_src, steps,
                                                               npt, chained)
    T = lambda a, dt=tdt: _t(a, cuda, dt)  # noqa: E731
    args = (T(w), T(gates), T(frac), T(lower, None), T(upper, None), T(pre, None))
    zeros = torch.zeros(depth, width, dtype=tdt, device=cuda)
    pay0, fin0 = delays.two_tap_rollout(zeros, 7, *args)
    pay1, fin1 = delays.two_tap_rollout(None, 7, *args, depth=depth, width=width)
    torch.testing.assert_close(pay1, pay0, rtol=0, atol=0)
    torch.testing.assert_close(fin1, fin0, rtol=0, atol=0)
    tw = args[0].clone().requires_grad_()
    pay, _ = delays.two_tap_rollout(None, 7, tw, *args[1:], depth=depth, width=width)
    pay.sum().backward()
    cpay = np.ones((steps, width), npt)
    _, dw, _, _ = oracle.two_tap_rollout_vjp(np.zeros((depth, width), npt), 7, w, gates, frac,
                                             lower, upper, cpay, pre_idx=pre)
    np.testing.assert_array_equal(tw.grad.cpu().numpy(), dw)


def test_device_slot_outside_the_ring_is_reported(cuda):
    q = torch.randn(5, 8, dtype=torch.float64, device=cuda)
    before = q.clone()
    v = torch.ones(3, dtype=torch.float64, device=cuda)
    a = torch.tensor([1, 9, 17], device=cuda)
    delays.delay_status()
    delays.ordered_two_tap_enqueue_(q, torch.tensor([7], device=cuda), v, v, v * 0.5, a, a + 8)
    assert delays.delay_status() == delays.ERR_SLOT
    torch.testing.assert_close(q, before, rtol=0, atol=0)
    with pytest.raises(RuntimeError, match="slot is outside the delivery ring"):
        delays.ordered_two_tap_enqueue_(q, 5, v, v, v, a, a)
    with pytest.raises(RuntimeError, match="address is outside the delivery ring"):
        delays.ordered_two_tap_enqueue_(q, 0, v, v, v, a, a + 100)


@pytest.mark.parametrize("taps", [2, 3])
@pytest.mark.parametrize("tag,npt,tdt", TAGS)
def test_reference_transition_cases(cuda, golden, tag, npt, tdt, taps):
    """The inputs of the reference's own transition tests (collisions, a wrap
    past the ring's end, sub-step delays clamped to one step): queue, slot,
    step and every gradient as the reference computes them."""
    z = golden(f"delay_{tag}.npz")
    q = (torch.arange(18).reshape(3, 6).t() / 10).to(tdt).contiguous().to(cuda).requires_grad_()
    w = torch.tensor([0.5, 1.0, -2.0, 3.0, 0.0], dtype=tdt, device=cuda, requires_grad=True)
    g = torch.tensor([-0.2, 0.4, 0.5, 1.0, 2.0], dtype=tdt, device=cuda, requires_grad=True)
    d = torch.tensor([0.02, 0.1, 0.23, 0.2, 0.6], dtype=tdt, device=cuda, requires_grad=True)
    L = lambda v: torch.tensor(v, dtype=torch.int64, device=cuda)  # noqa: E731
    tr = delays.dense_interpolated_delay_transition(
        q, L([4]), L([17]), w, g, d, torch.tensor(0.1, dtype=tdt, device=cuda),
        post_idx=L([1, 1, 2, 0, 1]), depth=6, width=3, taps=taps, sigma=0.5)
    # two taps: bit for bit.  Three taps: the Gaussian weights come from
    # torch's softmax on the device, whose exponential rounds differently from
    # the CPU's by an ulp (with the same weights the kernel is bit-exact:
    # test_three_tap_transition_and_gradients_match_reference)
    exact = taps == 2
    ulp = dict(rtol=4e-16, atol=4e-16) if tag == "f64" else dict(rtol=3e-7, atol=3e-7)
    check = (np.testing.assert_array_equal if exact else
             (lambda a, b: np.testing.assert_allclose(a, b, **ulp)))
    check(tr.queue.detach().cpu().numpy(), z[f"pure{taps}_queue"])
    assert int(tr.slot.item()) == z[f"pure{taps}_slot"]
    assert int(tr.global_step.item()) == z[f"pure{taps}_step"]
    (tr.queue * _t(z[f"pure{taps}_cot"], cuda, tdt)).sum().backward()
    np.testing.assert_array_equal(q.grad.cpu().numpy(), z[f"pure{taps}_dq"])
    check(w.grad.cpu().numpy(), z[f"pure{taps}_dw"])
    check(g.grad.cpu().numpy(), z[f"pure{taps}_dg"])
    tol = 1e-12 if tag == "f64" else 1e-5
    np.testing.assert_allclose(d.grad.cpu().numpy(), z[f"pure{taps}_dd"], rtol=tol, atol=tol)
    assert d.grad[0].item() == 0  # a sub-step delay is clamped to one step


@pytest.mark.parametrize("taps", [2, 3])
def test_empty_connections_clear_the_due_row(cuda, taps):
    """The reference's empty-transition case: no connections, depth 1."""
    queue = torch.tensor([[1.0, 2.0]], dtype=torch.float64, device=cuda)
    empty = torch.empty(0, dtype=torch.float64, device=cuda)
    slot = torch.zeros(1, dtype=torch.int64, device=cuda)
    tr = delays.dense_interpolated_delay_transition(
        queue, slot, slot, empty, empty, empty, torch.tensor(0.1, device=cuda),
        post_idx=torch.empty(0, dtype=torch.int64, device=cuda), depth=1, width=2, taps=taps,
        sigma=0.5)
    torch.testing.assert_close(tr.queue, torch.zeros_like(queue), rtol=0, atol=0)
    assert int(tr.slot.item()) == 0 and int(tr.global_step.item()) == 1
