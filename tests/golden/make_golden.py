"""Generate the golden fixtures in tests/golden/ by running the reference.

The reference (Dendra v0.30.1) is a Python package; this script imports it
from its source tree with the small stub/shim set in ``refshim/`` (empty
pandas/natsort/h5py/dask/matplotlib stand-ins and three torch.library
compatibility shims) and records its outputs on seeded inputs:

  hh_cable_{f64,f32}.npz   Unmyelinated + hh + bwd_euler_ub + somatic mono_rect
                           (64-cable workload geometry: diam 1 um, L 1000 um, dx 10 um)
  hh_extra_{f64,f32}.npz   Unmyelinated + hh with extra=(point field, mono_rect)
  tridiag.npz              pcr_solve_t / pcr_solve_parallel_t on random systems
  rates.npz                exprelr, _bounded_phi1, _linear_exact_step, HH rates
  dhs.npz                  build_morphology / build_dhs_layers plans and the
                           dense-matrix solve of the reference's DHS parity test
  events.npz               dense_fixed_delay_transition ring sequence, Exp2Syn
                           factor and the NetCon delay-rounding known answers
  adjoint_f64.npz          reference autograd gradients (gnabar, gkbar, gl, Ra) of
                           a somatic-trace MSE through the CPU cable update
  block3.npz               block_pcr_solve_t on 3x3 block-tridiagonal systems
  delay_{f64,f32}.npz      interpolated delays: the reference's ordered two-tap
                           CPU op and its VJP/gather ops (compiled from the
                           reference's _two_tap_enqueue_cpu.cpp by
                           torch.utils.cpp_extension into oracle/_ref/), the
                           pure-torch dense_interpolated_delay_transition (two
                           and three taps) and a 40-step rollout with autograd
  netstim_{f64,f32}.npz    NetStim renewal: netstim_initial_state and 600 steps of
                           netstim_renewal with supplied unit-exponential draws
  network_points.npz       a 16-cell Network of single-compartment HH cells with
                           Exp2Syn synapses, periodic NetStim drive and all-to-all
                           NetCons with delays, run through Network.run (CPU)
  netcon_tapes.npz         the bit-pack known-answer tapes: fan-in/out across
                           the ring wrap and the 63-bit word boundary
  thresholds.npz           the reference Thresholder's brackets on twelve HH
                           cables under a point-source pulse

Usage (in a container that holds the reference source):

    PYTHONPATH=<dendra-src>:tests/golden/refshim python tests/golden/make_golden.py

The fixtures are committed; tests never import the reference.
"""

from __future__ import annotations

import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))


def _ref():
    import dendra as dn  # noqa: F401

    return dn


def hh_cable(dtype, tag):
    dn = _ref()
    from dendra.models.mod import hh

    B, steps, dt = 3, 800, 0.025
    g = torch.Generator().manual_seed(1234)
    amp_na = 0.05 + 0.45 * torch.rand(B, generator=g, dtype=torch.float64)
    amp_na[0] = 0.5  # at least one cable spikes
    amp_na[2] = 0.02  # and one stays subthreshold
    with dn.ctx(JIT=0):
        # rhoa must be given to the constructor: the workspace reads the
        # constructor value (an in-place edit of model.rhoa is not picked up)
        model = dn.Unmyelinated([1.0] * B, L=1000.0, dx=10.0, celsius=6.3, v_init=-65.0,
                                dtype=dtype, integrator=dn.bwd_euler_ub(), rhoa=100.0)
        model.insert(hh)
        amp_ma = (amp_na * 1e-6).to(dtype).reshape(B, 1)
        model[..., 0].inject(dn.mono_rect(amp=amp_ma, delay=5.0, pw=1.0))
        model.initialize()
        m0 = model.mech.hh.m.detach().clone()
        rec = dn.Recorder(("v",))
        model.run(dt=dt, duration=steps * dt, callbacks=[rec])
        v = torch.stack([x.reshape(B, -1) for x in rec.rec["v"]]).to(torch.float64)
    K = v.shape[-1]
    out = dict(
        B=B, K=K, steps=steps, dt=dt, diam=1.0, dx=10.0, rhoa=100.0, celsius=6.3,
        v_init=-65.0, amp_ma=(amp_na * 1e-6).numpy(), delay=5.0, pw=1.0, comp=0,
        v_trace=v.numpy(),  # (steps+1, B, K)
        m0=m0.reshape(B, -1).double().numpy(),
        v_final=model.v.reshape(B, -1).double().numpy(),
        m_final=model.mech.hh.m.reshape(B, -1).double().numpy(),
        h_final=model.mech.hh.h.reshape(B, -1).double().numpy(),
        n_final=model.mech.hh.n.reshape(B, -1).double().numpy(),
    )
    keep = [0, K // 4, K // 2, 3 * K // 4, K - 1]
    out["trace_comps"] = np.array(keep)
    out["v_trace"] = out["v_trace"][:, :, keep]
    np.savez_compressed(os.path.join(HERE, f"hh_cable_{tag}.npz"), **out)
    print("hh_cable", tag, "K", K, "max v", float(v.max()))


def hh_extra(dtype, tag):
    dn = _ref()
    from dendra.models.mod import hh

    B, steps, dt = 3, 600, 0.005
    diam = [1.0, 2.0, 4.0]
    dist_um = torch.tensor([500.0, 200.0, 300.0], dtype=torch.float64)
    amp = torch.tensor([-1.0, -4.0, -8.0], dtype=torch.float64)  # cathodic, mA
    with dn.ctx(JIT=0):
        model = dn.Unmyelinated(diam, L=500.0, dx=10.0, celsius=6.3, v_init=-65.0,
                                dtype=dtype, integrator=dn.bwd_euler_ub(), rhoa=100.0)
        model.insert(hh)
        model.initialize()
        K = model.v.shape[-1]
        x = torch.linspace(-(K - 1) * 10.0 / 2, (K - 1) * 10.0 / 2, K, dtype=torch.float64)
        rhoe = 1.0 / 0.3 * 100.0  # sigma 0.3 S/m -> 333.33 ohm cm
        r = torch.sqrt(x[None, :] ** 2 + dist_um[:, None] ** 2) * 1e-4
        field = rhoe / (4 * torch.pi * r)  # mV/mA, (B, K)
        spatial = (field * amp[:, None]).to(dtype)
        rec = dn.Recorder(("v",))
        model.run(dt=dt, duration=steps * dt, callbacks=[rec],
                  extra=(spatial, dn.mono_rect(amp=1.0, delay=1.0, pw=0.1)))
        v = torch.stack([t.reshape(B, -1) for t in rec.rec["v"]]).to(torch.float64)
    out = dict(B=B, K=K, steps=steps, dt=dt, diam=np.array(diam), dx=10.0, rhoa=100.0,
               celsius=6.3, v_init=-65.0, field_times_amp=spatial.double().numpy(),
               delay=1.0, pw=0.1, v_trace=v.numpy(),
               v_final=model.v.reshape(B, -1).double().numpy())
    keep = [0, K // 4, K // 2, 3 * K // 4, K - 1]
    out["trace_comps"] = np.array(keep)
    out["v_trace"] = out["v_trace"][:, :, keep]
    np.savez_compressed(os.path.join(HERE, f"hh_extra_{tag}.npz"), **out)
    print("hh_extra", tag, "K", K, "max v", float(v.max()))


def tridiag():
    _ref()
    from dendra.models.integrators.tridiag.pcr import pcr_solve_parallel_t, pcr_solve_t

    out = {}
    g = torch.Generator().manual_seed(7)
    for K in (1, 2, 3, 7, 33, 101, 401):
        B = 6
        a = -torch.rand(B, K - 1, generator=g, dtype=torch.float64)
        c = -torch.rand(B, K - 1, generator=g, dtype=torch.float64)
        b = 2.5 + torch.rand(B, K, generator=g, dtype=torch.float64)
        d = torch.randn(B, K, generator=g, dtype=torch.float64)
        for tag, dt in (("f64", torch.float64), ("f32", torch.float32)):
            args = [t.to(dt) for t in (a, b, c, d)]
            out[f"K{K}_{tag}_thomas"] = pcr_solve_t(*args).numpy()
            out[f"K{K}_{tag}_pcr"] = pcr_solve_parallel_t(*args).numpy()
        out[f"K{K}_a"], out[f"K{K}_b"], out[f"K{K}_c"], out[f"K{K}_d"] = (
            t.numpy() for t in (a, b, c, d))
    np.savez_compressed(os.path.join(HERE, "tridiag.npz"), **out)
    print("tridiag", len(out))


def rates():
    _ref()
    from dendra.models.mechanisms._cnexp import _bounded_phi1, _linear_exact_step
    from dendra.models.mechanisms.ops import exprelr

    out = {}
    v = torch.linspace(-120.0, 60.0, 1801, dtype=torch.float64)
    v = torch.cat([v, torch.tensor([-40.0, -55.0, -40.0 + 1e-7, -55.0 - 3e-6])])
    for tag, dt in (("f64", torch.float64), ("f32", torch.float32)):
        vv = v.to(dt)
        ten = torch.full_like(vv, 10.0)
        # GLOBAL rate constants as the reference holds them (float32 values)
        am = float(np.float32(0.1)) * exprelr(-(vv + 40), ten)
        bm = 4.0 * torch.exp(-(vv + 65) / 18)
        ah = float(np.float32(0.07)) * torch.exp(-(vv + 65) / 20)
        bh = 1.0 / (torch.exp(-(vv + 35) / 10) + 1)
        an = float(np.float32(0.01)) * exprelr(-(vv + 55), ten)
        bn = 0.125 * torch.exp(-(vv + 65) / 80)
        out[f"v_{tag}"] = vv.numpy()
        out[f"rates_{tag}"] = torch.stack([am, am + bm, ah, ah + bh, an, an + bn], -1).numpy()
        z = torch.linspace(-0.5, 0.5, 201, dtype=dt)
        out[f"z_{tag}"] = z.numpy()
        out[f"phi1_{tag}"] = _bounded_phi1(z).numpy()
        # cnexp on a grid of (x, a, b) including both branches
        gx = torch.Generator().manual_seed(3)
        x = torch.rand(500, generator=gx, dtype=torch.float64).to(dt)
        bcoef = (10.0 ** (torch.rand(500, generator=gx, dtype=torch.float64) * 5 - 3)).to(dt)
        acoef = (bcoef.double() * torch.rand(500, generator=gx, dtype=torch.float64)).to(dt)
        dtt = torch.tensor(0.025, dtype=dt)
        out[f"cnexp_in_{tag}"] = torch.stack([x, acoef, bcoef], -1).numpy()
        out[f"cnexp_out_{tag}"] = _linear_exact_step(x, acoef - bcoef * x, acoef, -bcoef,
                                                     dtt).numpy()
    np.savez_compressed(os.path.join(HERE, "rates.npz"), **out)
    print("rates")


def dhs():
    _ref()
    from dendra.models.integrators.tree import build_dhs_layers, build_morphology

    out = {}
    parent = [-1, 0, 0, 1, 1, 2, 5]
    out["parity_parent"] = np.array(parent)
    for threads in (1, 8, 32):
        _, _, depth = build_morphology(parent)
        order, layer_ptr = build_dhs_layers(depth, threads)
        out[f"parity_order_t{threads}"] = order.numpy()
        out[f"parity_layer_ptr_t{threads}"] = layer_ptr.numpy()
    # a random tree (parents before children)
    rng = np.random.default_rng(11)
    K = 300
    par = [-1] + [int(rng.integers(max(0, i - 20), i)) for i in range(1, K)]
    _, _, depth = build_morphology(par)
    order, layer_ptr = build_dhs_layers(depth, 32)
    out["rand_parent"] = np.array(par)
    out["rand_depth"] = depth.numpy()
    out["rand_order_t32"] = order.numpy()
    out["rand_layer_ptr_t32"] = layer_ptr.numpy()

    def dense(par, d_mem, a_geom, rhs):
        matrix = torch.diag_embed(d_mem + a_geom)
        for child, p in enumerate(par):
            if p < 0:
                continue
            edge = a_geom[:, child]
            matrix[:, p, p] += edge
            matrix[:, child, p] -= edge
            matrix[:, p, child] -= edge
        return torch.linalg.solve(matrix, rhs.unsqueeze(-1)).squeeze(-1)

    batch, size = 5, len(parent)
    d_mem = torch.linspace(1.3, 2.6, batch * size, dtype=torch.float64).reshape(batch, size)
    a_geom = torch.linspace(0.015, 0.095, batch * size, dtype=torch.float64).reshape(batch, size)
    a_geom[:, 0] = 0.0
    rhs = torch.linspace(-1.7, 2.1, batch * size, dtype=torch.float64).reshape(batch, size)
    out["parity_d"], out["parity_a"], out["parity_b"] = d_mem.numpy(), a_geom.numpy(), rhs.numpy()
    out["parity_x"] = dense(parent, d_mem, a_geom, rhs).numpy()
    g = torch.Generator().manual_seed(5)
    d_r = 1.0 + torch.rand(4, K, generator=g, dtype=torch.float64)
    a_r = 0.5 * torch.rand(4, K, generator=g, dtype=torch.float64)
    a_r[:, 0] = 0
    b_r = torch.randn(4, K, generator=g, dtype=torch.float64)
    out["rand_d"], out["rand_a"], out["rand_b"] = d_r.numpy(), a_r.numpy(), b_r.numpy()
    out["rand_x"] = dense(par, d_r, a_r, b_r).numpy()
    np.savez_compressed(os.path.join(HERE, "dhs.npz"), **out)
    print("dhs")


def events():
    _ref()
    from dendra.models.mod.EXP2SYN import exp2syn  # noqa: F401
    from dendra.models.networks._event_delivery import dense_due, dense_fixed_delay_transition

    out = {}
    rng = np.random.default_rng(21)
    n_conn, width, depth, steps = 64, 16, 9, 30
    post = rng.integers(0, width, n_conn)
    delay = rng.integers(1, depth, n_conn)
    weight = rng.lognormal(-7, 0.5, n_conn)
    gates = (rng.random((steps, n_conn)) < 0.2).astype(np.float64)
    queue = torch.zeros(depth, width, dtype=torch.float64)
    slot = torch.zeros(1, dtype=torch.long)
    gstep = torch.zeros(1, dtype=torch.long)
    delivered = []
    for s in range(steps):
        due = dense_due(queue, slot).payload.clone()
        delivered.append(due.numpy())
        queue, slot, gstep, _ = dense_fixed_delay_transition(
            queue, slot, gstep, torch.as_tensor(weight), torch.as_tensor(gates[s]),
            post_idx=torch.as_tensor(post), delay_steps=torch.as_tensor(delay),
            depth=depth, width=width)
    out.update(post=post, delay=delay, weight=weight, gates=gates, depth=depth, width=width,
               delivered=np.stack(delivered), final_queue=queue.numpy(),
               final_slot=int(slot.item()))
    # NetCon delay rounding known answers (tests/networks/test_event_delivery_contract.py:103-116)
    ratios = np.array([0.49, 0.5, 0.51, 1.49, 1.5, 1.51, 2.5, 3.5])
    out["round_ratios"] = ratios
    out["round_delay_steps"] = np.array([0, 0, 1, 1, 2, 2, 2, 4])
    out["round_inference_steps"] = np.array([1, 1, 1, 1, 2, 2, 2, 4])
    # Exp2Syn normalisation factor (EXP2SYN.py:112-144) for a grid of taus
    tau1 = torch.tensor([0.5, 0.1, 1.0, 2.0, 4.999, 5.0], dtype=torch.float64)
    tau2 = torch.tensor([5.0, 10.0, 3.0, 2.0, 5.0, 5.0], dtype=torch.float64)
    from types import SimpleNamespace

    fake = SimpleNamespace(DE={"A": SimpleNamespace(tau1=tau1), "B": SimpleNamespace(tau2=tau2)})
    derived = exp2syn.derive_buffers(fake)
    out["exp2syn_tau1"], out["exp2syn_tau2"] = tau1.numpy(), tau2.numpy()
    out["exp2syn_factor"] = derived["factor"].numpy()
    np.savez_compressed(os.path.join(HERE, "events.npz"), **out)
    print("events")


def block3():
    """The reference's functional block PCR (tridiag/block.py:80-219) on seeded
    3x3 block-tridiagonal systems shaped like the multi-layer extracellular
    cable (diagonally dominant main blocks, negative diagonal couplings)."""
    _ref()
    from dendra.models.integrators.tridiag.block import block_pcr_solve_t

    out = {}
    g = torch.Generator().manual_seed(33)
    for K in (1, 2, 3, 8, 33, 101, 257):
        B = 4
        lower = -torch.rand(B, max(K - 1, 0), 3, generator=g, dtype=torch.float64)
        upper = -torch.rand(B, max(K - 1, 0), 3, generator=g, dtype=torch.float64)
        main = 0.3 * torch.randn(B, K, 3, 3, generator=g, dtype=torch.float64)
        main = main + torch.diag_embed(3.0 + torch.rand(B, K, 3, generator=g, dtype=torch.float64))
        rhs = torch.randn(B, K, 3, generator=g, dtype=torch.float64)
        for name, t in (("lower", lower), ("upper", upper), ("main", main), ("rhs", rhs)):
            out[f"K{K}_{name}"] = t.numpy()
        for tag, dt in (("f64", torch.float64), ("f32", torch.float32)):
            x = block_pcr_solve_t(lower.to(dt), main.to(dt), upper.to(dt), rhs.to(dt))
            out[f"K{K}_x_{tag}"] = x.double().numpy()
    np.savez_compressed(os.path.join(HERE, "block3.npz"), **out)
    print("block3", len(out))


def adjoint():
    """Reference autograd gradients of a somatic-trace MSE w.r.t. gnabar, gkbar,
    gl and Ra: one single-cable float64 model per cable (the reference's HH
    parameters are scalars per model), Unmyelinated(L=100, dx=10) -> K=11,
    somatic current clamp, 400 steps of 0.025 ms.  Targets come from the same
    model at hidden parameters (defaults x U[0.7, 1.3]); the gradient is taken
    at the defaults, through the reference's CPU path (pcr_solve_t)."""
    dn = _ref()
    from dendra.models.mod import hh

    steps, dt, K = 400, 0.025, 11
    amp_na = np.array([0.3, 0.2, 0.15])
    rng = np.random.default_rng(77)
    defaults = dict(gnabar=0.12, gkbar=0.036, gl=0.0003, rhoa=100.0)
    hidden = {k: (v * rng.uniform(0.7, 1.3, amp_na.size)).astype(np.float32).astype(np.float64)
              for k, v in defaults.items()}
    guess = {k: np.full(amp_na.size, float(np.float32(v))) for k, v in defaults.items()}

    def model_run(i, prm, grad):
        with dn.ctx(JIT=0, REQUIRE_GRAD=1 if grad else 0):
            model = dn.Unmyelinated([1.0], L=100.0, dx=10.0, celsius=6.3, v_init=-65.0,
                                    dtype=torch.float64, integrator=dn.bwd_euler_ub(),
                                    rhoa=float(prm["rhoa"][i]))
            model.insert(hh)
            amp = torch.tensor([[amp_na[i] * 1e-6]], dtype=torch.float64)
            model[..., 0].inject(dn.mono_rect(amp=amp, delay=1.0, pw=1.0))
            model.initialize()
            if grad:
                model.train()
            mech = model.mech.hh
            with torch.no_grad():
                mech.gnabar_param.fill_(float(prm["gnabar"][i]))
                mech.gkbar_param.fill_(float(prm["gkbar"][i]))
                mech.gl_param.fill_(float(prm["gl"][i]))
            rec = dn.Recorder(("v",))
            model.run(dt=dt, duration=steps * dt, callbacks=[rec])
            v0 = torch.stack([x.reshape(-1)[0] for x in rec.rec["v"]])
        return model, v0

    targets, traces, loss, grads = [], [], [], {k: [] for k in defaults}
    for i in range(amp_na.size):
        _, tgt = model_run(i, hidden, False)
        model, v0 = model_run(i, guess, True)
        L = ((v0 - tgt.detach()) ** 2).sum() / (steps + 1)
        named = dict(model.named_parameters())
        keys = {"gnabar": "integrator.mech.mechanisms.hh.gnabar_param",
                "gkbar": "integrator.mech.mechanisms.hh.gkbar_param",
                "gl": "integrator.mech.mechanisms.hh.gl_param", "rhoa": "rhoa_param"}
        g = torch.autograd.grad(L, [named[keys[k]] for k in defaults])
        for k, gk in zip(defaults, g):
            grads[k].append(float(gk))
        targets.append(tgt.detach().numpy())
        traces.append(v0.detach().numpy())
        loss.append(float(L))
    out = dict(K=K, steps=steps, dt=dt, diam=1.0, dx=10.0, celsius=6.3, v_init=-65.0,
               amp_ma=amp_na * 1e-6, delay=1.0, pw=1.0, comp=0,
               target=np.stack(targets), trace=np.stack(traces), loss=np.array(loss),
               **{f"hidden_{k}": v for k, v in hidden.items()},
               **{f"guess_{k}": v for k, v in guess.items()},
               **{f"grad_{k}": np.array(v) for k, v in grads.items()})
    np.savez_compressed(os.path.join(HERE, "adjoint_f64.npz"), **out)
    print("adjoint", out["loss"], {k: out["grad_" + k] for k in defaults})


def _two_tap_ops():
    """The reference's ordered two-tap CPU operators, built from its source."""
    os.environ.setdefault("TORCH_EXTENSIONS_DIR",
                          os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle", "_ref",
                                       "torch_ext"))
    from dendra.models.networks._two_tap_enqueue import get_cpu_two_tap_enqueue

    get_cpu_two_tap_enqueue()
    return torch.ops.dendra_native


def delay(dtype, tag):
    _ref()
    from dendra.models.networks._event_delivery import (
        delay_interpolation, dense_due, dense_interpolated_delay_transition)

    ops = _two_tap_ops()
    out = {}
    rng = np.random.default_rng(77 if tag == "f64" else 78)
    T = lambda a: torch.as_tensor(np.asarray(a)).to(dtype)  # noqa: E731
    L = lambda a: torch.as_tensor(np.asarray(a), dtype=torch.long)  # noqa: E731

    # one step of the ordered op: heavy collisions, a tap on the slot row
    depth, width, E, n_src = 7, 5, 48, 6
    post = rng.integers(0, width, E)
    lam = rng.uniform(1.0, 7.6, E)
    dt = 0.025
    delays = lam * dt
    off, frac = delay_interpolation(T(delays), T([dt]), dtype=dtype, taps=2, sigma=0.0)
    lower = (off.remainder(depth) * width + L(post))
    upper = (lower + width).remainder(depth * width)
    general_upper = L(rng.integers(0, depth * width, E))  # any column
    w = rng.standard_normal(E)
    g = rng.random(E)
    g[rng.random(E) < 0.3] = 0.0
    g_src = rng.random(n_src)
    pre = rng.integers(0, n_src, E)
    queue = rng.standard_normal((depth, width))
    slot = 3
    out.update(depth=depth, width=width, post=post, delays=delays, dt=dt, w=w, g=g,
               g_src=g_src, pre=pre, queue=queue, slot=slot, lower=lower.numpy(),
               upper=upper.numpy(), fraction=frac.numpy(), general_upper=general_upper.numpy())
    Q, S = T(queue), L([slot])
    out["op_edge"] = ops.ordered_two_tap_enqueue(Q, S, T(w), T(g), frac, lower, upper).numpy()
    out["op_src"] = ops.ordered_two_tap_enqueue_from_source(
        Q, S, T(w), T(g_src), frac, lower, upper, L(pre)).numpy()
    out["op_general"] = ops.ordered_two_tap_enqueue(
        Q, S, T(w), T(g), frac, lower, general_upper).numpy()
    pure = dense_interpolated_delay_transition(
        Q, S, L([0]), T(w), T(g), T(delays), T([dt]), post_idx=L(post), depth=depth,
        width=width, taps=2, sigma=0.0).queue.numpy()
    assert np.array_equal(pure, out["op_edge"]), "ordered op != pure-torch transition"
    cot = rng.standard_normal((depth, width))
    out["cot"] = cot
    for name, src in (("edge", None), ("src", L(pre))):
        gates = T(g) if src is None else T(g_src)
        dw, dg, df = ops.delay_ring_two_tap_vjp(T(cot), L([slot * width]), T(w), gates, frac,
                                                lower, upper, src)
        out[f"vjp_{name}_dw"], out[f"vjp_{name}_dg"], out[f"vjp_{name}_df"] = (
            dw.numpy(), dg.numpy(), df.numpy())
    lo, hi = ops.delay_ring_gather_two_tap(T(cot), L([slot * width]), lower, upper)
    out["gather_lo"], out["gather_hi"] = lo.numpy(), hi.numpy()

    # three taps, one step, with autograd of weights / gates / coefficients
    sigma = 0.6
    off3, c3 = delay_interpolation(T(delays), T([dt]), dtype=dtype, taps=3, sigma=sigma)
    wt, gt, ct = (T(w).requires_grad_(), T(g).requires_grad_(), c3.detach().requires_grad_())
    q3 = dense_interpolated_delay_transition(
        Q, S, L([0]), wt, gt, None, None, post_idx=L(post), depth=depth, width=width,
        taps=3, sigma=sigma, delay_taps=(off3, ct)).queue
    (q3 * T(cot)).sum().backward()
    out.update(sigma=sigma, offsets3=off3.numpy(), coeff3=c3.detach().numpy(),
               three_tap=q3.detach().numpy(), three_dw=wt.grad.numpy(),
               three_dg=gt.grad.numpy(), three_dc=ct.grad.numpy())

    # a rollout with autograd: source gates per step, delays differentiated
    depth, width, E, n_src, steps = 9, 6, 24, 5, 40
    post = rng.integers(0, width, E)
    pre = rng.integers(0, n_src, E)
    delays = rng.uniform(1.0, 8.7, E) * dt
    w = rng.standard_normal(E)
    gates = rng.random((steps, n_src))
    gates[rng.random((steps, n_src)) < 0.5] = 0.0
    queue0 = rng.standard_normal((depth, width))
    cpay = rng.standard_normal((steps, width))
    cfin = rng.standard_normal((depth, width))
    wt, gt, dlt, qt = (T(w).requires_grad_(), T(gates).requires_grad_(),
                       T(delays).requires_grad_(), T(queue0).requires_grad_())
    queue, slot, gs = qt, L([2]), L([0])
    payloads = []
    for k in range(steps):
        payloads.append(dense_due(queue, slot).payload)
        src_g = gt[k].index_select(0, L(pre))
        queue, slot, gs, _ = dense_interpolated_delay_transition(
            queue, slot, gs, wt, src_g, dlt, T([dt]), post_idx=L(post), depth=depth,
            width=width, taps=2, sigma=0.0)
    pay = torch.stack(payloads)
    loss = (pay * T(cpay)).sum() + (queue * T(cfin)).sum()
    loss.backward()
    out.update(r_depth=depth, r_width=width, r_post=post, r_pre=pre, r_delays=delays, r_w=w,
               r_gates=gates, r_queue0=queue0, r_slot0=2, r_cpay=cpay, r_cfin=cfin,
               r_payload=pay.detach().numpy(), r_final=queue.detach().numpy(),
               r_dw=wt.grad.numpy(), r_dgates=gt.grad.numpy(), r_ddelays=dlt.grad.numpy(),
               r_dqueue0=qt.grad.numpy())
    # the inputs of the reference's own transition tests
    # (tests/networks/test_pure_delay_interpolation.py:24-47): collisions, a
    # wrap past the ring's end, sub-step delays clamped to one step
    for taps in (2, 3):
        qt = (torch.arange(18).reshape(3, 6).t() / 10).to(dtype).contiguous().requires_grad_()
        wt = tt_ = torch.tensor([0.5, 1.0, -2.0, 3.0, 0.0], dtype=dtype, requires_grad=True)
        gt = torch.tensor([-0.2, 0.4, 0.5, 1.0, 2.0], dtype=dtype, requires_grad=True)
        dlt = torch.tensor([0.02, 0.1, 0.23, 0.2, 0.6], dtype=dtype, requires_grad=True)
        tr = dense_interpolated_delay_transition(
            qt, L([4]), L([17]), wt, gt, dlt, torch.tensor(0.1, dtype=dtype),
            post_idx=L([1, 1, 2, 0, 1]), depth=6, width=3, taps=taps, sigma=0.5)
        cq = torch.as_tensor(rng.standard_normal((6, 3))).to(dtype)
        (tr.queue * cq).sum().backward()
        out.update({f"pure{taps}_queue": tr.queue.detach().numpy(), f"pure{taps}_cot": cq.numpy(),
                    f"pure{taps}_dq": qt.grad.numpy(), f"pure{taps}_dw": wt.grad.numpy(),
                    f"pure{taps}_dg": gt.grad.numpy(), f"pure{taps}_dd": dlt.grad.numpy(),
                    f"pure{taps}_slot": int(tr.slot.item()), f"pure{taps}_step": int(
                        tr.global_step.item())})
        del tt_
    np.savez_compressed(os.path.join(HERE, f"delay_{tag}.npz"), **out)
    print("delay", tag)


def netstim(dtype, tag):
    _ref()
    from dendra.models.networks._netstim_renewal import netstim_initial_state, netstim_renewal

    rng = np.random.default_rng(91 if tag == "f64" else 92)
    N, T, dt = 9, 600, 0.025
    interval = np.array([10.0, 5.0, 200.0, 1.3, 7.0, 50.0, 0.02, 1e30, 3.0])
    noise = np.array([0.0, 0.5, 1.0, 1.0, 0.3, 0.0, 1.0, 0.7, 0.2])
    start = np.array([0.0, 2.0, 0.0, 1.5, 0.0, 10.0, 0.0, 0.0, 0.1])
    number = np.array([10**9, 3, 10**9, 5, 10**9, 2, 10**9, 10**9, 0], dtype=np.int64)
    draws0 = rng.exponential(size=N)
    draws = rng.exponential(size=(T, N))
    tt = lambda a: torch.as_tensor(a).to(dtype)  # noqa: E731
    state = netstim_initial_state(tt(interval), tt(start), tt(noise), tt(draws0))
    nxt, cnt, spk = [state.next_stoch_time.numpy().copy()], [state.spike_counts.numpy().copy()], []
    for k in range(T):
        t = torch.zeros((), dtype=dtype) + torch.tensor(float(k), dtype=dtype) * dt
        tr = netstim_renewal(state, tt(interval), tt(noise), torch.as_tensor(number), t,
                             tt(draws[k]), tau=0.5, bptt=False)
        state = tr.state
        nxt.append(state.next_stoch_time.numpy().copy())
        cnt.append(state.spike_counts.numpy().copy())
        spk.append(tr.spikes.numpy().astype(np.uint8))
    out = dict(interval=interval, noise=noise, start=start, number=number, dt=dt,
               draws0=draws0, draws=draws, next_time=np.stack(nxt), counts=np.stack(cnt),
               spikes=np.stack(spk))
    np.savez_compressed(os.path.join(HERE, f"netstim_{tag}.npz"), **out)
    print("netstim", tag, int(out["spikes"].sum()))


def network_points():
    """A 16-cell network of single-compartment HH cells (the reference's
    default Population geometry) with one Exp2Syn synapse each, driven by a
    periodic NetStim per cell (noise 0: no random draws) through one-to-one
    NetCons and coupled all-to-all (autapses included) with lognormal weights
    and U[1, 5] ms delays, run step by step through Network.run on the CPU
    (dense delay ring).  Records the NetStim emissions, the membrane trace of
    every cell, the synapse states and the connection list in the reference's
    edge order (source-major)."""
    dn = _ref()
    from dendra.models.mod import exp2syn, hh

    N, dt, steps = 16, 0.025, 2000
    w_bg, d_bg = 0.2, 1.0
    rng = np.random.default_rng(11)
    interval = rng.uniform(6.0, 14.0, N)
    start = rng.uniform(0.5, 4.0, N)
    W = rng.lognormal(-4.5, 0.5, (N, N))
    D = rng.uniform(1.0, 5.0, (N, N))
    with dn.ctx(JIT=0):
        pop = dn.Population(N=N, C=1, v_init=-65.0, celsius=6.3, dtype=torch.float64)
        pop.insert(hh)
        pop.insert(exp2syn.rename("syn"), tau1=0.5, tau2=5.0, e=0.0)
        stim = dn.NetStim(N=N, interval=torch.as_tensor(interval),
                          start=torch.as_tensor(start), noise=0.0, dtype=torch.float64)
        net = dn.Network({"cells": pop}, netstim=stim, track_netcon_events=False,
                         netcon_delay_backend="dense")
        net.connect_one_to_one(net.netstim[:], pop[:], pop.mech.syn, threshold=None,
                               weight=torch.full((N,), w_bg, dtype=torch.float64),
                               delay=torch.full((N,), d_bg, dtype=torch.float64))
        net.connect_dense(pop[:], pop[:], pop.mech.syn, threshold=0.0,
                          weight=torch.as_tensor(W.reshape(-1)),
                          delay=torch.as_tensor(D.reshape(-1)), allow_autapses=True)
        net.initialize(dt)
        syn = pop.mech.syn
        v = [pop.v.reshape(-1).clone()]
        A, B, emitted = [syn.A.reshape(-1).clone()], [syn.B.reshape(-1).clone()], []
        for _ in range(steps):
            net.run(steps=1)
            v.append(pop.v.reshape(-1).clone())
            A.append(syn.A.reshape(-1).clone())
            B.append(syn.B.reshape(-1).clone())
            emitted.append(stim.spikes.reshape(-1).clone())
    src = np.repeat(np.arange(N), N)  # connect_dense: source-major, then target
    dst = np.tile(np.arange(N), N)
    out = dict(N=N, dt=dt, steps=steps, celsius=6.3, v_init=-65.0,
               diam=float(pop.diam.reshape(-1)[0]), length=float(pop.dx.reshape(-1)[0]),
               tau1=0.5, tau2=5.0, e_syn=0.0, spk_thr=0.0, w_bg=w_bg, d_bg=d_bg,
               interval=interval, start=start, pre=src, post=dst, weight=W.reshape(-1),
               delay=D.reshape(-1), stim_emitted=torch.stack(emitted).numpy(),
               v=torch.stack(v).numpy(), A=torch.stack(A).numpy(), B=torch.stack(B).numpy())
    np.savez_compressed(os.path.join(HERE, "network_points.npz"), **out)
    up = (out["v"][1:] >= 0) & (out["v"][:-1] < 0)
    print("network_points spikes per cell", up.sum(0).tolist())


def netcon_tapes():
    """The reference's bit-pack known-answer tapes
    (tests/networks/test_backend_equivalence.py:93-205), recorded from its dense
    and bit-packed NetCon backends on the CPU: a fan-in/fan-out tape of three
    sources onto two targets through 1-3 step delays that wraps the ring, and a
    65-source one-to-one tape across the 63-bit word boundary.  ExpSyn g after
    each NetCon.advance is the running sum of the delivered weights."""
    dn = _ref()
    from dendra.models.mod import expsyn

    dt = 0.1
    out = {}
    w = torch.tensor([1.0, 2.0, 3.0, 4.0, 5.0, 6.0], dtype=torch.float64)
    dly = torch.tensor([0.1, 0.2, 0.3, 0.1, 0.2, 0.3], dtype=torch.float64)
    tape = np.array([[1, 1, 0], [0, 0, 1], [1, 0, 1], [0, 0, 0], [0, 1, 0], [1, 0, 0],
                     [0, 0, 0], [0, 0, 0], [0, 0, 0]], dtype=bool)
    active = np.zeros(65, dtype=bool)
    active[[0, 62, 63, 64]] = True
    word_tape = np.stack([active, np.zeros_like(active)])
    for backend in ("dense", "bitpacked_history"):
        post = dn.Population(N=2, C=1, v_init=-65.0, dtype=torch.float64)
        post.insert(expsyn.rename("syn"), e=0.0, tau=1.0)
        stim = dn.NetStim(N=3, dtype=torch.float64)
        net = dn.Network({"post": post}, netstim=stim, track_netcon_events=False,
                         netcon_delay_backend=backend)
        net.connect_dense(net.netstim[:], post[:], post.mech.syn, threshold=None, weight=w,
                          delay=dly)
        net.build(dt)
        net.init_synapses()
        nc = next(iter(net.synapses.values()))
        rows = []
        for spikes in tape:
            net.netstim.spikes.copy_(torch.as_tensor(spikes))
            nc.advance()
            rows.append(nc.syn.g.detach().reshape(-1).clone())
        out[f"fan_g_{backend}"] = torch.stack(rows).numpy()

        post = dn.Population(N=65, C=1, v_init=-65.0, dtype=torch.float64)
        post.insert(expsyn.rename("syn"), e=0.0, tau=1.0)
        stim = dn.NetStim(N=65, dtype=torch.float64)
        net = dn.Network({"post": post}, netstim=stim, netcon_delay_backend=backend)
        net.connect_one_to_one(net.netstim[:], post[:], post.mech.syn, threshold=None,
                               weight=torch.ones(65, dtype=torch.float64),
                               delay=torch.full((65,), dt, dtype=torch.float64))
        net.build(dt)
        net.init_synapses()
        nc = next(iter(net.synapses.values()))
        rows = []
        for spikes in word_tape:
            net.netstim.spikes.copy_(torch.as_tensor(spikes))
            nc.advance()
            rows.append(nc.syn.g.detach().reshape(-1).clone())
        out[f"word_g_{backend}"] = torch.stack(rows).numpy()
    out.update(dt=dt, fan_pre=np.array([0, 0, 1, 1, 2, 2]), fan_post=np.array([0, 1, 0, 1, 0, 1]),
               fan_weight=w.numpy(), fan_delay=dly.numpy(), fan_tape=tape, word_tape=word_tape)
    np.savez_compressed(os.path.join(HERE, "netcon_tapes.npz"), **out)
    print("netcon_tapes", out["fan_g_dense"][-1], out["word_g_dense"][-1][[0, 61, 62, 63, 64]])


def thresholds():
    """The reference Thresholder (models/instruments/thresholder.py) on twelve
    unbranched HH cables (Unmyelinated, L 2000 um, dx 20 um, diameters
    U[1, 4] um, float64) under a cathodic 0.1 ms point-source pulse at
    U[300, 1500] um: bound fixing from ub = 0.5 mA (doubling, at most ten
    times), bisection to rtol 1 % at dt 0.005 ms over 2 ms, activity = a 0 mV
    rising edge at compartment 5 or -5 (Active's default nodes), no
    conduction-block test.  Records the field it was given and the final
    brackets (NaN where bound fixing gave up)."""
    dn = _ref()
    from dendra.models import callbacks as cb
    from dendra.models.instruments.thresholder import Thresholder
    from dendra.models.mod import hh

    B, dt, tstop, pw = 12, 0.005, 2.0, 0.1
    rng = np.random.default_rng(21)
    D = rng.uniform(1.0, 4.0, B)
    dist = rng.uniform(300.0, 1500.0, B)
    with dn.ctx(JIT=0):
        model = dn.Unmyelinated(list(D), L=2000.0, dx=20.0, celsius=6.3, v_init=-65.0,
                                dtype=torch.float64, integrator=dn.bwd_euler_ub(), rhoa=100.0)
        model.insert(hh)
        model.initialize()
        K = model.v.shape[-1]
        x = torch.linspace(-(K - 1) * 20.0 / 2, (K - 1) * 20.0 / 2, K, dtype=torch.float64)
        r = torch.sqrt(x[None, :] ** 2 + torch.as_tensor(dist)[:, None] ** 2) * 1e-4
        field = (1.0 / 0.3 * 100.0) / (4 * torch.pi * r)
        th = Thresholder(model, cb.Active(threshold=0.0, node_check=[5, -5]), space=-field,
                         time=dn.mono_rect(amp=1.0, delay=0.0, pw=pw),
                         ub=torch.full((B,), 0.5, dtype=torch.float64),
                         lb=torch.zeros(B, dtype=torch.float64), rtol=0.01)
        ub, lb = th.calculate_thresholds(tstop=tstop, dt=dt, block_possible=False)
    out = dict(B=B, K=K, dx=20.0, diam=D, dist=dist, field=field.numpy(), pw=pw, dt=dt,
               tstop=tstop, ub0=0.5, lb0=0.0, rtol=0.01, ub=ub.numpy(), lb=lb.numpy())
    np.savez_compressed(os.path.join(HERE, "thresholds.npz"), **out)
    print("thresholds", out["ub"])


if __name__ == "__main__":
    what = sys.argv[1:] or ["rates", "tridiag", "dhs", "events", "cable", "extra", "adjoint",
                            "block3", "delay", "netstim", "network", "tapes", "thresholds"]
    if "rates" in what:
        rates()
    if "tridiag" in what:
        tridiag()
    if "dhs" in what:
        dhs()
    if "events" in what:
        events()
    if "cable" in what:
        hh_cable(torch.float64, "f64")
        hh_cable(torch.float32, "f32")
    if "extra" in what:
        hh_extra(torch.float64, "f64")
        hh_extra(torch.float32, "f32")
    if "adjoint" in what:
        adjoint()
    if "block3" in what:
        block3()
    if "delay" in what:
        delay(torch.float64, "f64")
        delay(torch.float32, "f32")
    if "netstim" in what:
        netstim(torch.float64, "f64")
        netstim(torch.float32, "f32")
    if "network" in what:
        network_points()
    if "tapes" in what:
        netcon_tapes()
    if "thresholds" in what:
        thresholds()
