"""Shared builders of the golden and synthetic test cases."""

from __future__ import annotations

import numpy as np
import torch

from dendra_gb300.cable import CablePopulation


def golden_cable_population(g, dtype, device="cpu", **kw):
    """The reference's run with the 64-cable workload's geometry, recorded in
    hh_cable_*.npz."""
    B, K = int(g["B"]), int(g["K"])
    pop = CablePopulation([K] * B, float(g["diam"]), float(g["dx"]), rhoa=float(g["rhoa"]),
                          celsius=float(g["celsius"]), v_init=float(g["v_init"]),
                          dtype=dtype, device=device, **kw)
    pop.inject(int(g["comp"]), torch.as_tensor(g["amp_ma"]), float(g["delay"]), float(g["pw"]))
    return pop.initialize(float(g["dt"]))


def golden_extra_population(g, dtype, device="cpu", **kw):
    """The reference's extracellular run recorded in hh_extra_*.npz."""
    B, K = int(g["B"]), int(g["K"])
    pop = CablePopulation([K] * B, torch.as_tensor(g["diam"]), float(g["dx"]),
                          rhoa=float(g["rhoa"]), celsius=float(g["celsius"]),
                          v_init=float(g["v_init"]), dtype=dtype, device=device, **kw)
    field = torch.as_tensor(g["field_times_amp"]).reshape(-1)
    pop.set_extracellular(field, 1.0, float(g["delay"]), float(g["pw"]))
    return pop.initialize(float(g["dt"]))


def as_f64(p):
    """Widen a problem dict's float arrays to float64 (the float64 reference of a run)."""
    return {k: (v.astype(np.float64) if isinstance(v, np.ndarray) and v.dtype.kind == "f" else v)
            for k, v in p.items()}


def oracle_traces(pop, steps, comps, spk_idx=None, ref64=False):
    """Run the oracle from pop's current state once per recorded compartment.

    ref64: run in float64 on the population's (float32) inputs, with the
    pulse gates on the float32 time grid the population itself sees.
    Returns (traces (steps+1, B, len(comps)), final problem dict, spikes).
    """
    import oracle

    out = []
    final = None
    spikes = None
    gate_f32 = ref64 and pop.dtype == torch.float32
    for c in comps:
        p = pop.problem_dict()
        if ref64:
            p = as_f64(p)
        p["rec_idx"] = np.full(pop.B, int(c), dtype=np.int32)
        if spk_idx is not None:
            p["spk_idx"] = np.full(pop.B, int(spk_idx), dtype=np.int32)
        tr, cnt, first, _ = oracle.cable_run(p, steps, gate_f32=gate_f32)
        out.append(tr)
        final = p
        spikes = (cnt, first)
    return np.stack(out, axis=-1).transpose(1, 0, 2), final, spikes


def synthetic_population(seed, n_cables, kmin, kmax, dtype, device, *, extra=True, intra=False,
                         dt=0.005, **kw):
    """A C2-style ragged population: odd K uniform in [kmin, kmax], diam U[0.5,4],
    length U[500,5000] um (dx = L/K), point source at U[0.5,3] mm with a cathodic
    0.1 ms pulse of U[0.1,2] mA starting at t=0."""
    rng = np.random.default_rng(seed)
    ks = 2 * rng.integers((kmin - 1) // 2, (kmax - 1) // 2 + 1, n_cables) + 1
    ks = np.clip(ks, kmin, kmax)
    diam = rng.uniform(0.5, 4.0, n_cables)
    length = rng.uniform(500.0, 5000.0, n_cables)
    dx = length / ks
    pop = CablePopulation(ks.tolist(), torch.as_tensor(diam), torch.as_tensor(dx), rhoa=100.0,
                          celsius=6.3, v_init=-65.0, dtype=dtype, device=device, **kw)
    if extra:
        dist = rng.uniform(500.0, 3000.0, n_cables)
        amp = -rng.uniform(0.1, 2.0, n_cables)
        x = pop.positions()
        cab = np.repeat(np.arange(n_cables), ks)
        r_um = torch.sqrt(x ** 2 + torch.as_tensor(dist[cab]) ** 2)
        field = (1.0 / 0.3 * 100.0) / (4 * torch.pi * r_um * 1e-4)
        pop.set_extracellular(field, torch.as_tensor(amp), 0.0, 0.1)
    if intra:
        pop.inject(0, torch.as_tensor(rng.uniform(0.05, 0.5, n_cables) * 1e-6), 0.5, 1.0)
    return pop.initialize(dt)


def oracle_thresholds(pop, lb, ub, n_steps, rtol=0.01, max_fix=10, max_tries=25, up=2.0,
                      spk=(60, 192)):
    """Reference bisection rules with every trial run by the float64 oracle."""
    import oracle

    base = as_f64(pop.problem_dict())
    B = pop.B
    lb = np.array(lb, dtype=np.float64) * np.ones(B)
    ub = np.array(ub, dtype=np.float64) * np.ones(B)

    def fired(amp):
        p = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in base.items()}
        p["ve_amp"] = -amp
        p["spk_idx"] = np.full(B, spk[0], dtype=np.int32)
        p["spk_idx2"] = np.full(B, spk[1], dtype=np.int32)
        _, cnt, _, _ = oracle.cable_run(p, n_steps, gate_f32=pop.dtype == torch.float32)
        return cnt > 0

    ignore = np.zeros(B, dtype=bool)
    tries = 0
    while True:
        act = fired(ub) | ignore
        if act.all():
            break
        if tries >= max_fix:
            ignore |= ~act
            ub[~act] = 1.0
            lb[~act] = 1.0
            break
        ub = np.where(~act, ub * up, ub)
        tries += 1
    assert not (fired(lb) & ~ignore).any()
    msk = ((ub - lb) / ub >= rtol) & ~ignore
    tries = 0
    while msk.any() and tries < max_tries:
        stim = (ub + lb) / 2
        f = fired(stim)
        ub = np.where(msk & f, stim, ub)
        lb = np.where(msk & ~f, stim, lb)
        msk = ((ub - lb) / ub >= rtol) & ~ignore
        tries += 1
    ignore |= msk
    ub[ignore] = np.nan
    lb[ignore] = np.nan
    return ub, lb


def golden_adjoint_population(g, dtype, device="cpu", params="guess", **kw):
    """The single-cable reference models of adjoint_f64.npz packed as one population
    (per-cable gnabar, gkbar, gl and Ra at the fixture's guess or hidden values)."""
    B, K = int(g["amp_ma"].size), int(g["K"])
    prm = {k: g[f"{params}_{k}"] for k in ("gnabar", "gkbar", "gl", "rhoa")}
    pop = CablePopulation([K] * B, float(g["diam"]), float(g["dx"]),
                          rhoa=torch.as_tensor(prm["rhoa"]), celsius=float(g["celsius"]),
                          v_init=float(g["v_init"]), dtype=dtype, device=device,
                          hh={k: torch.as_tensor(prm[k]) for k in ("gnabar", "gkbar", "gl")},
                          **kw)
    pop.inject(int(g["comp"]), torch.as_tensor(g["amp_ma"]), float(g["delay"]), float(g["pw"]))
    return pop.initialize(float(g["dt"]))


def mse_trace_grad(trace, target):
    """dLoss/dtrace of Loss = sum over cables of mean over samples of (trace - target)^2."""
    return 2.0 * (trace - target) / trace.shape[1]


def oracle_param_grads(p, steps, target, rec_idx=0):
    """Per-cable (gnabar, gkbar, gl, Ra) gradients of the MSE trace loss by the oracle.

    Returns (trace, loss per cable, dict of per-cable gradients, raw cable_grad output)."""
    import oracle

    B = int(p["cable_ptr"].size - 1)
    q = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in p.items()}
    q["rec_idx"] = np.full(B, rec_idx, dtype=np.int32)
    trace, *_ = oracle.cable_run({k: (v.copy() if isinstance(v, np.ndarray) else v)
                                  for k, v in q.items()}, steps)
    loss = ((trace - target) ** 2).mean(axis=1)
    raw = oracle.cable_grad(q, steps, mse_trace_grad(trace, target))
    counts = np.diff(p["cable_ptr"])
    cab = np.repeat(np.arange(B), counts)
    grads = {k: np.bincount(cab, raw["g_" + k], minlength=B) for k in ("gnabar", "gkbar", "gl")}
    axial = np.bincount(cab, raw["g_axial"], minlength=B)
    grads["rhoa"] = -axial / p["rhoa_per_cable"] if "rhoa_per_cable" in p else None
    return trace, loss, grads, raw
