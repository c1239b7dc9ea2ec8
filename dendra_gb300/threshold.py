"""Activation thresholds of myelinated-fibre-like cables by batched bisection.

Restates the reference Thresholder (models/instruments/thresholder.py):

* ``_fix_bounds`` (:835-871): multiply the upper bound by ``fix_bound_up`` until
  the fibre fires, at most ``max_tries_bound_fix`` times; lanes that never fire
  are ignored (NaN);
* the lower bound must not fire (:916-924);
* bisection (:926-960): ``stimamp = (ub + lb) / 2`` (arithmetic mode), fire ->
  ``ub = stimamp`` else ``lb = stimamp``, while ``(ub - lb) / ub >= rtol``
  (``check_tolerance`` :458-474, ``_relative_window`` :476-478), at most
  ``max_tries_thresh`` iterations; unconverged lanes become NaN;
* activity: a 0 mV rising edge at node 5 or node -5 (the ``Active`` default
  ``node_check=[5, -5]``, models/callbacks.py:1440-1475).

Every trial is one persistent ``dgb_cable_run`` launch over the lanes that
still need it (converged lanes are not simulated again; results are the same
as simulating them and discarding the outcome), with early exit once a fibre
has fired.
"""

from __future__ import annotations

import numpy as np
import torch

from .cable import HH_DEFAULTS, CablePopulation
from .workloads import RHOE_OHM_CM

N_NODES = 21
SEG_PER_INTERNODE = 11
NODE_LEN_UM = 1.0
K_FIBRE = N_NODES + (N_NODES - 1) * SEG_PER_INTERNODE  # 241
MYELIN_CM = 0.005  # uF/cm^2
MYELIN_G = 5.0e-6  # S/cm^2
# nodal HH channel densities relative to the HH defaults: nodes of Ranvier
# carry far denser Na/K channels than a squid axon, and a 1 um node with the
# plain HH densities cannot drive a 1.6 mm myelinated internode
NODE_DENSITY_SCALE = 10.0


def node_compartment(n):
    """Compartment index of node n (negative counts from the far end)."""
    n = n % N_NODES
    return n * (SEG_PER_INTERNODE + 1)


def fibre_params(n, seed=0):
    """Seeded fibre/stimulus parameters with the distributions of the 65,536-fibre
    threshold workload (241 compartments per fibre)."""
    rng = np.random.default_rng(seed)
    return dict(D=rng.uniform(2.0, 16.0, n), dist=rng.uniform(200.0, 5000.0, n),
                offset=rng.uniform(0.0, 1.0, n), pw=rng.uniform(0.05, 1.0, n))


def fibre_population(p, dtype=torch.float32, device="cuda", dt=0.005,
                     node_density_scale=NODE_DENSITY_SCALE, **kw):
    """Myelinated-fibre-like cables: 21 HH nodes (1 um long) and 20 passive
    internodes of 11 compartments (internode length 100 D), diameter D
    everywhere; point source at distance ``dist`` from the fibre axis, axially
    offset by ``offset`` internodes from the central node; cathodic pulse of
    width ``pw`` starting at t = 0 (amplitude set per trial)."""
    D = np.asarray(p["D"], dtype=np.float64)
    B = D.size
    L_int = 100.0 * D
    seg = L_int / SEG_PER_INTERNODE
    is_node = np.zeros(K_FIBRE, dtype=bool)
    is_node[::SEG_PER_INTERNODE + 1] = True
    dx = np.where(is_node[None, :], NODE_LEN_UM, seg[:, None])  # (B, K)
    # compartment centres along the fibre
    right = np.cumsum(dx, axis=1)
    x = right - dx / 2
    centre = x[:, node_compartment(N_NODES // 2)]
    x_src = centre + np.asarray(p["offset"]) * (L_int + NODE_LEN_UM)
    r_cm = np.sqrt((x - x_src[:, None]) ** 2 + np.asarray(p["dist"])[:, None] ** 2) * 1e-4
    field = RHOE_OHM_CM / (4 * np.pi * r_cm)
    # internodes: a myelin sheath of ~100 lamellae, cm 0.005 uF/cm^2 and leak
    # 5e-6 S/cm^2 (the bare membrane's 1 uF/cm^2 and pas 0.001 S/cm^2 / 200)
    scale = {"gnabar": node_density_scale, "gkbar": node_density_scale,
             "gl": node_density_scale, "el": 1.0}
    hh = {k: np.where(is_node, float(np.float32(HH_DEFAULTS[k] * scale[k])), v) for k, v in
          (("gnabar", 0.0), ("gkbar", 0.0), ("gl", MYELIN_G), ("el", -70.0))}
    hh = {k: np.tile(v, B) for k, v in hh.items()}
    hh.update(ena=HH_DEFAULTS["ena"], ek=HH_DEFAULTS["ek"])
    cm = np.tile(np.where(is_node, 1.0, MYELIN_CM), B)
    pop = CablePopulation([K_FIBRE] * B, np.tile(np.ones(K_FIBRE), B) * np.repeat(D, K_FIBRE),
                          torch.as_tensor(dx.reshape(-1)), rhoa=100.0, cm=cm, celsius=6.3,
                          v_init=-65.0, dtype=dtype, device=device, hh=hh, **kw)
    pop.set_extracellular(torch.as_tensor(field.reshape(-1)), torch.zeros(B, dtype=torch.float64),
                          0.0, torch.as_tensor(np.asarray(p["pw"])))
    return pop.initialize(dt)


class Thresholder:
    """Batched bisection on the GPU with the reference's rules.

    Amplitudes are positive magnitudes (mA) of a cathodic pulse.  Activity is
    a rising edge at either of two compartments: the fibre nodes ``node_check``
    (node indices of the myelinated fibre layout) or, for any other cables,
    ``compartments`` (local indices, negative counting from the far end, like
    the reference's ``Active(node_check=...)``).

    tune: pick the trial runs' cables per CTA (1, 2 or 4, every cable on 32
    lanes) by timing the candidates once per population shape
    (``autotune.tune_cable_run``, cached per process and in
    ``DGB_TUNE_CACHE``); the arithmetic, and so every threshold, is the same
    for each of them.
    """

    def __init__(self, pop: CablePopulation, lb, ub, *, rtol=0.01, atol=None,
                 max_tries_bound_fix=10, max_tries_thresh=25, fix_bound_up=2.0,
                 node_check=(5, -5), thr_mv=0.0, compartments=None, tune=True):
        if rtol is None and atol is None:
            raise ValueError("Either atol or rtol must be provided.")
        self.pop = pop
        self.B = pop.B
        dev = pop.device
        self.lb_initial = torch.as_tensor(lb, dtype=torch.float64).expand(self.B).clone().to(dev)
        self.ub_initial = torch.as_tensor(ub, dtype=torch.float64).expand(self.B).clone().to(dev)
        self.rtol, self.atol = rtol, atol
        self.max_tries_bound_fix = max_tries_bound_fix
        self.max_tries_thresh = max_tries_thresh
        self.fix_bound_up = fix_bound_up
        # detection compartments: fibre nodes (node_check) or, for any other
        # cable, two compartment indices (negative: from the far end)
        if compartments is None:
            self.spk = [node_compartment(n) for n in node_check]
        else:
            kk = torch.as_tensor(pop.n_comp, dtype=torch.int32)
            self.spk = [torch.where(torch.as_tensor(c) < 0, kk + int(c),
                                    torch.full_like(kk, int(c))) for c in compartments]
        self.thr = thr_mv
        if tune and pop.device.type == "cuda":
            from .autotune import tune_cable_run

            tune_cable_run(pop, n_steps=50, candidates=((1, 0, 0), (2, 0, 0), (4, 0, 0)))
        self.state0 = tuple(t.clone() for t in (pop.v, pop.m, pop.h, pop.n))
        self.trials = 0
        self.fibre_steps = 0

    def check_active(self, amp, lanes, n_steps):
        """Run one trial for the given lanes at amplitudes amp[lanes]; return fired (bool, all lanes)."""
        pop = self.pop
        for t, t0 in zip((pop.v, pop.m, pop.h, pop.n), self.state0):
            t.copy_(t0)
        pop.step_index = 0
        pop.t = 0.0
        pop._dev["ve_amp"].copy_((-amp).to(pop.dtype))
        cables = lanes.nonzero().squeeze(1).to(torch.int32)
        fired = torch.zeros(self.B, dtype=torch.bool, device=pop.device)
        if cables.numel() == 0:
            return fired
        res = pop.run(n_steps, spk_idx=self.spk[0], spk_idx2=self.spk[1], spk_thr=self.thr,
                      stop_on_spike=True, cables=cables)
        self.trials += 1
        self.fibre_steps += int(cables.numel()) * n_steps
        fired[cables.long()] = res.spk_count[cables.long()] > 0
        return fired

    def _tolerance_open(self, lb, ub):
        aw = ub - lb
        rw = aw / ub
        if self.atol is not None and self.rtol is not None:
            return (aw >= self.atol) | (rw >= self.rtol)
        if self.atol is not None:
            return aw >= self.atol
        return rw >= self.rtol

    def calculate_thresholds(self, n_steps, lb=None, ub=None, lb_verified=False):
        """Return (ub, lb) with NaN for ignored lanes; n_steps = horizon in steps.

        lb_verified: the caller has already run the lower bounds and none fired,
        so the lower-bound trial is not repeated."""
        lb = (self.lb_initial if lb is None else lb).clone()
        ub = (self.ub_initial if ub is None else ub).clone()
        ignore = torch.zeros(self.B, dtype=torch.bool, device=self.pop.device)
        everyone = ~ignore
        tries = 0
        while True:  # fix bounds
            active = self.check_active(ub, everyone & ~ignore, n_steps) | ignore
            if bool(active.all()):
                break
            if tries >= self.max_tries_bound_fix:
                failed = ~active
                ignore |= failed
                ub[failed] = 1.0
                lb[failed] = 1.0
                break
            ub = torch.where(~active, ub * self.fix_bound_up, ub)
            tries += 1
        if not lb_verified:
            act_lb = self.check_active(lb, ~ignore, n_steps) & ~ignore
        else:
            act_lb = torch.zeros_like(ignore)
        if bool(act_lb.any()):
            raise RuntimeError("Some lower bounds are active. Cannot proceed with bisection.")
        msk = self._tolerance_open(lb, ub) & ~ignore
        tries = 0
        while bool(msk.any()) and tries < self.max_tries_thresh:
            stim = (ub + lb) / 2
            fired = self.check_active(stim, msk, n_steps)
            ub = torch.where(msk & fired, stim, ub)
            lb = torch.where(msk & ~fired, stim, lb)
            msk = self._tolerance_open(lb, ub) & ~ignore
            tries += 1
        ignore |= msk
        ub = torch.where(ignore, torch.full_like(ub, float("nan")), ub)
        lb = torch.where(ignore, torch.full_like(lb, float("nan")), lb)
        return ub, lb


def horizon_steps(pw_max_ms, dt=0.005, extra_ms=4.0):
    """Trial horizon: the longest pulse plus 4 ms, in steps."""
    return int(np.ceil((float(pw_max_ms) + extra_ms) / dt))


def learned_thresholds(th: Thresholder, pred_ma, margin, n_steps, max_lb_fix=10):
    """Thresholds from a proposed bracket, confirmed by the same bisection.

    The bracket is ``pred * exp(-margin) .. pred * exp(margin)``.  Lanes whose
    lower end fires are moved down (halved) until it does not; the upper end
    goes through the Thresholder's bound fixing (doubling) as usual.  The
    bisection then narrows every lane to the tolerance, so the result satisfies
    exactly the same acceptance rule as plain bisection.  Returns (ub, lb).
    """
    pred = torch.as_tensor(pred_ma, dtype=torch.float64, device=th.pop.device)
    lb = pred * float(np.exp(-margin))
    ub = pred * float(np.exp(margin))
    lanes = torch.ones(th.B, dtype=torch.bool, device=th.pop.device)
    verified = False
    for _ in range(max_lb_fix):
        bad = th.check_active(lb, lanes, n_steps)
        if not bool(bad.any()):
            verified = True
            break
        ub = torch.where(bad, lb, ub)  # a firing lower end is a valid upper end
        lb = torch.where(bad, lb * 0.5, lb)
        lanes = bad
    # lower ends of lanes whose upper end fails get replaced by a verified
    # inactive value inside bound fixing (ub only grows), so they stay valid
    return th.calculate_thresholds(n_steps, lb=lb, ub=ub, lb_verified=verified)
