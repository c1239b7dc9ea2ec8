"""Population.run-level drop-in for plain unbranched HH populations.

The reference advances a model one step per Python iteration
(models/core.py:4175 ``Population.run`` -> integrators/core.py:769-834 ->
integrators/implicit.py:569-664).  A persistent multi-step kernel can only
replace that loop as a whole, so this module takes the model itself:

    res = dropin.run(model, dt=0.025, steps=2000, extra=(space, mono_rect(...)),
                     record=Recorder-like, raster=Raster-like)

reads what the reference's model holds (``v``; per-compartment ``diam``,
``dx``, ``rhoa``, ``cm``; ``celsius``; ``mech.hh`` GLOBALs and gates m, h, n;
``injections`` of rectangular pulses; ``t``), runs every step in one
``dgb_cable_run`` launch and writes ``v``, ``m``, ``h``, ``n`` and ``t`` back
into the model, as the reference's own run leaves them.  The time grid is the
reference's: ``t_k = t + k dt`` in binary64, cast to the state dtype
(core.py:1280-1305).

Only the plain subset is accepted: the backward-Euler unbranched integrator,
the HH mechanism alone, at most one rectangular current clamp per cable at
the same compartment for every cable, an optional extracellular
``(space, rectangular pulse)``, a voltage Recorder and threshold rasters.
Anything else raises :class:`Unsupported` with the reason, or calls the
caller's ``fallback`` (for instance the model's own ``run``) when one is
given.  No CPU path exists here: the run itself is the CUDA kernel.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

from .cable import CablePopulation

PLAIN_INTEGRATORS = ("_bwd_euler_ub", "bwd_euler_ub")
RECT_WAVEFORMS = ("mono_rect",)


class Unsupported(ValueError):
    """The model lies outside the plain subset this drop-in replaces."""


@dataclass
class PlainCableSpec:
    """What the drop-in reads from a model, on the host."""

    n_comp: int
    n_cables: int
    dtype: torch.dtype
    diam: torch.Tensor
    dx: torch.Tensor
    rhoa: torch.Tensor
    cm: torch.Tensor
    celsius: float
    hh: dict
    state: dict
    t0: float
    clamp: tuple | None


def _as_tensor(x):
    return x.detach() if isinstance(x, torch.Tensor) else torch.as_tensor(x)


def _scalar(x, what):
    t = _as_tensor(x)
    if t.numel() != 1:
        if t.numel() and bool((t.reshape(-1) == t.reshape(-1)[0]).all()):
            return float(t.reshape(-1)[0])
        raise Unsupported(f"{what} must be uniform")
    return float(t)


def _rect(waveform, what):
    """(amp, delay, pw) of a rectangular pulse waveform."""
    if type(waveform).__name__ not in RECT_WAVEFORMS:
        raise Unsupported(f"{what}: only rectangular pulses ({', '.join(RECT_WAVEFORMS)}) are "
                          f"accepted, got {type(waveform).__name__}")
    params = getattr(waveform, "params", None)
    if not isinstance(params, dict) or not {"amp", "delay", "pw"} <= set(params):
        raise Unsupported(f"{what}: the pulse carries no amp/delay/pw parameters")
    return params["amp"], params["delay"], params["pw"]


def _mechanisms(model):
    mech = getattr(model, "mech", None)
    table = getattr(mech, "mechanisms", None)
    if table is None or not hasattr(table, "keys"):
        raise Unsupported("the model exposes no mechanism table")
    for extra in ("voltage_processes", "material_processes", "ions", "materials"):
        group = getattr(mech, extra, None)
        if group is not None and hasattr(group, "keys") and len(list(group.keys())):
            raise Unsupported(f"the model carries {extra}, which this drop-in does not model")
    return list(table.keys())


def plain_cable_spec(model) -> PlainCableSpec:
    """Read a model of the plain subset; raise Unsupported otherwise."""
    integ = type(getattr(model, "integrator", None)).__name__
    if integ not in PLAIN_INTEGRATORS:
        raise Unsupported(f"integrator {integ} is not the unbranched backward-Euler one")
    names = _mechanisms(model)
    if names != ["hh"]:
        raise Unsupported(f"mechanisms {names}: only hh alone is accepted")
    v = _as_tensor(model.v)
    if v.ndim != 2:
        raise Unsupported(f"v of shape {tuple(v.shape)}: only (cables, compartments) is accepted")
    if v.dtype not in (torch.float32, torch.float64):
        raise Unsupported(f"state dtype {v.dtype} is not float32 or float64")
    B, K = v.shape
    if K > 1024:
        raise Unsupported(f"{K} compartments per cable exceed the kernel's 1024")

    def field(name):
        t = _as_tensor(getattr(model, name)).to(torch.float64)
        if t.shape != (B, K):
            t = t.expand(B, K)
        return t.reshape(-1).to(v.dtype).cpu()

    hh = model.mech.hh
    gates = {k: _as_tensor(getattr(hh, k)) for k in ("m", "h", "n")}
    for k, g in gates.items():
        if g.shape != v.shape:
            raise Unsupported(f"hh.{k} of shape {tuple(g.shape)} does not match v")
    celsius = _scalar(getattr(model, "celsius"), "celsius")
    params = {k: _scalar(getattr(hh, k), f"hh.{k}") for k in
              ("gnabar", "gkbar", "gl", "el", "ena", "ek")}
    clamp = None
    injections = list(getattr(model, "injections", []) or [])
    if len(injections) > 1:
        raise Unsupported("more than one injection")
    if injections:
        wave, _, index = injections[0]
        if not (isinstance(index, tuple) and len(index) == 2 and index[0] is Ellipsis
                and isinstance(index[1], int)):
            raise Unsupported(f"injection index {index!r}: only model[..., i] is accepted")
        amp, delay, pw = _rect(wave, "injection")
        if _as_tensor(amp).numel() not in (1, B):
            raise Unsupported("injection amplitude must be scalar or one per cable")
        # Python numbers stay numbers: the pulse holds them as float32 values
        clamp = (index[1] % K, amp if isinstance(amp, (int, float)) else
                 _as_tensor(amp).to(torch.float64).reshape(-1).expand(B).clone(), delay, pw)
    return PlainCableSpec(
        n_comp=K, n_cables=B, dtype=v.dtype, diam=field("diam"), dx=field("dx"),
        rhoa=field("rhoa"), cm=field("cm"), celsius=celsius, hh=params,
        state={"v": v, **gates}, t0=float(_as_tensor(getattr(model, "t", 0.0))), clamp=clamp)


@dataclass
class DropinResult:
    """Recordings of one drop-in run: ``v`` (T+1, cables, compartments) when a
    voltage recording was asked for (every ``record_every`` steps, at
    ``record_nodes`` or all compartments), and the raster (RasterState)."""

    v: torch.Tensor | None
    raster: object | None


def run(model, dt, steps=None, duration=None, *, extra=None, record=None, raster=None,
        spk_thr=0.0, raster_cap=256, device="cuda", fallback=None, fast_math=False):
    """Advance ``model`` like its ``run(dt=..., steps=... | duration=...)``
    would, on the GPU in one persistent launch, and write its state back.

    extra: ``(space, pulse)`` with space (cables, compartments) in mV per unit
    amplitude and a rectangular pulse (the reference's ``extra=`` argument).
    record: a Recorder-like object with ``states == ("v",)``, optional
    ``node_indices`` and ``save_every``; or True for every compartment.
    raster: a Raster/APCount-like object with ``node_check`` (and
    ``threshold``), or a list of compartments.
    fallback: called as ``fallback()`` when the model is outside the plain
    subset (else Unsupported is raised).
    """
    try:
        spec = plain_cable_spec(model)
        pulse = None
        if extra is not None:
            space, wave = extra
            amp, delay, pw = _rect(wave, "extra")
            space = _as_tensor(space)
            if space.numel() not in (spec.n_comp, spec.n_cables * spec.n_comp):
                raise Unsupported(f"extra space of shape {tuple(space.shape)} does not fit")
            if not isinstance(amp, (int, float)) and _as_tensor(amp).numel() not in (
                    1, spec.n_cables):
                raise Unsupported("extra amplitude must be scalar or one per cable")
            pulse = (space.expand(spec.n_cables, spec.n_comp).reshape(-1), amp, delay, pw)
        rec_nodes, rec_every = None, 1
        if record is not None and record is not False:
            if record is not True:
                states = tuple(getattr(record, "states", ("v",)))
                if states != ("v",):
                    raise Unsupported(f"recorded states {states}: only v is accepted")
                if getattr(record, "max_only", False):
                    raise Unsupported("max-only recording is not supported")
                idx = getattr(record, "node_indices", None)
                rec_nodes = None if idx is None else _as_tensor(idx).reshape(-1).long()
                rec_every = int(getattr(record, "save_every", None) or 1)
        checks, thr = None, float(spk_thr)
        if raster is not None:
            if hasattr(raster, "node_check"):
                checks = list(raster.node_check)
                thr = float(getattr(raster, "threshold", thr))
                if (float(getattr(raster, "t_start_check", 0.0)) != 0.0
                        or float(getattr(raster, "t_end_check", 1e9)) < 1e9):
                    raise Unsupported("raster windows are not supported")
            else:
                checks = list(raster)
            if not 1 <= len(checks) <= 4:
                raise Unsupported("1 to 4 raster compartments are accepted")
    except Unsupported:
        if fallback is not None:
            return fallback()
        raise
    if (steps is None) == (duration is None):
        raise ValueError("give exactly one of steps or duration")
    n_steps = int(steps) if steps is not None else int(np.floor(float(duration) / float(dt)
                                                                + 1e-9))
    B, K = spec.n_cables, spec.n_comp
    pop = CablePopulation([K] * B, spec.diam, spec.dx, rhoa=spec.rhoa, cm=spec.cm,
                          celsius=spec.celsius, dtype=spec.dtype, device=device,
                          hh={k: spec.hh[k] for k in ("gnabar", "gkbar", "gl", "el", "ena",
                                                      "ek")}, fast_math=fast_math)
    if pulse is not None:
        space, amp, delay, pw = pulse
        if not isinstance(amp, (int, float)):
            amp = _as_tensor(amp).double().reshape(-1).expand(B).cpu()
        pop.set_extracellular(space.to(spec.dtype).cpu(), amp, delay, pw)
    if spec.clamp is not None:
        i, amp, delay, pw = spec.clamp
        pop.inject(i, amp, delay, pw)
    pop.initialize(float(dt))
    dev = pop.device
    for k in ("v", "m", "h", "n"):  # the model's own state, not a fresh one
        getattr(pop, k).copy_(spec.state[k].reshape(-1).to(dev, spec.dtype))
    pop.t0_ms = spec.t0  # the reference's grid: t0 + k dt in binary64
    res = pop.run(n_steps, rec_every=rec_every, record_all=rec_nodes is not None or (
        record is not None and record is not False), raster=checks, raster_cap=raster_cap,
        spk_thr=thr)
    pop.check_status()
    # write the state back where the model keeps it
    with torch.no_grad():
        for k, dst in (("v", model.v), ("m", model.mech.hh.m), ("h", model.mech.hh.h),
                       ("n", model.mech.hh.n)):
            dst.copy_(getattr(pop, k).reshape(B, K).to(dst.device, dst.dtype))
        t = getattr(model, "t", None)
        new_t = spec.t0 + n_steps * float(dt)
        if isinstance(t, torch.Tensor):
            t.fill_(new_t)
        else:
            model.t = new_t
    v = None
    if res.trace_all is not None:
        v = res.trace_all.reshape(-1, B, K)
        if rec_nodes is not None:
            v = v[:, :, rec_nodes.to(v.device)]
    return DropinResult(v, res.raster)
