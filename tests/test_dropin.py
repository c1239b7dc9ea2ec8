"""The Population.run-level drop-in (dendra_gb300.dropin).

A stand-in model carries the attributes the reference's unbranched models hold
(v; per-compartment diam, dx, rhoa, cm; celsius; mech.hh GLOBALs and gates;
injections; integrator; t).  On the CPU: what the adapter reads and what it
refuses.  On the GPU: the reference's recorded run (hh_cable_f64.npz) through
the adapter, the state written back into the model, and, where the installed
reference is importable, a reference model against its own run.
"""

import os
import sys
from types import SimpleNamespace

import numpy as np
import pytest
import torch

from dendra_gb300 import dropin
from dendra_gb300.cable import HH_DEFAULTS, hh_steady_state

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class _bwd_euler_ub:  # the reference integrator's class name
    pass


class mono_rect:  # the reference waveform's class name, its params dict
    def __init__(self, amp, delay, pw):
        self.params = {"amp": amp, "delay": delay, "pw": pw, "tau": 0.1}


class exp2syn:
    pass


def stand_in(B, K, diam=1.0, dx=10.0, dtype=torch.float64, clamp=None):
    v = torch.full((B, K), -65.0, dtype=dtype)
    m, h, n = (x.reshape(B, K) for x in hh_steady_state(v.reshape(-1)))
    hh = SimpleNamespace(m=m, h=h, n=n, **{k: torch.tensor(HH_DEFAULTS[k], dtype=torch.float64)
                                          for k in ("gnabar", "gkbar", "gl", "el", "ena", "ek")})
    mech = SimpleNamespace(mechanisms={"hh": hh}, voltage_processes={}, material_processes={},
                           ions={}, materials={}, hh=hh)
    full = lambda x: torch.full((B, K), float(x), dtype=dtype)  # noqa: E731
    model = SimpleNamespace(v=v, diam=full(diam), dx=full(dx), rhoa=full(100.0), cm=full(1.0),
                            celsius=torch.tensor(6.3, dtype=torch.float64),
                            t=torch.tensor(0.0, dtype=torch.float64), mech=mech,
                            integrator=_bwd_euler_ub(), injections=[])
    if clamp is not None:
        model.injections = [(clamp, torch.Size([B]), (Ellipsis, 0))]
    return model


def test_reads_the_plain_subset():
    amp = torch.tensor([[1e-6], [2e-6], [3e-6]], dtype=torch.float64)
    model = stand_in(3, 21, clamp=mono_rect(amp, 1.0, 0.5))
    spec = dropin.plain_cable_spec(model)
    assert (spec.n_cables, spec.n_comp) == (3, 21)
    assert spec.clamp[0] == 0 and spec.clamp[1].tolist() == [1e-6, 2e-6, 3e-6]
    assert spec.hh["gnabar"] == HH_DEFAULTS["gnabar"] and spec.celsius == 6.3
    assert spec.diam.shape == (63,) and spec.t0 == 0.0


@pytest.mark.parametrize("change, reason", [
    (lambda m: setattr(m, "integrator", object()), "integrator"),
    (lambda m: m.mech.mechanisms.update(syn=exp2syn()), "mechanisms"),
    (lambda m: m.mech.ions.update(na=object()), "ions"),
    (lambda m: setattr(m, "v", m.v.reshape(1, 3, 21)), "shape"),
    (lambda m: setattr(m, "injections", [(object(), None, (Ellipsis, 0))]), "rectangular"),
    (lambda m: setattr(m, "injections", [(mono_rect(1.0, 0.0, 1.0), None, (0, 0))]), "index"),
    (lambda m: setattr(m, "celsius", torch.tensor([6.3, 20.0])), "celsius"),
])
def test_refuses_outside_the_subset(change, reason):
    model = stand_in(3, 21)
    change(model)
    with pytest.raises(dropin.Unsupported, match=reason):
        dropin.plain_cable_spec(model)
    # with a fallback the caller's own path runs instead (no GPU is touched)
    assert dropin.run(model, 0.025, steps=10, fallback=lambda: "fallback") == "fallback"


@pytest.mark.gpu
def test_reference_recording_through_the_dropin(cuda, golden):
    """hh_cable_f64.npz: the reference's Recorder(v) of 3 cables x 101 compartments,
    somatic clamp, 800 steps; the state written back equals its final state."""
    g = golden("hh_cable_f64.npz")
    B, K = int(g["B"]), int(g["K"])
    amp = torch.as_tensor(g["amp_ma"]).reshape(B, 1)
    model = stand_in(B, K, float(g["diam"]), float(g["dx"]),
                     clamp=mono_rect(amp, float(g["delay"]), float(g["pw"])))
    res = dropin.run(model, float(g["dt"]), steps=int(g["steps"]), record=True,
                     raster=[0], device=cuda)
    v = res.v.cpu().numpy()[:, :, g["trace_comps"]]
    assert np.abs(v - g["v_trace"]).max() < 1e-7
    np.testing.assert_allclose(model.v.numpy(), g["v_final"], rtol=0, atol=1e-7)
    for k in ("m", "h", "n"):
        np.testing.assert_allclose(getattr(model.mech.hh, k).numpy(), g[f"{k}_final"], rtol=0,
                                   atol=1e-9)
    assert float(model.t) == pytest.approx(int(g["steps"]) * float(g["dt"]))
    up = (g["v_trace"][1:, :, 0] >= 0) & (g["v_trace"][:-1, :, 0] < 0)
    np.testing.assert_array_equal(res.raster.count.cpu().numpy()[:, 0], up.sum(0))


_CHILD = r"""
import json, sys, warnings
import numpy as np, torch
warnings.filterwarnings("ignore")
import importlib.util, types
if importlib.util.find_spec("networkx") is None:
    sys.modules["networkx"] = types.ModuleType("networkx")
import dendra as dn
from dendra.models.mod import hh
from dendra_gb300 import dropin

def build():
    with dn.ctx(JIT=0):
        m = dn.Unmyelinated([1.0, 2.0, 3.0], L=600.0, dx=10.0, celsius=6.3, v_init=-65.0,
                            dtype=torch.float64, integrator=dn.bwd_euler_ub(), rhoa=100.0)
        m.insert(hh)
        m[..., 0].inject(dn.mono_rect(amp=torch.tensor([[2e-7], [5e-7], [1e-6]],
                                                       dtype=torch.float64), delay=1.0, pw=1.0))
        m.initialize()
    return m

K = build().v.shape[-1]
x = (torch.arange(K, dtype=torch.float64) - (K - 1) / 2) * 10.0
space = (-333.33 / (4 * np.pi * torch.sqrt(x ** 2 + 400.0 ** 2) * 1e-4)).expand(3, K).contiguous()
ours, theirs = build(), build()
steps, dt = 400, 0.025
res = dropin.run(ours, dt, steps=steps, record=True,
                 extra=(space, dn.mono_rect(amp=0.5, delay=2.0, pw=0.2)), device="cuda")
rec = dn.Recorder(("v",))
with dn.ctx(JIT=0):
    theirs.run(dt=dt, steps=steps, callbacks=[rec],
               extra=(space, dn.mono_rect(amp=0.5, delay=2.0, pw=0.2)))
ref = torch.stack([t.reshape(3, K) for t in rec.rec["v"]]).numpy()
print(json.dumps({"trace": float(np.abs(res.v.cpu().numpy() - ref).max()),
                  "final": float((ours.v - theirs.v).abs().max()),
                  "t": [float(ours.t), float(theirs.t)], "vmax": float(ref.max())}))
"""


@pytest.mark.gpu
def test_reference_model_against_its_own_run(cuda):
    """A reference Unmyelinated model (HH, somatic clamp, extracellular pulse)
    through the drop-in against the same model's own CPU run.  Runs in a child
    process: the reference imports with small torch.library shims that must
    not touch this process."""
    import json
    import subprocess

    ref = os.path.join(ROOT, "baseline", "_ref")
    shim = os.path.join(ROOT, "tests", "golden", "refshim")
    if not os.path.isdir(os.path.join(ref, "dendra")):
        pytest.skip("the reference is not installed in baseline/_ref")
    env = dict(os.environ, PYTHONPATH=os.pathsep.join([ref, shim, ROOT]))
    r = subprocess.run([sys.executable, "-c", _CHILD], env=env, capture_output=True, text=True,
                       timeout=600)
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    if r.returncode != 0 or not lines:
        tail = (r.stderr or r.stdout).strip().splitlines()[-1:]
        if "dendra" in (r.stderr or "") and "Error" in (r.stderr or "") and "dropin" not in (
                r.stderr or ""):
            pytest.skip(f"the reference does not run here: {tail}")
        raise AssertionError(f"child failed ({r.returncode}): {r.stderr[-2000:]}")
    out = json.loads(lines[-1])
    print("reference model through the drop-in:", out)
    assert out["vmax"] > 0  # the clamp and the pulse drive spikes
    assert out["trace"] < 1e-7 and out["final"] < 1e-7
    assert out["t"][0] == pytest.approx(out["t"][1])
