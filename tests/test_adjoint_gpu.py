"""Hand-written adjoint kernels against the reference's autograd gradient, the
oracle's reverse mode and central finite differences."""

import numpy as np
import pytest
import torch

import oracle
from dendra_gb300.adjoint import CableGradient, cable_traces
from dendra_gb300.cable import CablePopulation
from dendra_gb300.workloads import RHOE_OHM_CM
from tests._cases import golden_adjoint_population, oracle_param_grads, synthetic_population

pytestmark = pytest.mark.gpu

PARAMS = ("gnabar", "gkbar", "gl", "rhoa")


def _fit_step(run, g, cuda, dtype=torch.float64):
    prm = {k: torch.as_tensor(g[f"guess_{k}"], dtype=dtype, device=cuda).requires_grad_()
           for k in PARAMS}
    trace = cable_traces(run, prm["gnabar"], prm["gkbar"], prm["gl"], prm["rhoa"])
    target = torch.as_tensor(g["target"], device=cuda, dtype=trace.dtype)
    loss = ((trace - target) ** 2).mean(dim=1).sum()
    loss.backward()
    return trace, loss, {k: prm[k].grad.double().cpu().numpy() for k in PARAMS}


@pytest.mark.parametrize("every", [400, 150, 7])
def test_float64_gradient_matches_reference_autograd(golden, cuda, every):
    g = golden("adjoint_f64.npz")
    pop = golden_adjoint_population(g, torch.float64, device=cuda)
    run = CableGradient(pop, int(g["steps"]), rec_idx=0, checkpoint_every=every)
    trace, loss, grads = _fit_step(run, g, cuda)
    np.testing.assert_allclose(trace.detach().cpu().numpy(), g["trace"], rtol=0, atol=1e-7)
    np.testing.assert_allclose(float(loss.detach()), g["loss"].sum(), rtol=1e-8)
    for k in PARAMS:
        np.testing.assert_allclose(grads[k], g[f"grad_{k}"], rtol=1e-6, err_msg=k)


@pytest.mark.parametrize("fast", [False, True])
def test_float32_gradient_is_close_to_the_float64_reference(golden, cuda, fast):
    g = golden("adjoint_f64.npz")
    pop = golden_adjoint_population(g, torch.float32, device=cuda, fast_math=fast)
    run = CableGradient(pop, int(g["steps"]), rec_idx=0, checkpoint_every=100)
    _, _, grads = _fit_step(run, g, cuda, torch.float32)
    for k in PARAMS:
        ref = g[f"grad_{k}"]
        err = np.abs(grads[k] - ref).max() / np.abs(ref).max()
        assert err <= 2e-2, (k, err, grads[k], ref)


def _ragged_population(cuda, dtype, compress_uniform=True, planes=True, fast_math=False):
    """Ragged cables (K = 1 .. 200), per-compartment channel densities and
    geometry, extracellular point source plus a somatic current clamp."""
    rng = np.random.default_rng(11)
    ks = [1, 2, 3, 31, 32, 33, 64, 65, 101, 200]
    N = sum(ks)
    diam = rng.uniform(0.8, 2.0, N) if planes else np.repeat(rng.uniform(0.8, 2.0, len(ks)), ks)
    dx = np.repeat(rng.uniform(8.0, 15.0, len(ks)), ks)
    scale = rng.uniform(0.8, 1.2, N) if planes else np.ones(N)
    hh = {"gnabar": 0.12 * scale, "gkbar": 0.036 * scale[::-1].copy(), "gl": 0.0003 * scale}
    pop = CablePopulation(ks, torch.as_tensor(diam), torch.as_tensor(dx),
                          rhoa=torch.as_tensor(rng.uniform(80, 120, len(ks))), celsius=6.3,
                          v_init=-65.0, dtype=dtype, device=cuda, hh=hh,
                          compress_uniform=compress_uniform, fast_math=fast_math)
    x = pop.positions()
    cab = np.repeat(np.arange(len(ks)), ks)
    r_cm = torch.sqrt(x ** 2 + torch.as_tensor(rng.uniform(300, 800, len(ks))[cab]) ** 2) * 1e-4
    pop.set_extracellular(RHOE_OHM_CM / (4 * torch.pi * r_cm),
                          torch.as_tensor(-rng.uniform(0.02, 0.2, len(ks))), 1.0, 0.2)
    pop.inject(0, torch.as_tensor(rng.uniform(0.1, 0.4, len(ks)) * 1e-6), 2.0, 3.0)
    return pop.initialize(0.025)


def test_float64_adjoint_matches_the_oracle_on_ragged_cables(cuda):
    steps = 300
    pop = _ragged_population(cuda, torch.float64)
    p = pop.problem_dict()
    run = CableGradient(pop, steps, rec_idx=0, checkpoint_every=64)
    trace = run.forward()
    rng = np.random.default_rng(5)
    tg = rng.standard_normal(tuple(trace.shape))
    per = run.backward(torch.as_tensor(tg))
    p["rec_idx"] = np.zeros(pop.B, dtype=np.int32)
    ref = oracle.cable_grad(p, steps, tg)
    got = {"lam_v": run.lam0[0], "lam_m": run.lam0[1], "lam_h": run.lam0[2],
           "lam_n": run.lam0[3], "g_gnabar": run.grad_comp[0], "g_gkbar": run.grad_comp[1],
           "g_gl": run.grad_comp[2], "g_axial": run.grad_axial}
    for k, v in got.items():
        v = v.cpu().numpy()
        scale = np.abs(ref[k]).max()
        np.testing.assert_allclose(v, ref[k], rtol=1e-7, atol=1e-9 * scale, err_msg=k)
    assert per["gnabar"].shape == (pop.B,)


def test_uniform_compression_gives_the_same_gradient(cuda):
    steps = 120
    out = []
    for compress in (True, False):
        pop = _ragged_population(cuda, torch.float32, compress_uniform=compress, planes=False)
        if compress:
            assert pop.uniform_channels and pop.uniform_geometry
        run = CableGradient(pop, steps, checkpoint_every=50)
        trace = run.forward()
        run.backward(torch.ones_like(trace))
        out.append((run.lam0.clone(), run.grad_comp.clone(), run.grad_axial.clone()))
    for a, b in zip(*out):
        assert torch.equal(a, b)


@pytest.mark.parametrize("fast", [False, True])
def test_checkpoint_interval_and_stream_overlap_do_not_change_the_gradient(cuda, fast):
    steps = 200
    res = []
    for every, overlap in ((200, True), (64, True), (64, False), (1, True)):
        pop = _ragged_population(cuda, torch.float32, fast_math=fast)
        run = CableGradient(pop, steps, checkpoint_every=every, overlap=overlap)
        trace = run.forward()
        run.backward(torch.linspace(-1, 1, trace.numel(), device=cuda).reshape(trace.shape))
        res.append((trace, run.lam0, run.grad_comp, run.grad_axial))
    for other in res[1:]:
        for a, b in zip(res[0], other):
            assert torch.equal(a, b)


def test_gpu_gradient_matches_central_differences_of_the_gpu_forward(golden, cuda):
    """h = 1e-4 relative central differences of the product's own float64 forward."""
    g = golden("adjoint_f64.npz")
    steps = int(g["steps"])
    pop = golden_adjoint_population(g, torch.float64, device=cuda)
    run = CableGradient(pop, steps, rec_idx=0, checkpoint_every=128)
    _, _, grads = _fit_step(run, g, cuda)
    target = torch.as_tensor(g["target"], device=cuda)
    base = {k: torch.as_tensor(g[f"guess_{k}"], device=cuda) for k in PARAMS}
    h = 1e-4
    for k in PARAMS:
        losses = []
        for sgn in (1, -1):
            prm = dict(base)
            prm[k] = base[k] * (1 + sgn * h)
            run.set_params(prm["gnabar"], prm["gkbar"], prm["gl"], prm["rhoa"])
            tr = run.forward()
            losses.append(((tr - target) ** 2).mean(dim=1).cpu().numpy())
        fd = (losses[0] - losses[1]) / (2 * h * g[f"guess_{k}"])
        np.testing.assert_allclose(grads[k], fd, rtol=1e-5, atol=1e-5 * np.abs(fd).max(),
                                   err_msg=k)


def test_oracle_param_grads_helper_agrees_with_gpu_per_cable_sums(golden, cuda):
    g = golden("adjoint_f64.npz")
    pop = golden_adjoint_population(g, torch.float64, device=cuda)
    p = pop.problem_dict()
    p["rhoa_per_cable"] = g["guess_rhoa"]
    _, _, ref, _ = oracle_param_grads(p, int(g["steps"]), g["target"])
    run = CableGradient(pop, int(g["steps"]), rec_idx=0, checkpoint_every=100)
    _, _, grads = _fit_step(run, g, cuda)
    for k in PARAMS:
        np.testing.assert_allclose(grads[k], ref[k], rtol=1e-7, err_msg=k)


def test_fast_math_float32_adjoint_tracks_the_float64_oracle(cuda):
    """Ragged cables with every optional plane: the fast float32 gradient against
    the float64 oracle's reverse mode of the same (float32-rounded) problem."""
    from tests._cases import as_f64

    steps = 300
    pop = _ragged_population(cuda, torch.float32, fast_math=True)
    p = as_f64(pop.problem_dict())
    run = CableGradient(pop, steps, rec_idx=0, checkpoint_every=64)
    trace = run.forward()
    rng = np.random.default_rng(5)
    tg = rng.standard_normal(tuple(trace.shape)).astype(np.float32)
    run.backward(torch.as_tensor(tg))
    p["rec_idx"] = np.zeros(pop.B, dtype=np.int32)
    ref = oracle.cable_grad(p, steps, tg.astype(np.float64), gate_f32=True)
    got = {"g_gnabar": run.grad_comp[0], "g_gkbar": run.grad_comp[1], "g_gl": run.grad_comp[2],
           "g_axial": run.grad_axial, "lam_v": run.lam0[0]}
    for k, v in got.items():
        v = v.double().cpu().numpy()
        err = np.abs(v - ref[k]).max() / np.abs(ref[k]).max()
        assert err <= 5e-3, (k, err)


def test_tape_stage_wait_timeout_surfaces(cuda):
    """A tape-stage wait limited to zero polls gives up at once: each warp
    drains its posted copies at the full limit, sets error bit 4 and ends;
    backward() raises, and with the default restored the same gradient comes
    out on the same context.  The copies are real, in-bounds bulk loads:
    nothing faults or hangs."""
    from dendra_gb300 import _lib

    L = _lib.load()
    pop = synthetic_population(7, 64, 51, 201, torch.float32, cuda, fast_math=True)
    run = CableGradient(pop, 200, rec_idx=0, checkpoint_every=100, tune=False)
    g = torch.ones_like(run.forward())
    want = run.backward(g)
    try:
        assert L.dgb_cable_adjoint_set_wait_limit(0) == 0
        with pytest.raises(RuntimeError, match="error bits 0x4"):
            run.backward(g)
    finally:
        assert L.dgb_cable_adjoint_set_wait_limit(-1) == 0
    got = run.backward(g)
    for k in want:
        torch.testing.assert_close(got[k], want[k], rtol=0, atol=0)
