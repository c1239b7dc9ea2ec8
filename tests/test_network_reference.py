"""The network path pinned to the reference's own Network run.

network_points.npz records the reference (Network.run on the CPU, dense delay
ring) on 16 single-compartment HH cells with one Exp2Syn synapse each,
periodic NetStim drive through one-to-one NetCons (1 ms delay) and all-to-all
NetCons with lognormal weights and U[1, 5] ms delays.  The same network is
built here as a TreeNetwork of one-node cells; the NetStim emissions the
reference recorded, delayed by their NetCon's steps, are its background
events.  The oracle (CPU) and the GPU kernels must reproduce the reference's
spike steps exactly (which cell fires at which step: the routing of every
recurrent event shows in them), and its membrane potentials and synapse
states to rounding.

netcon_tapes.npz holds the reference's bit-pack known-answer tapes
(fan-in/out across the ring wrap, the 63-bit word boundary); the packing and
delivery kernels must reproduce the running ExpSyn conductance exactly.
"""

import numpy as np
import pytest
import torch

import oracle
from dendra_gb300.netcon import (DenseRing, build_delivery, inference_delay_steps, n_words_for,
                                 pack_source_spikes, source_word_and_mask)
from dendra_gb300.network import Cell, TreeNetwork


def point_network(g, dtype, device):
    N, dt = int(g["N"]), float(g["dt"])
    cells = [Cell(np.array([-1]), np.array([float(g["length"])]), np.array([float(g["diam"])]))
             for _ in range(N)]
    _, d_bg = inference_delay_steps(torch.tensor([float(g["d_bg"])]), dt)
    emitted = np.asarray(g["stim_emitted"], dtype=bool)
    bg_steps = [np.nonzero(emitted[:, c])[0] + int(d_bg[0]) for c in range(N)]
    return TreeNetwork(cells, [np.array([0])] * N, g["pre"], g["post"], g["delay"], g["weight"],
                       dt=dt, dtype=dtype, device=device, celsius=float(g["celsius"]),
                       v_init=float(g["v_init"]), tau1=float(g["tau1"]), tau2=float(g["tau2"]),
                       e_syn=float(g["e_syn"]), spk_thr=float(g["spk_thr"]), bg_steps=bg_steps,
                       bg_weight=float(g["w_bg"]))


def reference_raster(v, thr=0.0):
    """Rising edges of the recorded v at each step's start (the NetCon's
    detection on v before the population solve), latch starting below."""
    above = v[:-1] >= thr
    below_prev = np.vstack([np.ones((1, v.shape[1]), dtype=bool), v[:-2] < thr])
    return (above & below_prev).astype(np.uint8)


def test_oracle_network_matches_reference(golden):
    g = golden("network_points.npz")
    steps = int(g["steps"])
    net = point_network(g, torch.float64, "cpu")
    pd = net.problem_dict(steps)
    raster = oracle.net_run(pd, steps)
    ref = reference_raster(g["v"])
    assert ref.sum() >= 40
    np.testing.assert_array_equal(raster, ref)
    err = np.abs(pd["v"] - g["v"][-1]).max()
    print(f"oracle network vs reference: final max |dV| {err:.3e} mV")
    assert err < 1e-9
    np.testing.assert_allclose(pd["A"], g["A"][-1], rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(pd["B"], g["B"][-1], rtol=1e-12, atol=1e-15)


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_gpu_network_matches_reference(cuda, golden, dtype):
    g = golden("network_points.npz")
    steps = int(g["steps"])
    net = point_network(g, dtype, cuda)
    bits = net.run(steps).cpu().numpy()
    ref = reference_raster(g["v"])
    np.testing.assert_array_equal(bits, ref)
    v = net.v.double().cpu().numpy()
    err = np.abs(v - g["v"][-1]).max()
    print(f"GPU network {dtype} vs reference: final max |dV| {err:.3e} mV")
    # float32: the same spike steps; the potentials of spiking cells carry
    # float32 rounding amplified through action potentials (the stated
    # float32 tolerance for spiking traces, 2e-2 mV)
    assert err < (1e-9 if dtype == torch.float64 else 2e-2)
    rtol = 1e-12 if dtype == torch.float64 else 1e-4
    np.testing.assert_allclose(net.A.double().cpu().numpy(), g["A"][-1], rtol=rtol, atol=1e-15)
    np.testing.assert_allclose(net.B.double().cpu().numpy(), g["B"][-1], rtol=rtol, atol=1e-15)


def _tape_running_g(pre, post, weight, delay_ms, dt, tape, n_post, device, packed):
    """Running sum of the delivered weights per target after each step, through
    the bit-packed history (pack + build_delivery) or the dense ring."""
    _, steps = inference_delay_steps(torch.as_tensor(delay_ms), dt)
    depth = int(steps.max()) + 1
    pre_t = torch.as_tensor(pre, device=device)
    post_t = torch.as_tensor(post, device=device)
    w = torch.as_tensor(weight, dtype=torch.float64, device=device)
    g = torch.zeros(n_post, dtype=torch.float64, device=device)
    rows = []
    if packed:
        n_src = tape.shape[1]
        hist = torch.zeros((depth, n_words_for(n_src)), dtype=torch.int64, device=device)
        word, mask = source_word_and_mask(pre_t)
        d = steps.to(device)
        for s, spikes in enumerate(tape):
            t = torch.tensor([s % depth], device=device)
            pack_source_spikes(torch.as_tensor(spikes, device=device), hist, t)
            out = torch.zeros(n_post, dtype=torch.float64, device=device)
            build_delivery(hist, t, d, word, mask, post_t, w, out)
            g = g + out
            rows.append(g.clone())
    else:
        ring = DenseRing(depth, n_post, pre, post, steps.numpy(), weight, device=device,
                         dtype=torch.float64)
        for spikes in tape:
            g = g + ring.due()
            rows.append(g.clone())
            ring.transition(torch.as_tensor(spikes, device=device))
    return torch.stack(rows).cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("packed", [True, False])
def test_netcon_known_answer_tapes(cuda, golden, packed):
    g = golden("netcon_tapes.npz")
    dt = float(g["dt"])
    fan = _tape_running_g(g["fan_pre"], g["fan_post"], g["fan_weight"], g["fan_delay"], dt,
                          g["fan_tape"], 2, cuda, packed)
    np.testing.assert_array_equal(fan, g["fan_g_dense"])
    np.testing.assert_array_equal(fan, g["fan_g_bitpacked_history"])
    n = g["word_tape"].shape[1]
    word = _tape_running_g(np.arange(n), np.arange(n), np.ones(n), np.full(n, dt), dt,
                           g["word_tape"], n, cuda, packed)
    np.testing.assert_array_equal(word, g["word_g_dense"])
    np.testing.assert_array_equal(word, g["word_g_bitpacked_history"])


@pytest.mark.gpu
def test_uniform_delivery_word_boundary_tape(cuda, golden):
    """The 63-bit word-boundary tape (one delay for every connection) through
    build_delivery_uniform equals the reference's recorded conductance."""
    from dendra_gb300.netcon import build_delivery_uniform

    g = golden("netcon_tapes.npz")
    tape = g["word_tape"]
    n = tape.shape[1]
    depth = 2
    hist = torch.zeros((depth, n_words_for(n)), dtype=torch.int64, device=cuda)
    idx = torch.arange(n, device=cuda)
    word, mask = source_word_and_mask(idx)
    w = torch.ones(n, dtype=torch.float64, device=cuda)
    gsum = torch.zeros(n, dtype=torch.float64, device=cuda)
    rows = []
    for s, spikes in enumerate(tape):
        t = torch.tensor([s % depth], device=cuda)
        pack_source_spikes(torch.as_tensor(spikes, device=cuda), hist, t)
        out = torch.zeros(n, dtype=torch.float64, device=cuda)
        build_delivery_uniform(hist, t, 1, word, mask, idx, w, out)
        gsum = gsum + out
        rows.append(gsum.clone())
    np.testing.assert_array_equal(torch.stack(rows).cpu().numpy(), g["word_g_dense"])
