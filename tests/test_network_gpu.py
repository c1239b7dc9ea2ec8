"""Branched-cell spiking network on the GPU against the float64 network oracle."""

import numpy as np
import pytest
import torch

import oracle
from dendra_gb300.network import random_network

pytestmark = pytest.mark.gpu


def _raster(r, window=None):
    return r.cpu().numpy()


def _ref64(dtype, seed, **kw):
    net, n_steps = random_network(16, k_range=(30, 400), syn_per_cell=12, seed=seed, dtype=dtype,
                                  device="cpu", t_stop_ms=60.0, **kw)
    pd = net.problem_dict(n_steps)
    if dtype == torch.float32:  # float64 reference on the float32 network's inputs
        for grp in ("nodes", "syn"):
            pd[grp] = {k: v.astype(np.float64) for k, v in pd[grp].items()}
        for k in ("v", "m", "h", "n", "A", "B", "ring"):
            pd[k] = pd[k].astype(np.float64)
    raster = oracle.net_run(pd, n_steps)
    return pd, raster, n_steps


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("seed", [3, 8])
def test_network_matches_oracle(cuda, dtype, seed):
    kw = dict(bg_weight=0.05)
    pd, ref_raster, n_steps = _ref64(dtype, seed, **kw)
    net, _ = random_network(16, k_range=(30, 400), syn_per_cell=12, seed=seed, dtype=dtype,
                            device=cuda, t_stop_ms=60.0, **kw)
    bits = net.run(n_steps)
    raster = _raster(bits, net.window)
    assert ref_raster.sum() > 0  # the case has spikes
    # spike routing: which cell fires at which step, exactly
    np.testing.assert_array_equal(raster, ref_raster)
    np.testing.assert_array_equal(net.spike_count.cpu().numpy(), pd["spike_count"])
    v = net.v.double().cpu().numpy()
    tol = 1e-9 if dtype == torch.float64 else 1e-3
    assert np.abs(v - pd["v"]).max() < tol
    # float32: 2400 rounded decay multiplies accumulate a few 1e-6 relative
    np.testing.assert_allclose(net.B.double().cpu().numpy(), pd["B"], rtol=1e-4 if dtype ==
                               torch.float32 else 1e-12, atol=1e-12)
    assert int(net.slot) == pd["slot"]


def test_network_window_split_is_exact(cuda):
    """One long run equals the same steps in several calls (ring and slot carried)."""
    a, n = random_network(8, k_range=(30, 200), syn_per_cell=6, seed=5, dtype=torch.float64,
                          device=cuda, t_stop_ms=40.0, bg_weight=0.05)
    b, _ = random_network(8, k_range=(30, 200), syn_per_cell=6, seed=5, dtype=torch.float64,
                          device=cuda, t_stop_ms=40.0, bg_weight=0.05)
    ra = _raster(a.run(n), a.window)
    rb = np.concatenate([_raster(b.run(n // 2), b.window), _raster(b.run(n // 2), b.window)])
    np.testing.assert_array_equal(ra, rb)
    torch.testing.assert_close(a.v, b.v, rtol=0, atol=0)


def test_chain_and_layer_schedules_give_identical_runs(cuda):
    from dendra_gb300.network import random_network

    out = []
    for chains in (True, False):
        net, n = random_network(40, k_range=(100, 900), syn_per_cell=20, seed=12,
                                dtype=torch.float32, device=cuda, t_stop_ms=25.0,
                                rate_hz=40.0, chains=chains)
        out.append((net.run(n), net.v.clone(), net.A.clone(), net.B.clone()))
    for a, b in zip(*out):
        assert torch.equal(a, b)
    assert int(out[0][0].sum()) > 0


@pytest.mark.parametrize("dtype", [torch.float64])
def test_network_with_device_netstim_background(cuda, dtype):
    """Background events generated on the device by a NetStim per cell; the
    oracle runs on the same event bits (read back from the device)."""
    net, n_steps = random_network(16, k_range=(30, 400), syn_per_cell=12, seed=4, dtype=dtype,
                                  device=cuda, t_stop_ms=60.0, bg_weight=0.05, rate_hz=40.0,
                                  bg="netstim")
    pd = net.problem_dict(n_steps)
    assert pd["bg_bits"] is not None and int(np.unpackbits(pd["bg_bits"].view(np.uint8)).sum())
    if dtype == torch.float32:
        for grp in ("nodes", "syn"):
            pd[grp] = {k: v.astype(np.float64) for k, v in pd[grp].items()}
        for k in ("v", "m", "h", "n", "A", "B", "ring"):
            pd[k] = pd[k].astype(np.float64)
    ref = oracle.net_run(pd, n_steps)
    raster = net.run(n_steps).cpu().numpy()
    assert ref.sum() > 0
    np.testing.assert_array_equal(raster, ref)


def _driven(device, dtype=torch.float64):
    """Branched cells with an extracellular pulse (a point-like field over each
    tree's nodes) and a clamp at a dendritic node: the tree step's edge
    currents g (ve_child - ve_parent) and injected current."""
    from dendra_gb300.network import TreeNetwork, random_cell

    rng = np.random.default_rng(17)
    cells = [random_cell(rng, int(rng.integers(40, 160))) for _ in range(6)]
    N = sum(c.parent.size for c in cells)
    syn_node = [np.array([0, 1]) for _ in cells]
    pre = rng.integers(0, len(cells), 12)
    post = np.arange(12)
    field = -rng.uniform(50.0, 400.0, N)  # mV per mA, cathodic
    amp = rng.uniform(0.5, 2.0, len(cells))
    node = [int(rng.integers(1, c.parent.size)) for c in cells]
    return TreeNetwork(cells, syn_node, pre, post, rng.uniform(1.0, 3.0, 12),
                       rng.lognormal(-6.0, 0.5, 12), dt=0.025, dtype=dtype, device=device,
                       extracellular=(field, amp, 1.0, 0.3),
                       clamp=(node, rng.uniform(0.5, 2.0, len(cells)) * 1e-6, 2.0, 3.0))


def test_tree_step_drive_matches_oracle(cuda):
    """Extracellular edge currents and the injected current of the tree step
    (integrators/tree.py:1262-1302) against the oracle's restatement."""
    n_steps = 400
    ref64 = _driven("cpu")
    pd = ref64.problem_dict(n_steps)
    ref = oracle.net_run(pd, n_steps)
    net = _driven(cuda)
    raster = net.run(n_steps).cpu().numpy()
    assert ref.sum() > 0
    np.testing.assert_array_equal(raster, ref)
    assert np.abs(net.v.cpu().numpy() - pd["v"]).max() < 1e-9
    # the drive matters: without it the cells stay at rest
    quiet = _driven("cpu")
    quiet.drive = {}
    pq = quiet.problem_dict(n_steps)
    oracle.net_run(pq, n_steps)
    assert np.abs(pq["v"] - pd["v"]).max() > 1.0

@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_size_classes_give_identical_runs(cuda, dtype):
    """Cells of at most half the largest size run in their own window launch
    (smaller shared memory per cell, more cells per SM): the per-cell
    arithmetic is unchanged, so the run is identical bit for bit."""
    from dendra_gb300.network import random_network

    out = []
    for classes in (True, False):
        net, n = random_network(24, k_range=(60, 900), syn_per_cell=12, seed=21, dtype=dtype,
                                device=cuda, t_stop_ms=20.0, rate_hz=40.0,
                                size_classes=classes)
        assert (net.classes is not None) == classes
        out.append((net.run(n), net.v.clone(), net.A.clone(), net.spike_count.clone()))
    assert int(out[0][0].sum()) > 0
    for a, b in zip(*out):
        assert torch.equal(a, b)
