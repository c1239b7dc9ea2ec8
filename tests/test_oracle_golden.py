"""The CPU oracle against vectors produced by the reference itself (CPU only)."""

import numpy as np
import pytest
import torch

import oracle
from tests._cases import golden_cable_population, golden_extra_population, oracle_traces


@pytest.mark.parametrize("tag,dtype", [("f64", np.float64), ("f32", np.float32)])
def test_hh_rates_match_reference(golden, tag, dtype):
    g = golden("rates.npz")
    v = g[f"v_{tag}"]
    got = oracle.hh_rates(v, 1.0, dtype=dtype)
    ref = g[f"rates_{tag}"]
    tol = 1e-14 if tag == "f64" else 2e-6
    np.testing.assert_allclose(got, ref, rtol=tol, atol=tol * 1e-3)


@pytest.mark.parametrize("tag,dtype", [("f64", np.float64), ("f32", np.float32)])
def test_phi1_and_cnexp_match_reference(golden, tag, dtype):
    g = golden("rates.npz")
    np.testing.assert_array_equal(oracle.phi1(g[f"z_{tag}"], dtype=dtype), g[f"phi1_{tag}"])
    x, a, b = g[f"cnexp_in_{tag}"].T
    got = oracle.cnexp(x, a, b, dtype(0.025), dtype=dtype)
    tol = 1e-14 if tag == "f64" else 1e-6
    np.testing.assert_allclose(got, g[f"cnexp_out_{tag}"], rtol=tol, atol=tol)


@pytest.mark.parametrize("K", [1, 2, 3, 7, 33, 101, 401])
@pytest.mark.parametrize("tag,dtype", [("f64", np.float64), ("f32", np.float32)])
def test_thomas_and_pcr_match_reference(golden, K, tag, dtype):
    g = golden("tridiag.npz")
    a, b, c, d = (g[f"K{K}_{x}"].astype(dtype) for x in "abcd")
    th = oracle.thomas(a, b, c, d)
    pc = oracle.pcr(a, b, c, d)
    if tag == "f64":
        np.testing.assert_array_equal(th, g[f"K{K}_{tag}_thomas"])
        np.testing.assert_allclose(pc, g[f"K{K}_{tag}_pcr"], rtol=1e-13, atol=1e-14)
    else:
        np.testing.assert_allclose(th, g[f"K{K}_{tag}_thomas"], rtol=2e-6, atol=2e-6)
        np.testing.assert_allclose(pc, g[f"K{K}_{tag}_pcr"], rtol=2e-5, atol=2e-6)


def test_dhs_matches_reference_dense_solve(golden):
    g = golden("dhs.npz")
    for case in ("parity", "rand"):
        parent = g[f"{case}_parent"]
        x_ref = g[f"{case}_x"]
        threads = (1, 8, 32) if case == "parity" else (32,)
        for t in threads:
            order = g[f"{case}_order_t{t}"]
            lptr = g[f"{case}_layer_ptr_t{t}"]
            x = oracle.dhs_solve(g[f"{case}_d"], g[f"{case}_a"], g[f"{case}_b"], parent, order,
                                 lptr)
            np.testing.assert_allclose(x, x_ref, rtol=3e-12, atol=3e-12)


def _spike_steps(trace, thr=0.0):
    above = trace >= thr
    return [list(np.nonzero(above[1:, b] & ~above[:-1, b])[0] + 1) for b in range(trace.shape[1])]


@pytest.mark.parametrize("tag", ["f64", "f32"])
def test_cable_run_matches_reference_traces(golden, tag):
    """Oracle run of Unmyelinated+hh+bwd_euler_ub vs the reference's own run."""
    g = golden(f"hh_cable_{tag}.npz")
    dtype = torch.float64 if tag == "f64" else torch.float32
    pop = golden_cable_population(g, dtype)
    # initial gates: steady state at v_init like the reference
    m0 = pop.m.numpy().reshape(int(g["B"]), -1)
    tol0 = 1e-15 if tag == "f64" else 1e-7
    np.testing.assert_allclose(m0, g["m0"], rtol=tol0, atol=tol0)
    steps = int(g["steps"])
    tr, final, _ = oracle_traces(pop, steps, g["trace_comps"])
    ref = g["v_trace"]
    err = np.abs(tr - ref).max()
    # float64: identical arithmetic up to operation order; float32: rounding
    assert err <= (1e-9 if tag == "f64" else 2e-3), err
    for c in range(ref.shape[2]):
        assert _spike_steps(tr[:, :, c]) == _spike_steps(ref[:, :, c])
    assert any(len(s) for s in _spike_steps(ref[:, :, 0]))  # the case does spike
    vf = final["v"].reshape(int(g["B"]), -1)
    assert np.abs(vf - g["v_final"]).max() <= (1e-9 if tag == "f64" else 2e-3)


@pytest.mark.parametrize("tag", ["f64", "f32"])
def test_cable_run_with_extracellular_matches_reference(golden, tag):
    g = golden(f"hh_extra_{tag}.npz")
    dtype = torch.float64 if tag == "f64" else torch.float32
    pop = golden_extra_population(g, dtype)
    steps = int(g["steps"])
    tr, final, _ = oracle_traces(pop, steps, g["trace_comps"])
    ref = g["v_trace"]
    scale = max(1.0, np.abs(ref).max() / 100.0)
    err = np.abs(tr - ref).max()
    assert err <= (1e-9 if tag == "f64" else 5e-3) * scale, err
    for c in range(ref.shape[2]):
        assert _spike_steps(tr[:, :, c]) == _spike_steps(ref[:, :, c])


def test_oracle_float32_is_within_tolerance_of_float64(golden):
    """The float32 reference path and the float64 reference run differ by < 1e-3 mV·(scale)."""
    g64 = golden("hh_cable_f64.npz")
    g32 = golden("hh_cable_f32.npz")
    assert np.abs(g64["v_trace"] - g32["v_trace"]).max() < 0.05


@pytest.mark.parametrize("K", [1, 2, 3, 8, 33, 101, 257])
def test_block3_thomas_matches_reference_block_pcr(golden, K):
    """The oracle's 3x3 block Thomas against the reference's block PCR
    (tridiag/block.py) on the same systems (different elimination orders)."""
    g = golden("block3.npz")
    args = [g[f"K{K}_{n}"] for n in ("lower", "main", "upper", "rhs")]
    x64 = oracle.block3_solve(*args)
    np.testing.assert_allclose(x64, g[f"K{K}_x_f64"], rtol=1e-11, atol=1e-12)
    x32 = oracle.block3_solve(*(a.astype(np.float32) for a in args))
    np.testing.assert_allclose(x32, g[f"K{K}_x_f32"], rtol=1e-4, atol=1e-5)
