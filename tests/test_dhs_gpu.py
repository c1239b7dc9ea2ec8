"""DHS/Hines tree solves on the GPU against the reference's dense oracle and the C oracle."""

import numpy as np
import pytest
import torch

import oracle
from dendra_gb300.tree import (ForestPlan, build_dhs_layers, build_morphology, dhs_solve_cuda,
                               dhs_solve_forest)

pytestmark = pytest.mark.gpu

# tests/test_cuda_solver_parity.py:66-110 tolerances
TOL = {torch.float32: dict(rtol=5e-5, atol=5e-6), torch.float64: dict(rtol=3e-12, atol=3e-12)}


def _plan(parent, threads, dev):
    _, _, depth = build_morphology(list(parent))
    order, layer_ptr = build_dhs_layers(depth, threads)
    return (torch.as_tensor(np.asarray(parent), device=dev), order.to(dev).long(),
            layer_ptr.to(dev).long())


@pytest.mark.parametrize("threads", [1, 8, 32])
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_matches_reference_dense_oracle(cuda, golden, threads, dtype):
    g = golden("dhs.npz")
    for case in ("parity", "rand"):
        if case == "rand" and threads != 32:
            continue
        parent = g[f"{case}_parent"]
        d, a, b = (torch.as_tensor(g[f"{case}_{x}"]).to(cuda, dtype) for x in "dab")
        x = dhs_solve_cuda(d, a, b, *_plan(parent, threads, cuda), threads=threads)
        ref = torch.as_tensor(g[f"{case}_x"]).to(cuda, dtype)
        torch.testing.assert_close(x, ref, **TOL[dtype])


def _random_tree(rng, K, branch=8):
    """Random binary-branching tree with unbranched runs of ~branch nodes."""
    parent = [-1]
    tips = [0]
    while len(parent) < K:
        p = tips.pop(rng.integers(len(tips))) if tips else int(rng.integers(len(parent)))
        n = int(min(K - len(parent), rng.integers(1, 2 * branch)))
        prev = p
        for _ in range(n):
            parent.append(prev)
            prev = len(parent) - 1
        tips.append(prev)
        if len(parent) < K and rng.random() < 0.7:
            tips.append(p)
    return parent


@pytest.mark.parametrize("K", [1, 2, 37, 500, 2000])
def test_random_batches_match_oracle(cuda, K):
    rng = np.random.default_rng(K)
    parent = _random_tree(rng, K)
    B = 33
    d = 1.0 + rng.random((B, K))
    a = 0.5 * rng.random((B, K))
    a[:, 0] = 0.0
    b = rng.standard_normal((B, K))
    p, order, lptr = _plan(parent, 32, cuda)
    x = dhs_solve_cuda(*(torch.as_tensor(t, device=cuda) for t in (d, a, b)), p, order, lptr)
    ref = oracle.dhs_solve(d, a, b, np.asarray(parent), order.cpu().numpy(), lptr.cpu().numpy())
    np.testing.assert_allclose(x.cpu().numpy(), ref, rtol=1e-11, atol=1e-12)
    x32 = dhs_solve_cuda(*(torch.as_tensor(t, device=cuda).float() for t in (d, a, b)), p, order,
                         lptr)
    np.testing.assert_allclose(x32.cpu().numpy(), ref, rtol=5e-5, atol=5e-5)


def test_deterministic(cuda):
    rng = np.random.default_rng(1)
    parent = _random_tree(rng, 900)
    args = [torch.as_tensor(t, device=cuda, dtype=torch.float32) for t in (
        1.0 + rng.random((64, 900)), rng.random((64, 900)), rng.standard_normal((64, 900)))]
    plan = _plan(parent, 32, cuda)
    x0 = dhs_solve_cuda(*args, *plan)
    for _ in range(3):
        torch.testing.assert_close(dhs_solve_cuda(*args, *plan), x0, rtol=0, atol=0)


def test_gradients_match_dense_autograd(cuda, golden):
    g = golden("dhs.npz")
    parent = g["parity_parent"]
    d, a, b = (torch.as_tensor(g[f"parity_{x}"][:3]).to(cuda).requires_grad_() for x in "dab")
    w = torch.linspace(-1, 1, b.numel(), device=cuda, dtype=torch.float64).reshape(b.shape)
    x = dhs_solve_cuda(d, a, b, *_plan(parent, 32, cuda))
    (x * w).sum().backward()
    grads = [t.grad.clone() for t in (d, a, b)]
    for t in (d, a, b):
        t.grad = None
    M = torch.diag_embed(d + a)
    for child, p in enumerate(parent.tolist()):
        if p < 0:
            continue
        e = a[:, child]
        M = M + 0.0
        M[:, p, p] = M[:, p, p] + e
        M[:, child, p] = M[:, child, p] - e
        M[:, p, child] = M[:, p, child] - e
    xd = torch.linalg.solve(M, b.unsqueeze(-1)).squeeze(-1)
    (xd * w).sum().backward()
    for gk, t in zip(grads, (d, a, b)):
        torch.testing.assert_close(gk, t.grad, rtol=3e-10, atol=3e-10)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_forest_of_distinct_trees(cuda, dtype):
    rng = np.random.default_rng(7)
    sizes = [1, 2, 5, 200, 731, 2000, 64, 33]
    parents = [_random_tree(rng, K) for K in sizes]
    plan = ForestPlan(parents, device=cuda)
    N = plan.n_nodes
    d = 1.0 + rng.random(N)
    a = 0.5 * rng.random(N)
    b = rng.standard_normal(N)
    x = dhs_solve_forest(*(torch.as_tensor(t, device=cuda, dtype=dtype) for t in (d, a, b)), plan)
    x = x.double().cpu().numpy()
    for t, parent in enumerate(parents):
        lo, hi = plan.node_ptr[t], plan.node_ptr[t + 1]
        _, _, depth = build_morphology(parent)
        order, lptr = build_dhs_layers(depth, 32)
        aa = a[lo:hi].copy()
        ref = oracle.dhs_solve(d[None, lo:hi], aa[None], b[None, lo:hi], np.asarray(parent),
                               order.numpy(), lptr.numpy())[0]
        tol = dict(rtol=1e-11, atol=1e-12) if dtype == torch.float64 else dict(rtol=5e-5, atol=5e-5)
        np.testing.assert_allclose(x[lo:hi], ref, **tol)


def test_contract_errors(cuda):
    d = torch.ones(2, 3, device=cuda)
    plan = _plan([-1, 0, 0], 32, cuda)
    with pytest.raises(ValueError, match="CUDA"):
        dhs_solve_cuda(d.cpu(), d.cpu(), d.cpu(), *[t.cpu() for t in plan])
    with pytest.raises(ValueError, match="identical"):
        dhs_solve_cuda(d, d[:, :2], d, *plan)
    with pytest.raises(ValueError, match="divide 32"):
        dhs_solve_cuda(d, d, d, *plan, threads=3)
    with pytest.raises(TypeError, match="int32 or int64"):
        dhs_solve_cuda(d, d, d, plan[0].float(), plan[1], plan[2])


def test_tree_beyond_shared_memory(cuda):
    # 40,000 float64 nodes: the accumulators live in a global workspace
    rng = np.random.default_rng(40)
    K = 40000
    parent = _random_tree(rng, K)
    B = 5
    d = 1.0 + rng.random((B, K))
    a = 0.5 * rng.random((B, K))
    a[:, 0] = 0.0
    b = rng.standard_normal((B, K))
    p, order, lptr = _plan(parent, 32, cuda)
    x = dhs_solve_cuda(*(torch.as_tensor(t, device=cuda) for t in (d, a, b)), p, order, lptr)
    ref = oracle.dhs_solve(d, a, b, np.asarray(parent), order.cpu().numpy(), lptr.cpu().numpy())
    np.testing.assert_allclose(x.cpu().numpy(), ref, rtol=1e-11, atol=1e-12)


def test_chain_and_layer_schedules_are_bit_identical(cuda):
    # dhs_solve_cuda runs the chain schedule; the C entry dgb_dhs_solve the
    # depth-layer schedule of the same elimination
    from dendra_gb300 import _lib
    from dendra_gb300.tree import _device_topology

    rng = np.random.default_rng(77)
    for K, dt in ((1, torch.float64), (2, torch.float32), (333, torch.float32),
                  (1500, torch.float64)):
        parent = _random_tree(rng, K)
        B = 65
        d = torch.as_tensor(1.0 + rng.random((B, K)), device=cuda, dtype=dt)
        a = torch.as_tensor(0.5 * rng.random((B, K)), device=cuda, dtype=dt)
        b = torch.as_tensor(rng.standard_normal((B, K)), device=cuda, dtype=dt)
        p, order, lptr = _plan(parent, 32, cuda)
        x = dhs_solve_cuda(d, a, b, p, order, lptr)
        par, o, lp, cptr, cidx = _device_topology(p, order, lptr)
        y = torch.empty_like(b)
        rc = _lib.load().dgb_dhs_solve(_lib.dtype_code(dt), B, K, d.data_ptr(), a.data_ptr(),
                                       b.data_ptr(), par.data_ptr(), o.data_ptr(), lp.data_ptr(),
                                       lp.numel() - 1, cptr.data_ptr(), cidx.data_ptr(),
                                       y.data_ptr(), _lib.stream_ptr(cuda))
        assert rc == 0
        torch.testing.assert_close(x, y, rtol=0, atol=0)
