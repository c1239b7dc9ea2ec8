"""3x3 block tree solves (multi-layer extracellular trees) on the GPU against the
dense matrix the reference's dhs_kernel_bt.py factors (the reference's own
block tree solvers need Triton on a GPU or the absent dendra-solvers package,
so the dense restatement is the accuracy reference), with gradients against dense autograd."""

import numpy as np
import pytest
import torch

import oracle
from dendra_gb300.tree import build_dhs_layers, build_morphology, dhs_bt_solve_cuda
from tests.test_dhs_gpu import _random_tree

pytestmark = pytest.mark.gpu


def _plan(parent, dev, threads=16):
    _, _, depth = build_morphology(list(parent))
    order, layer_ptr = build_dhs_layers(depth, threads)
    return (torch.as_tensor(np.asarray(parent), device=dev), order.to(dev).long(),
            layer_ptr.to(dev).long())


def _system(rng, B, K, parent):
    """Diagonally dominant node blocks (membrane + two extracellular layers)."""
    D = 0.3 * rng.standard_normal((B, K, 3, 3))
    D += np.eye(3) * (3.0 + rng.random((B, K, 1, 1)))
    G = 0.2 + rng.random((B, K, 3))
    G[:, [i for i, p in enumerate(parent) if p < 0]] *= 0.1  # root: a leak to ground
    b = rng.standard_normal((B, K, 3))
    return D, G, b


@pytest.mark.parametrize("K", [1, 2, 9, 120, 700])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_matches_dense_solve(cuda, K, dtype):
    rng = np.random.default_rng(K)
    parent = _random_tree(rng, K, branch=5)
    B = 7
    D, G, b = _system(rng, B, K, parent)
    x = dhs_bt_solve_cuda(*(torch.as_tensor(t, device=cuda, dtype=dtype) for t in (D, G, b)),
                          *_plan(parent, cuda))
    ref = oracle.dhs_block3_solve(D, G, b, parent)
    tol = dict(rtol=1e-11, atol=1e-12) if dtype == torch.float64 else dict(rtol=2e-4, atol=2e-5)
    np.testing.assert_allclose(x.cpu().numpy(), ref, **tol)


def test_deterministic(cuda):
    rng = np.random.default_rng(3)
    parent = _random_tree(rng, 400)
    args = [torch.as_tensor(t, device=cuda, dtype=torch.float32) for t in _system(rng, 16, 400,
                                                                                   parent)]
    plan = _plan(parent, cuda)
    x0 = dhs_bt_solve_cuda(*args, *plan)
    for _ in range(3):
        torch.testing.assert_close(dhs_bt_solve_cuda(*args, *plan), x0, rtol=0, atol=0)


def test_gradients_match_dense_autograd(cuda):
    rng = np.random.default_rng(5)
    K, B = 30, 3
    parent = _random_tree(rng, K, branch=4)
    D, G, b = (torch.as_tensor(t, device=cuda).requires_grad_() for t in _system(rng, B, K,
                                                                                    parent))
    w = torch.linspace(-1, 1, b.numel(), device=cuda, dtype=torch.float64).reshape(b.shape)
    x = dhs_bt_solve_cuda(D, G, b, *_plan(parent, cuda))
    (x * w).sum().backward()
    grads = [t.grad.clone() for t in (D, G, b)]
    for t in (D, G, b):
        t.grad = None
    A = torch.zeros(B, 3 * K, 3 * K, dtype=torch.float64, device=cuda)
    eye = torch.eye(3, dtype=torch.float64, device=cuda)
    for i in range(K):
        A[:, 3 * i:3 * i + 3, 3 * i:3 * i + 3] = D[:, i] + G[:, i].unsqueeze(-1) * eye
    A = A + 0.0
    for c, p in enumerate(parent):
        if p < 0:
            continue
        for r in range(3):
            g = G[:, c, r]
            A[:, 3 * p + r, 3 * p + r] = A[:, 3 * p + r, 3 * p + r] + g
            A[:, 3 * c + r, 3 * p + r] = A[:, 3 * c + r, 3 * p + r] - g
            A[:, 3 * p + r, 3 * c + r] = A[:, 3 * p + r, 3 * c + r] - g
    xd = torch.linalg.solve(A, b.reshape(B, 3 * K, 1)).reshape(B, K, 3)
    (xd * w).sum().backward()
    for gk, t in zip(grads, (D, G, b)):
        torch.testing.assert_close(gk, t.grad, rtol=1e-9, atol=1e-10)


def test_tree_beyond_shared_memory(cuda):
    # 3,000 float64 nodes need 288 KB of scratch: the global-workspace path,
    # checked by the residual of the block Hines system
    rng = np.random.default_rng(30)
    K = 3000
    parent = _random_tree(rng, K, branch=5)
    B = 3
    D, G, b = _system(rng, B, K, parent)
    Dt, Gt, bt = (torch.as_tensor(t, device=cuda) for t in (D, G, b))
    x = dhs_bt_solve_cuda(Dt, Gt, bt, *_plan(parent, cuda))
    par = torch.as_tensor(np.asarray(parent), device=cuda)
    has = par >= 0
    ps = par.clamp_min(0)
    # D_i x_i + g_i (x_i - x_p) (root: g_i x_i) + sum_c g_c (x_i - x_c) - b_i
    res = (Dt @ x.unsqueeze(-1)).squeeze(-1) + Gt * x - bt
    res = res - torch.where(has.view(1, -1, 1), Gt * x[:, ps], torch.zeros_like(x))
    res = res.index_add(1, ps[has], Gt[:, has] * x[:, ps[has]] - Gt[:, has] * x[:, has])
    assert float(res.abs().max()) < 1e-10 * float(bt.abs().max())
