"""Functional solver facade (the reference's integrators/_cuda_functional.py):
reverse, forward-mode and vmap rules of every solve against dense float64
linear algebra and against the drop-in solvers."""

import numpy as np
import pytest
import torch

from dendra_gb300 import functional as F
from dendra_gb300.solvers import solve_bt_spd_cuda, thomas_solve_cuda_bt, thomas_solve_cuda_t
from dendra_gb300.tree import build_dhs_layers, build_morphology, dhs_solve_cuda
from tests.test_dhs_multi_gpu import case as multi_case
from tests.test_dhs_multi_gpu import hines_dense

pytestmark = pytest.mark.gpu
TOL = dict(rtol=1e-9, atol=1e-11)


def tri_dense(a, b, c):
    return torch.diag_embed(b) + torch.diag_embed(a, -1) + torch.diag_embed(c, 1)


def block_dense(lower, main, upper):
    B, K = main.shape[:2]
    A = torch.zeros(B, 3 * K, 3 * K, dtype=main.dtype, device=main.device)
    for k in range(K):
        A[:, 3 * k:3 * k + 3, 3 * k:3 * k + 3] = main[:, k]
        if k + 1 < K:
            A[:, 3 * k:3 * k + 3, 3 * k + 3:3 * k + 6] = torch.diag_embed(upper[:, k])
            A[:, 3 * k + 3:3 * k + 6, 3 * k:3 * k + 3] = torch.diag_embed(lower[:, k])
    return A


def tri_case(dev, B=4, K=17, seed=0):
    g = torch.Generator().manual_seed(seed)
    a = -torch.rand(B, K - 1, generator=g, dtype=torch.float64)
    c = -torch.rand(B, K - 1, generator=g, dtype=torch.float64)
    b = 3 + torch.rand(B, K, generator=g, dtype=torch.float64)
    d = torch.randn(B, K, generator=g, dtype=torch.float64)
    return [t.to(dev) for t in (a, b, c, d)]


@pytest.mark.parametrize("solve", [F.thomas_solve, F.pcr_solve])
def test_tridiagonal_rules(cuda, solve):
    a, b, c, d = tri_case(cuda)
    x = solve(a, b, c, d)
    torch.testing.assert_close(x, thomas_solve_cuda_t(a, b, c, d), **TOL)
    dense = lambda a, b, c, d: torch.linalg.solve(tri_dense(a, b, c), d)
    tangents = [torch.randn_like(t) for t in (a, b, c, d)]
    _, jv = torch.func.jvp(solve, (a, b, c, d), tuple(tangents))
    _, jr = torch.func.jvp(dense, (a, b, c, d), tuple(tangents))
    torch.testing.assert_close(jv, jr, **TOL)
    w = torch.randn_like(d)
    grads = torch.func.grad(lambda *t: (solve(*t) * w).sum(), argnums=(0, 1, 2, 3))(a, b, c, d)
    refs = torch.func.grad(lambda *t: (dense(*t) * w).sum(), argnums=(0, 1, 2, 3))(a, b, c, d)
    for gg, rr in zip(grads, refs):
        torch.testing.assert_close(gg, rr, **TOL)
    # vmap over a leading dimension of the right-hand side, and of the diagonal
    dd = torch.randn(3, *d.shape, dtype=d.dtype, device=cuda)
    out = torch.func.vmap(lambda r: solve(a, b, c, r))(dd)
    for v in range(3):
        torch.testing.assert_close(out[v], solve(a, b, c, dd[v]), rtol=0, atol=0)
    bb = b.unsqueeze(0) + torch.rand(2, *b.shape, dtype=b.dtype, device=cuda)
    out = torch.func.vmap(lambda m: solve(a, m, c, d))(bb)
    for v in range(2):
        torch.testing.assert_close(out[v], solve(a, bb[v], c, d), rtol=0, atol=0)
    # second order: the Hessian-vector product of a quadratic loss
    hv = torch.func.jvp(lambda m: torch.func.grad(lambda mm: (solve(a, mm, c, d) ** 2).sum())(m),
                        (b,), (tangents[1],))[1]
    hr = torch.func.jvp(lambda m: torch.func.grad(lambda mm: (dense(a, mm, c, d) ** 2).sum())(m),
                        (b,), (tangents[1],))[1]
    torch.testing.assert_close(hv, hr, rtol=1e-8, atol=1e-10)


def block_case(dev, B=3, K=9, seed=1, spd=False):
    g = torch.Generator().manual_seed(seed)
    lower = -torch.rand(B, K - 1, 3, generator=g, dtype=torch.float64)
    upper = lower.clone() if spd else -torch.rand(B, K - 1, 3, generator=g, dtype=torch.float64)
    m = 0.3 * torch.randn(B, K, 3, 3, generator=g, dtype=torch.float64)
    main = m + m.transpose(-1, -2) if spd else m
    main = main + 6 * torch.eye(3, dtype=torch.float64)
    rhs = torch.randn(B, K, 3, generator=g, dtype=torch.float64)
    return [t.to(dev) for t in (lower, main, upper, rhs)]


def test_block_rules(cuda):
    lower, main, upper, rhs = block_case(cuda)
    x = F.block_thomas_solve(lower, main, upper, rhs)
    torch.testing.assert_close(x, thomas_solve_cuda_bt(lower, main, upper, rhs), rtol=0, atol=0)

    def dense(lo, m, up, r):
        return torch.linalg.solve(block_dense(lo, m, up), r.reshape(r.shape[0], -1)).view_as(r)

    args = (lower, main, upper, rhs)
    tangents = tuple(torch.randn_like(t) for t in args)
    _, jv = torch.func.jvp(F.block_thomas_solve, args, tangents)
    _, jr = torch.func.jvp(dense, args, tangents)
    torch.testing.assert_close(jv, jr, **TOL)
    w = torch.randn_like(rhs)
    grads = torch.func.grad(lambda *t: (F.block_thomas_solve(*t) * w).sum(), argnums=(0, 1, 2, 3))(*args)
    refs = torch.func.grad(lambda *t: (dense(*t) * w).sum(), argnums=(0, 1, 2, 3))(*args)
    for gg, rr in zip(grads, refs):
        torch.testing.assert_close(gg, rr, **TOL)
    rr = torch.randn(2, *rhs.shape, dtype=rhs.dtype, device=cuda)
    out = torch.func.vmap(lambda r: F.block_thomas_solve(lower, main, upper, r))(rr)
    torch.testing.assert_close(out[1], F.block_thomas_solve(lower, main, upper, rr[1]), rtol=0, atol=0)


def test_block_spd_rules(cuda):
    lower, main, upper, rhs = block_case(cuda, spd=True)
    x = F.block_spd_solve(lower, main, upper, rhs)
    torch.testing.assert_close(x, solve_bt_spd_cuda(lower, main, upper, rhs), rtol=0, atol=0)
    dense = lambda lo, m, up, r: torch.linalg.solve(
        block_dense(lo, 0.5 * (m + m.transpose(-1, -2)), up), r.reshape(r.shape[0], -1)).view_as(r)
    torch.testing.assert_close(x, dense(lower, main, upper, rhs), **TOL)
    # tangents of a symmetric system (lower == upper, symmetric main blocks)
    tl = torch.randn_like(lower)
    tm = torch.randn_like(main)
    tm = tm + tm.transpose(-1, -2)
    tr = torch.randn_like(rhs)
    _, jv = torch.func.jvp(lambda lo, m, r: F.block_spd_solve(lo, m, lo, r), (lower, main, rhs),
                           (tl, tm, tr))
    _, jr = torch.func.jvp(lambda lo, m, r: dense(lo, m, lo, r), (lower, main, rhs), (tl, tm, tr))
    torch.testing.assert_close(jv, jr, **TOL)
    rr = torch.randn(2, *rhs.shape, dtype=rhs.dtype, device=cuda)
    out = torch.func.vmap(lambda r: F.block_spd_solve(lower, main, upper, r))(rr)
    torch.testing.assert_close(out[0], F.block_spd_solve(lower, main, upper, rr[0]), rtol=0, atol=0)


def tree_case(dev, K=31, B=4, seed=2, block=False):
    rng = np.random.default_rng(seed)
    parent = np.array([-1] + [int(rng.integers(0, i)) for i in range(1, K)])
    _, _, depth = build_morphology([int(p) for p in parent])
    order, layers = build_dhs_layers(depth, 8)
    shape = (B, K, 3) if block else (B, K)
    main = torch.as_tensor(rng.uniform(0.5, 2.0, shape if not block else (B, K, 3, 3)),
                           device=dev)
    if block:
        main = 0.2 * main + 4 * torch.eye(3, dtype=main.dtype, device=dev)
    edge = torch.as_tensor(rng.uniform(0.5, 3.0, shape), device=dev)
    rhs = torch.as_tensor(rng.normal(size=shape), device=dev)
    topo = (torch.as_tensor(parent, device=dev), order.to(dev), layers.to(dev))
    return parent, topo, main, edge, rhs


def test_tree_rules(cuda):
    parent, topo, main, edge, rhs = tree_case(cuda)
    solve = lambda m, e, r: F.dhs_solve(m, e, r, *topo, threads=8)
    x = solve(main, edge, rhs)
    torch.testing.assert_close(x, dhs_solve_cuda(main, edge, rhs, *topo, threads=8), rtol=0, atol=0)
    dense = lambda m, e, r: torch.linalg.solve(hines_dense(m, e, parent), r)
    args = (main, edge, rhs)
    tangents = tuple(torch.randn_like(t) for t in args)
    torch.testing.assert_close(torch.func.jvp(solve, args, tangents)[1],
                               torch.func.jvp(dense, args, tangents)[1], **TOL)
    w = torch.randn_like(rhs)
    grads = torch.func.grad(lambda *t: (solve(*t) * w).sum(), argnums=(0, 1, 2))(*args)
    refs = torch.func.grad(lambda *t: (dense(*t) * w).sum(), argnums=(0, 1, 2))(*args)
    for gg, rr in zip(grads, refs):
        torch.testing.assert_close(gg, rr, **TOL)
    ee = edge.unsqueeze(0) * (1 + torch.rand(2, *edge.shape, dtype=edge.dtype, device=cuda))
    out = torch.func.vmap(lambda e: solve(main, e, rhs))(ee)
    torch.testing.assert_close(out[1], solve(main, ee[1], rhs), rtol=0, atol=0)


def test_block_tree_rules(cuda):
    parent, topo, main, edge, rhs = tree_case(cuda, K=13, block=True)
    solve = lambda m, e, r: F.dhs_bt_solve(m, e, r, *topo, threads=8)

    def dense(m, e, r):
        B, K = r.shape[:2]
        A = torch.zeros(B, 3 * K, 3 * K, dtype=r.dtype, device=r.device)
        for i in range(K):
            A[:, 3 * i:3 * i + 3, 3 * i:3 * i + 3] = m[:, i] + torch.diag_embed(e[:, i])
            p = int(parent[i])
            if p >= 0:
                A[:, 3 * p:3 * p + 3, 3 * p:3 * p + 3] += torch.diag_embed(e[:, i])
                A[:, 3 * i:3 * i + 3, 3 * p:3 * p + 3] -= torch.diag_embed(e[:, i])
                A[:, 3 * p:3 * p + 3, 3 * i:3 * i + 3] -= torch.diag_embed(e[:, i])
        return torch.linalg.solve(A, r.reshape(B, -1)).view_as(r)

    args = (main, edge, rhs)
    torch.testing.assert_close(solve(*args), dense(*args), **TOL)
    tangents = tuple(torch.randn_like(t) for t in args)
    torch.testing.assert_close(torch.func.jvp(solve, args, tangents)[1],
                               torch.func.jvp(dense, args, tangents)[1], **TOL)
    w = torch.randn_like(rhs)
    grads = torch.func.grad(lambda *t: (solve(*t) * w).sum(), argnums=(0, 1, 2))(*args)
    refs = torch.func.grad(lambda *t: (dense(*t) * w).sum(), argnums=(0, 1, 2))(*args)
    for gg, rr in zip(grads, refs):
        torch.testing.assert_close(gg, rr, **TOL)


def test_multi_rules(cuda):
    morphs, rows_of, plan, d, g, b, Ks, threads = multi_case(cuda, seed=5)
    solve = lambda m, e, r: F.dhs_multi_solve(m, e, r, *plan, K_stride=Ks, L_max=8,
                                              threads=threads, grid_x=None)

    def dense(m, e, r):
        out = torch.zeros_like(r)
        for parent, rows in zip(morphs, rows_of):
            K = len(parent)
            idx = torch.as_tensor(rows, device=r.device)
            x = torch.linalg.solve(hines_dense(m[idx, :K], e[idx, :K], parent), r[idx, :K])
            out = out.index_put((idx.unsqueeze(1), torch.arange(K, device=r.device)), x)
        return out

    args = (d, g, b)
    torch.testing.assert_close(solve(*args), dense(*args), **TOL)
    tangents = tuple(torch.randn_like(t) for t in args)
    torch.testing.assert_close(torch.func.jvp(solve, args, tangents)[1],
                               torch.func.jvp(dense, args, tangents)[1], **TOL)
    w = torch.randn_like(b)
    grads = torch.func.grad(lambda *t: (solve(*t) * w).sum(), argnums=(0, 1, 2))(*args)
    refs = torch.func.grad(lambda *t: (dense(*t) * w).sum(), argnums=(0, 1, 2))(*args)
    for gg, rr in zip(grads, refs):
        torch.testing.assert_close(gg, rr, **TOL)
    bb = torch.randn(3, *b.shape, dtype=b.dtype, device=cuda)
    out = torch.func.vmap(lambda r: solve(d, g, r))(bb)
    for v in range(3):
        torch.testing.assert_close(out[v], solve(d, g, bb[v]), rtol=0, atol=0)
