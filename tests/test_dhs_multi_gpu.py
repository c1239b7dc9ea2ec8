"""Row-padded multi-morphology tree solve with the reference's signature
(triton/dhs_kernel_multi.py:831-888) against dense solves, dense autograd and
the single-topology solve; the reference's argument checks
(triton/_contracts.py:271-341)."""

import numpy as np
import pytest
import torch

from dendra_gb300.tree import (build_dhs_layers, build_morphology, dhs_solve_cuda,
                               dhs_solve_multi_cuda)
from tests.test_contraction_plan import random_tree

pytestmark = pytest.mark.gpu


def _dhs_order(parent, threads):
    _, _, depth = build_morphology([int(p) for p in parent])
    order, layer_ptr = build_dhs_layers(depth, threads)
    return order.numpy(), layer_ptr.numpy()


def multi_plan(morphs, rows_of, threads, B, dev):
    """Concatenated per-morphology tables and per-warp row groups of at most
    32 // threads rows, as the reference's planner lays them out."""
    P, O, L, p_off, o_off, l_off = [], [], [], [], [], []
    for parent in morphs:
        order, lptr = _dhs_order(parent, threads)
        p_off.append(sum(map(len, P)))
        o_off.append(sum(map(len, O)))
        l_off.append(sum(map(len, L)))
        P.append(np.asarray(parent))
        O.append(order)
        L.append(lptr)
    npw = 32 // threads
    warps = []
    for m, rows in enumerate(rows_of):
        for s in range(0, len(rows), npw):
            chunk = rows[s:s + npw]
            assert list(chunk) == list(range(chunk[0], chunk[0] + len(chunk)))
            warps.append((p_off[m], o_off[m], l_off[m], len(L[m]) - 1, chunk[0], len(chunk)))
    w = np.asarray(warps, dtype=np.int64).T

    def t(x, dt=torch.int64):
        return torch.as_tensor(np.asarray(x), dtype=dt, device=dev)

    return (t(np.concatenate(P)), t(np.concatenate(O)), t(np.concatenate(L)), t(w[0]),
            t(w[1]), t(w[2]), t(w[3], torch.int32), t(w[4]), t(w[5], torch.int32))


def hines_dense(d, g, parent):
    K = len(parent)
    A = torch.diag_embed(d + g)
    for i in range(K):
        p = int(parent[i])
        if p >= 0:
            A[..., p, p] = A[..., p, p] + g[..., i]
            A[..., i, p] = A[..., i, p] - g[..., i]
            A[..., p, i] = A[..., p, i] - g[..., i]
    return A


def case(dev, dtype=torch.float64, threads=8, seed=0):
    rng = np.random.default_rng(seed)
    morphs = [random_tree(rng, 5, 0.3), random_tree(rng, 40, 0.2), random_tree(rng, 120, 0.05)]
    # keep every parent before its child in the row? not required: any order
    rows_of = [list(range(0, 10)), list(range(10, 17)), list(range(18, 31))]  # row 17, 31 uncovered
    B, Ks = 32, 128
    plan = multi_plan(morphs, rows_of, threads, B, dev)
    d = torch.as_tensor(rng.uniform(0.1, 2.0, (B, Ks)), dtype=dtype, device=dev)
    g = torch.as_tensor(rng.uniform(0.5, 5.0, (B, Ks)), dtype=dtype, device=dev)
    b = torch.as_tensor(rng.normal(size=(B, Ks)), dtype=dtype, device=dev)
    return morphs, rows_of, plan, d, g, b, Ks, threads


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_matches_dense_and_single_topology_solves(cuda, dtype):
    morphs, rows_of, plan, d, g, b, Ks, threads = case(cuda, dtype)
    L_max = int(max(int(t) for t in plan[6].cpu()))
    x = dhs_solve_multi_cuda(d, g, b, *plan, K_stride=Ks, L_max=L_max, threads=threads)
    tol = dict(rtol=5e-5, atol=5e-6) if dtype == torch.float32 else dict(rtol=3e-12, atol=3e-12)
    covered = torch.zeros(d.shape[0], dtype=torch.bool)
    for parent, rows in zip(morphs, rows_of):
        K = len(parent)
        r = torch.as_tensor(rows)
        covered[r] = True
        A = hines_dense(d[r, :K].double(), g[r, :K].double(), parent)
        ref = torch.linalg.solve(A, b[r, :K].double())
        torch.testing.assert_close(x[r, :K].double(), ref, **tol)
        assert (x[r, K:] == 0).all()  # padding untouched (zero)
        order, lptr = _dhs_order(parent, threads)
        dev = cuda
        one = dhs_solve_cuda(d[r, :K].contiguous(), g[r, :K].contiguous(), b[r, :K].contiguous(),
                             torch.as_tensor(parent, device=dev), torch.as_tensor(order, device=dev),
                             torch.as_tensor(lptr, device=dev), threads=threads)
        torch.testing.assert_close(x[r, :K], one, rtol=0, atol=0)  # same kernel, same order
    assert (x[~covered.to(x.device)] == 0).all()


def test_gradients_match_dense_autograd(cuda):
    morphs, rows_of, plan, d, g, b, Ks, threads = case(cuda, seed=3)
    w = torch.randn_like(b)
    ins = [t.clone().requires_grad_() for t in (d, g, b)]
    (dhs_solve_multi_cuda(*ins, *plan, K_stride=Ks, L_max=8, threads=threads) * w).sum().backward()
    for parent, rows in zip(morphs, rows_of):
        K = len(parent)
        r = torch.as_tensor(rows, device=cuda)
        ref = [t[r, :K].detach().clone().requires_grad_() for t in (d, g, b)]
        A = hines_dense(ref[0], ref[1], parent)
        (torch.linalg.solve(A, ref[2]) * w[r, :K]).sum().backward()
        for a, rr in zip(ins, ref):
            torch.testing.assert_close(a.grad[r, :K], rr.grad, rtol=1e-10, atol=1e-12)
            assert (a.grad[r, K:] == 0).all()


def test_reference_argument_checks(cuda):
    morphs, rows_of, plan, d, g, b, Ks, threads = case(cuda)
    with pytest.raises(ValueError, match="K_stride must equal"):
        dhs_solve_multi_cuda(d, g, b, *plan, K_stride=Ks - 1, L_max=4, threads=threads)
    with pytest.raises(TypeError, match="L_max must be an integer"):
        dhs_solve_multi_cuda(d, g, b, *plan, K_stride=Ks, L_max=4.0, threads=threads)
    with pytest.raises(ValueError, match="grid_x must equal"):
        dhs_solve_multi_cuda(d, g, b, *plan, K_stride=Ks, L_max=4, threads=threads, grid_x=1)
    bad = list(plan)
    bad[8] = bad[8][:-1]
    with pytest.raises(ValueError, match="one entry per warp"):
        dhs_solve_multi_cuda(d, g, b, *bad, K_stride=Ks, L_max=4, threads=threads)
    bad = list(plan)
    bad[0] = bad[0].float()
    with pytest.raises(TypeError, match="int32 or int64"):
        dhs_solve_multi_cuda(d, g, b, *bad, K_stride=Ks, L_max=4, threads=threads)
    with pytest.raises(ValueError, match="divide 32"):
        dhs_solve_multi_cuda(d, g, b, *plan, K_stride=Ks, L_max=4, threads=3)
    bad = list(plan)
    bad[7] = bad[7].clone()
    bad[7][1] = bad[7][0]  # two warps on the same rows
    with pytest.raises(ValueError, match="covered by two warps"):
        dhs_solve_multi_cuda(d, g, b, *bad, K_stride=Ks, L_max=4, threads=threads)
