"""Tree-contraction solve on the GPU.

* bit-exact against the oracle's restatement of the same plan (f32 and f64);
* the reference's dense-oracle fixture of the tree solve (the DHS parity case
  of tests/test_cuda_solver_parity.py) within that test's tolerances;
* equal to the DHS solve within the reference's contraction-vs-DHS
  tolerances (tests/func/test_tree_contraction_integration.py:131-144);
* gradients (tree_contraction.py:596-609), the forward-mode tangent and vmap
  against dense float64 autograd.
"""

import ctypes

import numpy as np
import pytest
import torch

import oracle
from dendra_gb300 import _lib
from dendra_gb300.contraction import TreeContractionPlan, prepare, solve
from dendra_gb300.tree import build_dhs_layers, build_morphology, dhs_solve_cuda
from tests.test_contraction_plan import random_tree, ref_parent, systems

pytestmark = pytest.mark.gpu

DTYPES = [torch.float32, torch.float64]
NP = {torch.float32: np.float32, torch.float64: np.float64}


def run(parent, cap, d, g, b, dev, dtype):
    plan = TreeContractionPlan(parent, cap)
    t = [torch.as_tensor(a).to(dev, dtype) for a in (d, g, b)]
    return plan, solve(*t, plan)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("cap", [None, 1, 3, 16])
@pytest.mark.parametrize("K,branch,B", [(1, 0.0, 5), (2, 0.0, 3), (9, 0.3, 40), (64, 0.0, 33),
                                        (300, 0.1, 70), (500, 0.6, 9)])
def test_bit_exact_against_oracle(cuda, dtype, cap, K, branch, B):
    rng = np.random.default_rng(K + 7 * B)
    parent = random_tree(rng, K, branch)
    d, g, b = systems(rng, B, K, NP[dtype])
    plan, x = run(parent, cap, d, g, b, cuda, dtype)
    ref = oracle.tree_contract_solve(d, g, b, plan.tables)
    np.testing.assert_array_equal(x.cpu().numpy(), ref)


@pytest.mark.parametrize("threads", [32, 64, 128, 256])
def test_every_block_width_is_bit_exact(cuda, threads):
    rng = np.random.default_rng(threads)
    parent = random_tree(rng, 700, 0.05)
    d, g, b = systems(rng, 50, 700, np.float32)
    for cap in (16, None):
        plan = TreeContractionPlan(parent, cap, threads=threads)
        x = solve(*(torch.as_tensor(a).to(cuda) for a in (d, g, b)), plan)
        np.testing.assert_array_equal(x.cpu().numpy(),
                                      oracle.tree_contract_solve(d, g, b, plan.tables))


@pytest.mark.parametrize("dtype", DTYPES)
def test_large_tree_many_rows(cuda, dtype):
    # C3-sized tree (2000 nodes, runs of several compartments), 600 rows
    rng = np.random.default_rng(11)
    parent = random_tree(rng, 2000, 0.03)
    d, g, b = systems(rng, 600, 2000, NP[dtype])
    for cap in (16, None):
        plan, x = run(parent, cap, d, g, b, cuda, dtype)
        rows = [0, 1, 311, 599]
        ref = oracle.tree_contract_solve(d[rows], g[rows], b[rows], plan.tables)
        np.testing.assert_array_equal(x.cpu().numpy()[rows], ref)


TOL_FIX = {torch.float32: dict(rtol=5e-5, atol=5e-6), torch.float64: dict(rtol=3e-12, atol=3e-12)}


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("cap", [None, 2, 16])
def test_reference_dense_fixture(cuda, golden, dtype, cap):
    g = golden("dhs.npz")
    for case in ("parity", "rand"):
        parent = g[f"{case}_parent"]
        d, a, b = (torch.as_tensor(g[f"{case}_{x}"]).to(cuda, dtype) for x in "dab")
        x = solve(d, a, b, TreeContractionPlan(parent, cap))
        torch.testing.assert_close(x, torch.as_tensor(g[f"{case}_x"]).to(cuda, dtype),
                                   **TOL_FIX[dtype])


# contraction vs DHS states (v) of the reference's integration test
TOL_DHS = {torch.float32: dict(rtol=1e-6, atol=1e-5), torch.float64: dict(rtol=2e-11, atol=1e-11)}


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("cap", [2, None])
def test_matches_dhs(cuda, dtype, cap):
    rng = np.random.default_rng(3)
    for parent in (ref_parent(), random_tree(rng, 400, 0.08)):
        K = parent.size
        # cable-like systems: a membrane shunt (C/dt + G) of the scale of the
        # axial conductances, voltages of tens of mV
        d = rng.uniform(0.5, 1.5, (16, K))
        gg = rng.uniform(0.5, 3.0, (16, K))
        v = rng.uniform(-70, -50, (16, K))
        _, _, depth = build_morphology([int(p) for p in parent])
        order, layer_ptr = build_dhs_layers(depth, 16)
        t = [torch.as_tensor(a).to(cuda, dtype) for a in (d, gg, v)]
        x_dhs = dhs_solve_cuda(*t, torch.as_tensor(parent).to(cuda), order.to(cuda),
                               layer_ptr.to(cuda), threads=16)
        x = solve(*t, TreeContractionPlan(parent, cap))
        torch.testing.assert_close(x, x_dhs, **TOL_DHS[dtype])


def dense_reference(parent, d, g, b):
    K = parent.size
    A = torch.diag_embed(d + g)
    for i in range(K):
        p = int(parent[i])
        if p >= 0:
            A[:, p, p] = A[:, p, p] + g[:, i]
            A[:, i, p] = A[:, i, p] - g[:, i]
            A[:, p, i] = A[:, p, i] - g[:, i]
    return torch.linalg.solve(A, b)


@pytest.mark.parametrize("cap", [None, 2])
def test_gradients_match_dense_autograd(cuda, cap):
    rng = np.random.default_rng(4)
    parent = random_tree(rng, 23, 0.3)
    d, g, b = systems(rng, 4, 23)
    w = torch.as_tensor(rng.normal(size=(4, 23)), device=cuda)
    plan = TreeContractionPlan(parent, cap)
    ins = [torch.as_tensor(a, device=cuda).requires_grad_() for a in (d, g, b)]
    (solve(*ins, plan) * w).sum().backward()
    ref = [torch.as_tensor(a, device=cuda).requires_grad_() for a in (d, g, b)]
    (dense_reference(parent, *ref) * w).sum().backward()
    for a, r in zip(ins, ref):
        torch.testing.assert_close(a.grad, r.grad, rtol=1e-10, atol=1e-12)
    # gradcheck through the custom backward
    small = [torch.as_tensor(a[:2], device=cuda).requires_grad_() for a in (d, g, b)]
    assert torch.autograd.gradcheck(lambda *t: solve(*t, plan), small)


def test_forward_mode_vmap_and_functional_grad(cuda):
    rng = np.random.default_rng(6)
    parent = ref_parent()
    plan = prepare(TreeContractionPlan(parent, 2), cuda)
    d, g, b = (torch.as_tensor(a, device=cuda) for a in systems(rng, 3, 8))
    td, tg, tb = (torch.as_tensor(rng.normal(size=(3, 8)), device=cuda) for _ in range(3))
    _, tangent = torch.func.jvp(lambda *t: solve(*t, plan), (d, g, b), (td, tg, tb))
    _, ref = torch.func.jvp(lambda *t: dense_reference(parent, *t), (d, g, b), (td, tg, tb))
    torch.testing.assert_close(tangent, ref, rtol=1e-10, atol=1e-12)
    # vmap over a leading dimension of the right-hand side only
    bb = torch.as_tensor(rng.normal(size=(5, 3, 8)), device=cuda)
    out = torch.func.vmap(lambda r: solve(d, g, r, plan))(bb)
    for v in range(5):
        torch.testing.assert_close(out[v], solve(d, g, bb[v], plan), rtol=0, atol=0)
    # per-sample gradients through vmap(grad)
    w = torch.as_tensor(rng.normal(size=(4, 3, 8)), device=cuda)

    def loss(dd, gg, ww):
        return (solve(dd, gg, b, plan) * ww).sum()

    gd, gg = torch.func.vmap(torch.func.grad(loss, argnums=(0, 1)), in_dims=(None, None, 0))(d, g, w)
    for v in range(4):
        ref = [t.clone().requires_grad_() for t in (d, g)]
        (dense_reference(parent, ref[0], ref[1], b) * w[v]).sum().backward()
        torch.testing.assert_close(gd[v], ref[0].grad, rtol=1e-10, atol=1e-12)
        torch.testing.assert_close(gg[v], ref[1].grad, rtol=1e-10, atol=1e-12)


def test_contract_errors(cuda):
    plan = TreeContractionPlan(np.array([-1, 0, 1]))
    x = torch.ones(2, 3, device=cuda)
    with pytest.raises(ValueError, match="matching the plan"):
        solve(torch.ones(2, 4, device=cuda), x, x, plan)
    with pytest.raises(ValueError, match="float32 or float64"):
        solve(x.half(), x.half(), x.half(), plan)
    with pytest.raises(ValueError, match="same-shaped strided CUDA"):
        solve(x, x.cpu(), x, plan)
    # a tree whose scratch needs the global workspace refuses a launch without one
    big = TreeContractionPlan(np.arange(30000) - 1, None)
    y = torch.ones(1, 30000, device=cuda, dtype=torch.float64)
    L = _lib.load()
    st = big.struct(y.device)
    assert L.dgb_tree_contract_work_size(1, ctypes.byref(st), 1) > 0
    x = torch.empty_like(y)
    assert L.dgb_tree_contract_solve(1, 1, ctypes.byref(st), y.data_ptr(), y.data_ptr(),
                                     y.data_ptr(), x.data_ptr(), None, 0, None) == -1
    # empty batch
    e = torch.ones(0, 3, device=cuda)
    assert solve(e, e, e, plan).shape == (0, 3)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("cap", [16, None])
def test_trees_beyond_shared_memory(cuda, dtype, cap):
    # scratch in the global workspace: a 30,000-node cable and a 20,000-node
    # branched tree, bit-exact against the oracle like the on-chip path
    rng = np.random.default_rng(21)
    for parent in (np.arange(30000) - 1, random_tree(rng, 20000, 0.02)):
        K = parent.size
        plan = TreeContractionPlan(parent, cap)
        d, g, b = systems(rng, 3, K, NP[dtype])
        x = solve(*(torch.as_tensor(a).to(cuda, dtype) for a in (d, g, b)), plan)
        np.testing.assert_array_equal(x.cpu().numpy(), oracle.tree_contract_solve(d, g, b, plan.tables))
