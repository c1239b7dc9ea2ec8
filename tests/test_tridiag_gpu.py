"""Batched tridiagonal solves on the GPU against the reference and the oracle."""

import numpy as np
import pytest
import torch

import oracle
from dendra_gb300 import solvers
from dendra_gb300.solvers import pcr_solve_cuda_t, thomas_solve_cuda_t

pytestmark = pytest.mark.gpu

# reference parity tolerances (tests/test_cuda_solver_parity.py:66-110)
TOL = {torch.float32: dict(rtol=5e-5, atol=5e-6), torch.float64: dict(rtol=3e-12, atol=3e-12)}


@pytest.mark.parametrize("K", [1, 2, 3, 7, 33, 101, 401])
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("solve", [thomas_solve_cuda_t, pcr_solve_cuda_t])
def test_matches_reference_golden(cuda, golden, K, dtype, solve):
    g = golden("tridiag.npz")
    a, b, c, d = (torch.as_tensor(g[f"K{K}_{x}"]).to(cuda, dtype) for x in "abcd")
    x = solve(a, b, c, d)
    tag = "f64" if dtype == torch.float64 else "f32"
    ref = torch.as_tensor(g[f"K{K}_f64_thomas"]).to(cuda, dtype)
    torch.testing.assert_close(x, ref, **TOL[dtype])
    ref_same = torch.as_tensor(g[f"K{K}_{tag}_thomas"]).to(cuda, dtype)
    torch.testing.assert_close(x, ref_same, **TOL[dtype])


@pytest.mark.parametrize("K", [1, 5, 31, 32, 33, 64, 65, 129, 200, 401, 512, 777, 1024])
@pytest.mark.parametrize("lanes", [0, 4, 8, 16, 32])
def test_random_systems_match_oracle_every_split(cuda, K, lanes):
    rng = np.random.default_rng(K * 7 + lanes)
    B = 257
    a = -rng.random((B, K - 1))
    c = -rng.random((B, K - 1))
    b = 2.2 + rng.random((B, K))
    d = rng.standard_normal((B, K))
    ref = oracle.thomas(a, b, c, d)
    args = [torch.as_tensor(t, device=cuda) for t in (a, b, c, d)]
    if lanes == 0:
        x = thomas_solve_cuda_t(*args)
    else:  # a split too narrow for K widens to 32 lanes inside the library
        x = solvers.tridiag_solve_lanes(*args, lanes)
    np.testing.assert_allclose(x.cpu().numpy(), ref, rtol=1e-11, atol=1e-12)
    x32 = thomas_solve_cuda_t(*[t.float() for t in args])
    np.testing.assert_allclose(x32.cpu().numpy(), ref, rtol=5e-5, atol=5e-6)


def test_gradients_match_dense_autograd(cuda):
    """Adjoint (transpose solve) vs dense fp64 autograd (reference tolerance 3e-10)."""
    rng = np.random.default_rng(3)
    B, K = 4, 37
    a = torch.as_tensor(-rng.random((B, K - 1)), device=cuda).requires_grad_()
    c = torch.as_tensor(-rng.random((B, K - 1)), device=cuda).requires_grad_()
    b = torch.as_tensor(2.5 + rng.random((B, K)), device=cuda).requires_grad_()
    d = torch.as_tensor(rng.standard_normal((B, K)), device=cuda).requires_grad_()
    w = torch.as_tensor(rng.standard_normal((B, K)), device=cuda)
    x = thomas_solve_cuda_t(a, b, c, d)
    (x * w).sum().backward()
    grads = [t.grad.clone() for t in (a, b, c, d)]
    for t in (a, b, c, d):
        t.grad = None
    A = torch.diag_embed(b) + torch.diag_embed(a, -1) + torch.diag_embed(c, 1)
    xd = torch.linalg.solve(A, d.unsqueeze(-1)).squeeze(-1)
    (xd * w).sum().backward()
    for gk, t in zip(grads, (a, b, c, d)):
        torch.testing.assert_close(gk, t.grad, rtol=3e-10, atol=3e-10)


def test_contract_errors(cuda):
    a = torch.zeros(2, 3, device=cuda)
    b = torch.ones(2, 4, device=cuda)
    with pytest.raises(ValueError, match="must be CUDA tensors"):
        thomas_solve_cuda_t(a.cpu(), b.cpu(), a.cpu(), b.cpu())
    with pytest.raises(TypeError, match="float32 and float64"):
        thomas_solve_cuda_t(a.half(), b.half(), a.half(), b.half())
    with pytest.raises(ValueError, match="a must have shape"):
        thomas_solve_cuda_t(b, b, a, b)
    with pytest.raises(ValueError, match="same dtype"):
        thomas_solve_cuda_t(a, b.double(), a, b)
    # no length limit: 1,100 rows run the sequential recurrence
    big = torch.ones(1, 1100, device=cuda)
    x = thomas_solve_cuda_t(-0.25 * big[:, 1:], big, -0.25 * big[:, 1:], big)
    assert torch.isfinite(x).all()


@pytest.mark.parametrize("K", [1025, 5000])
def test_long_systems_equal_sequential_thomas(cuda, K):
    # beyond the register-resident chunks: the serial recurrence, bit-identical
    # to the oracle's sequential Thomas in both precisions
    rng = np.random.default_rng(K)
    B = 300
    a = -rng.random((B, K - 1))
    c = -rng.random((B, K - 1))
    b = 2.2 + rng.random((B, K))
    d = rng.standard_normal((B, K))
    for dt in (np.float64, np.float32):
        args = [torch.as_tensor(t.astype(dt), device=cuda) for t in (a, b, c, d)]
        ref = oracle.thomas(*(t.astype(dt) for t in (a, b, c, d)))
        np.testing.assert_array_equal(thomas_solve_cuda_t(*args).cpu().numpy(), ref)
        np.testing.assert_array_equal(pcr_solve_cuda_t(*args).cpu().numpy(), ref)
    # the adjoint (transpose solve) of a long system
    at, bt, ct, dtn = (torch.as_tensor(t[:3], device=cuda).requires_grad_() for t in (a, b, c, d))
    w = torch.as_tensor(rng.standard_normal((3, K)), device=cuda)
    (thomas_solve_cuda_t(at, bt, ct, dtn) * w).sum().backward()
    A = (torch.diag_embed(bt.detach()) + torch.diag_embed(at.detach(), -1)
         + torch.diag_embed(ct.detach(), 1))
    g = torch.linalg.solve(A.transpose(-1, -2), w)
    torch.testing.assert_close(dtn.grad, g, rtol=1e-9, atol=1e-11)
