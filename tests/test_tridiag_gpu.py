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


def _raw_solve(a, b, c, d, x, lanes):
    """dgb_tridiag_solve_lanes on raw pointers (views may start anywhere)."""
    from dendra_gb300 import _lib

    L = _lib.load()
    B, K = b.shape
    rc = L.dgb_tridiag_solve_lanes(_lib.dtype_code(d.dtype), B, K, a.data_ptr(), b.data_ptr(),
                                   c.data_ptr(), d.data_ptr(), x.data_ptr(), int(lanes),
                                   _lib.stream_ptr(d.device))
    _lib.check(rc, "dgb_tridiag_solve_lanes")


def _bands(rng, B, K, dtype, device, offset=0):
    """Diagonally dominant bands; with offset > 0 every band is a view that
    starts `offset` elements into its buffer (not 16-byte aligned)."""
    out = []
    for shape, gen in (((B, K - 1), lambda s: -rng.random(s)), ((B, K), lambda s: 2.2 + rng.random(s)),
                       ((B, K - 1), lambda s: -rng.random(s)), ((B, K), rng.standard_normal)):
        n = shape[0] * shape[1]
        buf = torch.empty(n + offset, dtype=dtype, device=device)
        view = buf[offset:].view(shape)
        view.copy_(torch.as_tensor(gen(shape)))
        out.append(view)
    return out


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("K", [1, 2, 3, 7, 31, 33, 101, 129, 401, 403, 600, 777, 1024])
@pytest.mark.parametrize("lanes", [0, 4, 8, 16, 32])
def test_bulk_staged_equals_register_direct(cuda, dtype, K, lanes):
    """Aligned bands run the bulk-staged kernel (shared-memory stages filled
    by cp.async.bulk; long systems in two- or one-warp CTAs), bands offset by
    one element the register-direct one: the arithmetic is the same, so the
    solutions agree bit for bit, for ragged last tiles (B not a multiple of
    the tile) and every lane split."""
    from dendra_gb300.solvers import tridiag_status

    for B in (1, 5, 259):
        seed = K * 1000 + lanes * 10 + B
        al = _bands(np.random.default_rng(seed), B, K, dtype, cuda)
        un = _bands(np.random.default_rng(seed), B, K, dtype, cuda, offset=1)
        assert all(t.data_ptr() % 16 == 0 for t in al)
        assert all(t.data_ptr() % 16 != 0 for t in un if t.numel())
        x_al = torch.full((B, K), float("nan"), dtype=dtype, device=cuda)
        x_un = torch.full((B * K + 1,), float("nan"), dtype=dtype, device=cuda)[1:].view(B, K)
        _raw_solve(*al, x_al, lanes)
        _raw_solve(*un, x_un, lanes)
        tridiag_status(cuda)
        assert torch.equal(x_al, x_un), (B, K, lanes)
        # in place (x aliases d), as the reference's kernels allow
        d_in = al[3].clone()
        _raw_solve(al[0], al[1], al[2], d_in, d_in, lanes)
        tridiag_status(cuda)
        assert torch.equal(d_in, x_al)


def test_bulk_stage_wait_timeout_surfaces(cuda):
    """A stage wait limited to zero polls gives up at once: each CTA drains its
    posted copies at the full limit, flags the fault and ends; the status call
    raises DgbTimeout, and with the default restored the same solve is right on
    the same context.  The copies are real, in-bounds bulk loads: nothing
    faults or hangs."""
    from dendra_gb300 import _lib
    from dendra_gb300.solvers import tridiag_status

    L = _lib.load()
    rng = np.random.default_rng(11)
    B, K = 4096, 401
    a, b, c, d = _bands(rng, B, K, torch.float32, cuda)
    x = torch.empty_like(d)
    try:
        assert L.dgb_tridiag_set_wait_limit(0) == 0
        _raw_solve(a, b, c, d, x, 0)
        with pytest.raises(_lib.DgbTimeout, match="still usable"):
            tridiag_status(cuda)
    finally:
        assert L.dgb_tridiag_set_wait_limit(-1) == 0
    tridiag_status(cuda)  # the flag was cleared by the read
    _raw_solve(a, b, c, d, x, 0)
    tridiag_status(cuda)
    ref = oracle.thomas(*(t.double().cpu().numpy() for t in (a, b, c, d)))
    np.testing.assert_allclose(x.double().cpu().numpy(), ref, rtol=5e-5, atol=5e-6)
