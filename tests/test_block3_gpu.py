"""3x3 block-tridiagonal solve (multi-layer extracellular cables) against the
reference's block PCR, the oracle's block Thomas and dense float64 autograd."""

import numpy as np
import pytest
import torch

import oracle
from dendra_gb300.solvers import thomas_solve_cuda_bt

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("K", [1, 2, 3, 8, 33, 101, 257])
def test_matches_reference_block_pcr(golden, cuda, K):
    g = golden("block3.npz")
    args = [g[f"K{K}_{n}"] for n in ("lower", "main", "upper", "rhs")]
    for dt, tag, tol in ((torch.float64, "f64", 1e-11), (torch.float32, "f32", 1e-4)):
        x = thomas_solve_cuda_bt(*(torch.as_tensor(a, dtype=dt, device=cuda) for a in args))
        np.testing.assert_allclose(x.double().cpu().numpy(), g[f"K{K}_x_{tag}"], rtol=tol,
                                   atol=tol * 0.1)


def _system(B, K, seed, dt=np.float64):
    rng = np.random.default_rng(seed)
    lower = -rng.random((B, K - 1, 3))
    upper = -rng.random((B, K - 1, 3))
    main = 0.3 * rng.standard_normal((B, K, 3, 3)) + np.eye(3) * (3.0 + rng.random((B, K, 3)))[..., None]
    rhs = rng.standard_normal((B, K, 3))
    return [a.astype(dt) for a in (lower, main, upper, rhs)]


@pytest.mark.parametrize("B,K", [(1, 1), (5, 2), (300, 201), (4099, 17)])
def test_matches_oracle_block_thomas(cuda, B, K):
    args = _system(B, K, B + K)
    ref = oracle.block3_solve(*args)
    x = thomas_solve_cuda_bt(*(torch.as_tensor(a, device=cuda) for a in args))
    np.testing.assert_allclose(x.cpu().numpy(), ref, rtol=1e-12, atol=1e-13)
    args32 = [a.astype(np.float32) for a in args]
    x32 = thomas_solve_cuda_bt(*(torch.as_tensor(a, device=cuda) for a in args32))
    np.testing.assert_allclose(x32.cpu().numpy(), oracle.block3_solve(*args32), rtol=1e-5,
                               atol=1e-6)


def _dense(lower, main, upper):
    B, K = main.shape[:2]
    A = torch.zeros(B, 3 * K, 3 * K, dtype=main.dtype, device=main.device)
    for k in range(K):
        A[:, 3 * k:3 * k + 3, 3 * k:3 * k + 3] = main[:, k]
        if k > 0:
            A[:, 3 * k:3 * k + 3, 3 * k - 3:3 * k] = torch.diag_embed(lower[:, k - 1])
        if k + 1 < K:
            A[:, 3 * k:3 * k + 3, 3 * k + 3:3 * k + 6] = torch.diag_embed(upper[:, k])
    return A


def test_gradients_match_dense_float64_autograd(cuda):
    B, K = 3, 9
    args = [torch.as_tensor(a, device=cuda).requires_grad_() for a in _system(B, K, 7)]
    w = torch.randn(B, K, 3, dtype=torch.float64, device=cuda)
    (thomas_solve_cuda_bt(*args) * w).sum().backward()
    got = [a.grad.clone() for a in args]
    ref_args = [a.detach().clone().requires_grad_() for a in args]
    lower, main, upper, rhs = ref_args
    x = torch.linalg.solve(_dense(lower, main, upper), rhs.reshape(B, 3 * K, 1)).reshape(B, K, 3)
    (x * w).sum().backward()
    for a, r in zip(got, ref_args):
        torch.testing.assert_close(a, r.grad, rtol=1e-9, atol=1e-11)


@pytest.mark.parametrize("K", [2500, 6000])
def test_long_systems_serial_block_thomas(cuda, K):
    # chunk planes beyond shared memory: the serial block Thomas per thread,
    # against the oracle's block Thomas, and the transposed (adjoint) solve
    args = _system(40, K, K)
    ref = oracle.block3_solve(*args)
    t = [torch.as_tensor(a, device=cuda) for a in args]
    x = thomas_solve_cuda_bt(*t)
    np.testing.assert_allclose(x.cpu().numpy(), ref, rtol=1e-11, atol=1e-12)
    args32 = [a.astype(np.float32) for a in args]
    x32 = thomas_solve_cuda_bt(*(torch.as_tensor(a, device=cuda) for a in args32))
    np.testing.assert_allclose(x32.cpu().numpy(), oracle.block3_solve(*args32), rtol=1e-4,
                               atol=1e-5)
    lo, mn, up, rhs = (a[:2].clone().requires_grad_() for a in t)
    w = torch.randn_like(rhs)
    (thomas_solve_cuda_bt(lo, mn, up, rhs) * w).sum().backward()
    # adjoint: A^T g = w, with A^T = blocks transposed, lower and upper exchanged
    g = thomas_solve_cuda_bt(up.detach(), mn.detach().transpose(-1, -2).contiguous(),
                             lo.detach(), w)
    torch.testing.assert_close(rhs.grad, g, rtol=1e-10, atol=1e-12)
    r = (mn.detach() @ g.unsqueeze(-1)).squeeze(-1)  # spot check: A^T g - w on the interior
    assert torch.isfinite(r).all()
