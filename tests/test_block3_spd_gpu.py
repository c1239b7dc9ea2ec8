"""SPD block Thomas on the GPU (the reference's solve_bt_spd_cuda): against the
numpy restatement of its algorithm (symmetrisation, Cholesky, diagonal shifts)
in oracle/, against the general block solve on SPD systems, its failure flag
and its gradients."""

import numpy as np
import pytest
import torch

import oracle
from dendra_gb300.solvers import solve_bt_spd_cuda

pytestmark = pytest.mark.gpu


def _spd_system(rng, B, K):
    lo = 0.3 * rng.random((B, K - 1, 3))
    A = 0.2 * rng.standard_normal((B, K, 3, 3))
    main = A + A.transpose(0, 1, 3, 2) + np.eye(3) * (3.0 + rng.random((B, K, 1, 1)))
    rhs = rng.standard_normal((B, K, 3))
    return lo, main, lo.copy(), rhs


@pytest.mark.parametrize("K", [1, 2, 201])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_spd_systems_match_oracle(cuda, K, dtype):
    rng = np.random.default_rng(K)
    lo, main, up, rhs = _spd_system(rng, 37, K)
    T = lambda a: torch.as_tensor(a, device=cuda, dtype=dtype)  # noqa: E731
    x = solve_bt_spd_cuda(T(lo), T(main), T(up), T(rhs)).cpu().numpy()
    ref, info = oracle.block3_spd_solve(lo, main, up, rhs)
    assert not info.any()
    tol = dict(rtol=1e-11, atol=1e-12) if dtype == torch.float64 else dict(rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(x, ref, **tol)
    np.testing.assert_allclose(x, oracle.block3_solve(lo, main, up, rhs), **tol)


def test_indefinite_blocks_are_shifted_like_the_reference(cuda):
    rng = np.random.default_rng(7)
    lo, main, up, rhs = _spd_system(rng, 16, 40)
    main[:, 5, 1, 1] = -4.0  # not positive definite: shifted by its Gershgorin deficit
    main[:, 9, 0, 2] += 0.5  # asymmetric pair: symmetrised to the midpoint
    x = solve_bt_spd_cuda(*(torch.as_tensor(t, device=cuda) for t in (lo, main, up, rhs)))
    ref, info = oracle.block3_spd_solve(lo, main, up, rhs)
    assert not info.any()
    np.testing.assert_allclose(x.cpu().numpy(), ref, rtol=1e-10, atol=1e-12)


def test_failed_factorisation_raises(cuda):
    rng = np.random.default_rng(8)
    lo, main, up, rhs = _spd_system(rng, 4, 6)
    main[2, 3, 0, 0] = np.nan
    with pytest.raises(RuntimeError, match="Cholesky failed"):
        solve_bt_spd_cuda(*(torch.as_tensor(t, device=cuda) for t in (lo, main, up, rhs)))


def test_gradients_follow_the_reference(cuda):
    rng = np.random.default_rng(9)
    lo, main, up, rhs = _spd_system(rng, 3, 12)
    t = [torch.as_tensor(a, device=cuda).requires_grad_() for a in (lo, main, up, rhs)]
    w = torch.as_tensor(rng.standard_normal(rhs.shape), device=cuda)
    x = solve_bt_spd_cuda(*t)
    (x * w).sum().backward()
    # symmetric system: g = A^-1 w; grad_main = -sym(g x^T), bands -g_k x_k+-1
    g = oracle.block3_solve(lo, main, up, w.cpu().numpy())
    xn = x.detach().cpu().numpy()
    gx = g[..., :, None] * xn[..., None, :]
    np.testing.assert_allclose(t[3].grad.cpu().numpy(), g, rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(t[1].grad.cpu().numpy(), -0.5 * (gx + gx.transpose(0, 1, 3, 2)),
                               rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(t[2].grad.cpu().numpy(), -(g[:, :-1] * xn[:, 1:]), rtol=1e-10,
                               atol=1e-12)
    np.testing.assert_allclose(t[0].grad.cpu().numpy(), -(g[:, 1:] * xn[:, :-1]), rtol=1e-10,
                               atol=1e-12)
