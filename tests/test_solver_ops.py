"""The tridiagonal solve as a torch.library operator: its fake rule (no GPU
needed) and, on the GPU, vmap, batched gradients and a torch.compile trace
agreeing with plain calls — the compatibility the reference's operator
registrations provide (triton/t_kernel_thomas.py:192-215)."""

import numpy as np
import pytest
import torch

from dendra_gb300.solvers import thomas_solve_cuda_t, tridiag_solve_op


def test_fake_rule_gives_the_solution_shape():
    from torch._subclasses.fake_tensor import FakeTensorMode

    with FakeTensorMode():
        a = torch.empty(4, 9, device="cuda", dtype=torch.float64)
        b = torch.empty(4, 10, device="cuda", dtype=torch.float64)
        x = thomas_solve_cuda_t(a, b, a, b)
        assert x.shape == (4, 10) and x.dtype == torch.float64 and x.device.type == "cuda"
        y = tridiag_solve_op(a, b, a, b, 0, True)
        assert y.shape == (4, 10)


def test_contract_errors_before_any_device_work():
    """Shape and device checks run on the host, with the reference's messages
    (triton/_contracts.py:87-159), so they raise without a GPU."""
    from dendra_gb300.solvers import pcr_solve_cuda_t

    a, c = torch.zeros(2, 3), torch.zeros(2, 3)
    b, d = torch.ones(2, 4), torch.zeros(2, 4)
    for solve in (thomas_solve_cuda_t, pcr_solve_cuda_t):
        with pytest.raises(ValueError, match="must be CUDA tensors"):
            solve(a, b, c, d)
        with pytest.raises(ValueError, match=r"d must have shape \(2, 4\), got \(2, 5\)"):
            solve(a, b, c, torch.zeros(2, 5))
        with pytest.raises(ValueError, match=r"a must have shape \(2, 3\)"):
            solve(b, b, c, d)


def _system(rng, B, K, dev):
    a = -rng.random((B, K - 1))
    c = -rng.random((B, K - 1))
    b = 3.0 + rng.random((B, K))
    d = rng.standard_normal((B, K))
    return [torch.as_tensor(t, device=dev) for t in (a, b, c, d)]


@pytest.mark.gpu
def test_vmap_matches_separate_solves(cuda):
    rng = np.random.default_rng(0)
    V, B, K = 5, 7, 33
    a, b, c, d = _system(rng, V * B, K, cuda)
    shape = lambda t: t.reshape(V, B, -1)  # noqa: E731
    x = torch.func.vmap(thomas_solve_cuda_t)(shape(a), shape(b), shape(c), shape(d))
    ref = thomas_solve_cuda_t(a, b, c, d).reshape(V, B, K)
    torch.testing.assert_close(x, ref, rtol=0, atol=0)
    # a mapped right-hand side with shared matrices
    x2 = torch.func.vmap(thomas_solve_cuda_t, in_dims=(None, None, None, 0))(
        a[:B], b[:B], c[:B], shape(d))
    ref2 = torch.stack([thomas_solve_cuda_t(a[:B], b[:B], c[:B], d.reshape(V, B, K)[v])
                        for v in range(V)])
    torch.testing.assert_close(x2, ref2, rtol=0, atol=0)


@pytest.mark.gpu
def test_batched_gradients_and_compile_trace(cuda):
    rng = np.random.default_rng(1)
    a, b, c, d = _system(rng, 6, 40, cuda)
    w = torch.as_tensor(rng.standard_normal((3, 6, 40)), device=cuda)

    # batched vector-Jacobian products: the backward's own solve runs under
    # vmap (the operator's vmap rule), as the reference's adjoint operator does
    bb, dd = b.clone().requires_grad_(), d.clone().requires_grad_()
    x = thomas_solve_cuda_t(a, bb, c, dd)
    gb, gd = torch.autograd.grad(x, (bb, dd), grad_outputs=w, is_grads_batched=True)
    for v in range(3):
        bb, dd = b.clone().requires_grad_(), d.clone().requires_grad_()
        (thomas_solve_cuda_t(a, bb, c, dd) * w[v]).sum().backward()
        torch.testing.assert_close(gb[v], bb.grad, rtol=1e-12, atol=1e-12)
        torch.testing.assert_close(gd[v], dd.grad, rtol=1e-12, atol=1e-12)
    compiled = torch.compile(lambda a_, b_, c_, d_: thomas_solve_cuda_t(a_, b_, c_, d_) * 2.0,
                             backend="aot_eager", fullgraph=True)
    torch.testing.assert_close(compiled(a, b, c, d), thomas_solve_cuda_t(a, b, c, d) * 2.0,
                               rtol=0, atol=0)
