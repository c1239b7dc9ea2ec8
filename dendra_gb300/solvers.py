"""Solver callables with the reference's signatures, backed by sm_103a kernels.

Drop-ins for the solver objects ``_bwd_euler_ub._select_solver`` installs as
``self._solve`` (dendra/models/integrators/implicit.py:364-440):

* :func:`thomas_solve_cuda_t` — replaces triton/t_kernel_thomas.py:218-232
* :func:`pcr_solve_cuda_t`    — replaces triton/pcr_kernel_thomas.py:199-226
* :func:`thomas_solve_cuda_bt` — the 3x3 block solver ``_bwd_euler_bt`` selects
  on CUDA (implicit.py:905-950), replaces triton/bt_kernel.py:195-298

Both take ``a (B,K-1), b (B,K), c (B,K-1), d (B,K)`` CUDA tensors of one float
dtype and return a fresh ``x (B,K)``.  Gradients follow the reference's
``ThomasSolve.backward`` (t_kernel_thomas.py:147-189): one transpose solve
``A^T y = grad_x`` on the kernel, then ``grad_b = -y x``,
``grad_a = -y[:,1:] x[:,:-1]``, ``grad_c = -y[:,:-1] x[:,1:]``.
Argument checks raise the reference's exception types and messages
(triton/_contracts.py:87-159).
"""

from __future__ import annotations

import torch

from . import _lib

_FLOAT_DTYPES = (torch.float32, torch.float64)


def _validate_float_group(named):
    first_name, first = named[0]
    if first.device.type != "cuda":
        raise ValueError("Triton solver inputs must be CUDA tensors")
    if first.dtype not in _FLOAT_DTYPES:
        raise TypeError("Triton solvers support only float32 and float64")
    for name, tensor in named[1:]:
        if tensor.device != first.device:
            raise ValueError(
                f"{name} must be on the same device as {first_name}; "
                f"got {tensor.device} and {first.device}"
            )
        if tensor.dtype != first.dtype:
            raise ValueError(
                f"{name} must have the same dtype as {first_name}; "
                f"got {tensor.dtype} and {first.dtype}"
            )


def validate_tridiagonal(a, b, c, d):
    """Shape/dtype/device contract of a batched scalar tridiagonal solve."""
    named = (("a", a), ("b", b), ("c", c), ("d", d))
    for name, t in named:
        if not isinstance(t, torch.Tensor):
            raise TypeError(f"{name} must be a torch.Tensor")
    if b.ndim != 2:
        raise ValueError(f"b must have shape (B, K), got {tuple(b.shape)}")
    batch, size = map(int, b.shape)
    if batch < 1 or size < 1:
        raise ValueError("B and K must both be >= 1")
    band = (batch, size - 1)
    if tuple(a.shape) != band:
        raise ValueError(f"a must have shape {band}, got {tuple(a.shape)}")
    if tuple(c.shape) != band:
        raise ValueError(f"c must have shape {band}, got {tuple(c.shape)}")
    if tuple(d.shape) != (batch, size):
        raise ValueError(f"d must have shape {(batch, size)}, got {tuple(d.shape)}")
    _validate_float_group(named)
    return batch, size


def _solve(a, b, c, d, method, lanes=0):
    B, K = b.shape
    a, b, c, d = (t.contiguous() for t in (a, b, c, d))
    x = torch.empty_like(d)
    L = _lib.load()
    with torch.cuda.device(d.device):
        st = _lib.stream_ptr(d.device)
        if lanes:
            rc = L.dgb_tridiag_solve_lanes(_lib.dtype_code(d.dtype), B, K, a.data_ptr(),
                                           b.data_ptr(), c.data_ptr(), d.data_ptr(),
                                           x.data_ptr(), int(lanes), st)
        else:
            rc = L.dgb_tridiag_solve(_lib.dtype_code(d.dtype), method, B, K, a.data_ptr(),
                                     b.data_ptr(), c.data_ptr(), d.data_ptr(), x.data_ptr(), st)
    _lib.check(rc, "dgb_tridiag_solve")
    return x


def _solve_transpose(a, b, c, g):
    B, K = b.shape
    a, b, c, g = (t.contiguous() for t in (a, b, c, g))
    y = torch.empty_like(g)
    L = _lib.load()
    with torch.cuda.device(g.device):
        rc = L.dgb_tridiag_solve_transpose(_lib.dtype_code(g.dtype), B, K, a.data_ptr(),
                                           b.data_ptr(), c.data_ptr(), g.data_ptr(),
                                           y.data_ptr(), _lib.stream_ptr(g.device))
    _lib.check(rc, "dgb_tridiag_solve_transpose")
    return y


# The solve as a torch.library operator, like the reference's
# (t_kernel_thomas.py:192-215): a fake (shape) rule for torch.compile, the
# transpose-solve adjoint as its autograd rule, and a vmap rule that folds
# mapped dimensions into the system batch.
@torch.library.custom_op("dendra_gb300::tridiag_solve", mutates_args=())
def tridiag_solve_op(a: torch.Tensor, b: torch.Tensor, c: torch.Tensor, d: torch.Tensor,
                     method: int, transpose: bool) -> torch.Tensor:
    """x with A x = d (transpose: A^T x = d); A has sub-diagonal a, diagonal b,
    super-diagonal c."""
    if transpose:
        return _solve_transpose(a, b, c, d)
    return _solve(a, b, c, d, method)


@tridiag_solve_op.register_fake
def _(a, b, c, d, method, transpose):
    return d.new_empty(d.shape)


def _tridiag_setup(ctx, inputs, output):
    a, b, c, _, method, transpose = inputs
    ctx.save_for_backward(a, b, c, output)
    ctx.method, ctx.transpose = method, transpose


def _tridiag_backward(ctx, grad_x):
    # ThomasSolve.backward (t_kernel_thomas.py:147-189): one solve with the
    # transposed matrix, then outer products along the three diagonals
    a, b, c, x = ctx.saved_tensors
    need = ctx.needs_input_grad
    if not any(need[:4]):
        return None, None, None, None, None, None
    y = tridiag_solve_op(a, b, c, grad_x.contiguous(), ctx.method, not ctx.transpose)
    lower = -y[:, 1:] * x[:, :-1]   # cotangent of the sub-diagonal actually used
    upper = -y[:, :-1] * x[:, 1:]
    grad_a, grad_c = (upper, lower) if ctx.transpose else (lower, upper)
    return (grad_a if need[0] else None, -y * x if need[1] else None,
            grad_c if need[2] else None, y if need[3] else None, None, None)


tridiag_solve_op.register_autograd(_tridiag_backward, setup_context=_tridiag_setup)


@tridiag_solve_op.register_vmap
def _(info, in_dims, a, b, c, d, method, transpose):
    V = info.batch_size

    def fold(t, dim):
        t = t.movedim(dim, 0) if dim is not None else t.unsqueeze(0).expand(V, *t.shape)
        return t.reshape(V * t.shape[1], *t.shape[2:]).contiguous()

    a, b, c, d = (fold(t, dim) for t, dim in zip((a, b, c, d), in_dims[:4]))
    x = tridiag_solve_op(a, b, c, d, method, transpose)
    return x.reshape(V, -1, x.shape[-1]), 0


def thomas_solve_cuda_t(a, b, c, d):
    """Batched tridiagonal solve (drop-in for the reference's Triton Thomas)."""
    validate_tridiagonal(a, b, c, d)
    return tridiag_solve_op(a, b, c, d, _lib.THOMAS, False)


def pcr_solve_cuda_t(a, b, c, d):
    """Batched tridiagonal solve (drop-in for the reference's Triton PCR)."""
    validate_tridiagonal(a, b, c, d)
    return tridiag_solve_op(a, b, c, d, _lib.PCR, False)


def tridiag_status(device) -> None:
    """Raise ``DgbTimeout`` if a bounded stage wait inside a bulk-staged
    tridiagonal solve on ``device`` gave up since the last call (those systems
    were then not solved).  Synchronises the current stream."""
    with torch.cuda.device(device):
        rc = _lib.load().dgb_tridiag_status(_lib.stream_ptr(device))
    _lib.check(rc, "bulk-staged tridiagonal solve")


def tridiag_solve_lanes(a, b, c, d, lanes: int):
    """Forward-only solve with an explicit lanes-per-system split (autotuner)."""
    validate_tridiagonal(a, b, c, d)
    return _solve(a, b, c, d, _lib.THOMAS, lanes=lanes)


# The increment-RHS contract is granted to these solver identities only
# (mirrors _BWD_EULER_INCREMENT_SOLVERS, integrators/implicit.py:59-82).
INCREMENT_SOLVERS = (thomas_solve_cuda_t, pcr_solve_cuda_t)


# ---------------------------------------------------------------------------
# 3x3 block-tridiagonal systems (multi-layer extracellular cables)
# ---------------------------------------------------------------------------
def validate_block_tridiagonal(lower, main, upper, rhs):
    """Contract of a batched 3x3 block-tridiagonal solve (triton/_contracts.py:162-196)."""
    named = (("lower", lower), ("main", main), ("upper", upper), ("rhs", rhs))
    for name, t in named:
        if not isinstance(t, torch.Tensor):
            raise TypeError(f"{name} must be a torch.Tensor")
    if rhs.ndim != 3 or rhs.shape[-1] != 3:
        raise ValueError(f"rhs must have shape (B, K, 3), got {tuple(rhs.shape)}")
    batch, size, _ = map(int, rhs.shape)
    if batch < 1 or size < 1:
        raise ValueError("B and K must both be >= 1")
    band = (batch, size - 1, 3)
    if tuple(lower.shape) != band:
        raise ValueError(f"lower must have shape {band}, got {tuple(lower.shape)}")
    if tuple(upper.shape) != band:
        raise ValueError(f"upper must have shape {band}, got {tuple(upper.shape)}")
    expected_main = (batch, size, 3, 3)
    if tuple(main.shape) != expected_main:
        raise ValueError(f"main must have shape {expected_main}, got {tuple(main.shape)}")
    _validate_float_group(named)
    return batch, size


def _block3(lower, main, upper, rhs, transpose):
    B, K = rhs.shape[:2]
    lower, main, upper, rhs = (t.contiguous() for t in (lower, main, upper, rhs))
    x = torch.empty_like(rhs)
    L = _lib.load()
    code = _lib.dtype_code(rhs.dtype)
    nwork = L.dgb_block3_work_size(code, B, K)
    work = torch.empty(nwork, dtype=torch.uint8, device=rhs.device) if nwork else None
    with torch.cuda.device(rhs.device):
        rc = L.dgb_block3_solve(code, B, K, lower.data_ptr(), main.data_ptr(), upper.data_ptr(),
                                rhs.data_ptr(), x.data_ptr(),
                                None if work is None else work.data_ptr(), int(transpose),
                                _lib.stream_ptr(rhs.device))
    _lib.check(rc, "dgb_block3_solve")
    return x


class _Block3Solve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, lower, main, upper, rhs):
        x = _block3(lower, main, upper, rhs, False)
        ctx.save_for_backward(lower, main, upper, x)
        return x

    @staticmethod
    def backward(ctx, grad_x):
        # adjoint solve A^T g = grad_x on the kernel (transposed blocks,
        # exchanged bands), then the outer products of triton/bt_kernel.py:268-290
        lower, main, upper, x = ctx.saved_tensors
        g = _block3(lower, main, upper, grad_x.contiguous(), True)
        grad_main = -(g.unsqueeze(-1) * x.unsqueeze(-2))
        grad_upper = -(g[:, :-1] * x[:, 1:])
        grad_lower = -(g[:, 1:] * x[:, :-1])
        return grad_lower, grad_main, grad_upper, g


def thomas_solve_cuda_bt(lower, main, upper, rhs):
    """Drop-in for the reference's thomas_solve_cuda_bt (triton/bt_kernel.py:295-298).

    lower, upper: (B, K-1, 3) diagonals of the off-diagonal blocks; main:
    (B, K, 3, 3); rhs: (B, K, 3).  Returns x (B, K, 3); differentiable."""
    validate_block_tridiagonal(lower, main, upper, rhs)
    return _Block3Solve.apply(lower, main, upper, rhs)


# ---------------------------------------------------------------------------
# SPD block Thomas (triton/bt_spd_kernel.py:583-755)
# ---------------------------------------------------------------------------
def _symmetric_part(value):
    """(value + value^T) / 2 per 3x3 block without overflow or loss of
    subnormals (the reference's integrators/_symmetry.py:6-30 rule)."""
    t = value.transpose(-1, -2)
    lim = torch.finfo(value.dtype)
    half_max = lim.max / 2.0
    bounded = (value.abs() <= half_max) & (t.abs() <= half_max)
    extreme = torch.where(value.abs() < 2.0 * lim.tiny, value + t * 0.5,
                          torch.where(t.abs() < 2.0 * lim.tiny, value * 0.5 + t,
                                      value * 0.5 + t * 0.5))
    return torch.where(bounded, (value + t) * 0.5, extreme)


def _block3_spd(lower, main, upper, rhs):
    B, K = rhs.shape[:2]
    lower, main, upper, rhs = (t.contiguous() for t in (lower, main, upper, rhs))
    x = torch.empty_like(rhs)
    chol = torch.empty(B, K, 9, dtype=rhs.dtype, device=rhs.device)
    info = torch.empty(B, K, dtype=torch.int32, device=rhs.device)
    with torch.cuda.device(rhs.device):
        rc = _lib.load().dgb_block3_spd_solve(
            _lib.dtype_code(rhs.dtype), B, K, lower.data_ptr(), main.data_ptr(),
            upper.data_ptr(), rhs.data_ptr(), x.data_ptr(), chol.data_ptr(), info.data_ptr(),
            _lib.stream_ptr(rhs.device))
    _lib.check(rc, "dgb_block3_spd_solve")
    # the reference asserts on the device; here the host reads the flags, so
    # a failed factorisation raises without faulting the context
    if bool((info != 0).any()):
        raise RuntimeError("solve_bt_spd_cuda: Cholesky failed after all diagonal bumps")
    return x, chol


def _block3_spd_with_chol(lower, upper, chol, rhs):
    B, K = rhs.shape[:2]
    rhs = rhs.contiguous()
    x = torch.empty_like(rhs)
    with torch.cuda.device(rhs.device):
        rc = _lib.load().dgb_block3_spd_solve_chol(
            _lib.dtype_code(rhs.dtype), B, K, lower.contiguous().data_ptr(),
            upper.contiguous().data_ptr(), chol.data_ptr(), rhs.data_ptr(), x.data_ptr(),
            _lib.stream_ptr(rhs.device))
    _lib.check(rc, "dgb_block3_spd_solve_chol")
    return x


class _Block3SpdSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, lower, main, upper, rhs):
        x, chol = _block3_spd(lower, main, upper, rhs)
        ctx.save_for_backward(lower, upper, x, chol)
        return x

    @staticmethod
    def backward(ctx, grad_x):
        # the reference's _SolveBTSPDCudaConsumeUnchecked.backward
        # (bt_spd_kernel.py:697-712): the cached factors solve the (symmetric)
        # system again; the main-block gradient is the symmetric part
        lower, upper, x, chol = ctx.saved_tensors
        g = _block3_spd_with_chol(lower, upper, chol, grad_x)
        grad_main = -_symmetric_part(g.unsqueeze(-1) * x.unsqueeze(-2))
        grad_upper = -(g[:, :-1] * x[:, 1:])
        grad_lower = -(g[:, 1:] * x[:, :-1])
        return grad_lower, grad_main, grad_upper, g


def solve_bt_spd_cuda(lower, main, upper, rhs):
    """Drop-in for the reference's solve_bt_spd_cuda (triton/bt_spd_kernel.py:744-755):
    SPD block Thomas on (B, K) systems of 3x3 blocks (lower/upper (B, K-1, 3),
    main (B, K, 3, 3), rhs (B, K, 3)); blocks are symmetrised and, when not
    positive definite, shifted on the diagonal like the reference's;
    differentiable with the reference's gradients."""
    validate_block_tridiagonal(lower, main, upper, rhs)
    return _Block3SpdSolve.apply(lower, main, upper, rhs)
