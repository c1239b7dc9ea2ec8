"""Functional solver facade on the GB300 kernels.

Mirror of the reference's functional CUDA solvers
(models/integrators/_cuda_functional.py: ``thomas_solve`` :594,
``pcr_solve`` :599, ``block_thomas_solve`` :604, ``block_spd_solve`` :609,
``dhs_solve`` :615, ``dhs_bt_solve`` :620, ``dhs_multi_solve`` :625), which the
reference's functional integrators import (integrators/implicit.py:16-17,
mechanisms/_spatial.py:837-841, 1980).  Every solve is a
``torch.autograd.Function`` with

* a reverse rule: the adjoint is a solve with the transposed matrix (lower and
  upper bands exchanged, main blocks transposed; trees are symmetric in their
  edges), then the reference's parameter gradients (:247-271, :365-374,
  :503-517);
* a forward-mode rule: ``dx = A^-1 (drhs - dA x)`` (:273-293, :376-393,
  :519-535), one more solve;
* a vmap rule: mapped dimensions fold into the solver batch, one launch
  (the topology must be shared, as the reference requires).

The reverse and forward rules call the same autograd functions, so higher
derivatives compose.  All launches are the package's CUDA kernels; there is no
CPU path.
"""

from __future__ import annotations

import torch

from . import _lib
from . import solvers as _sv
from . import tree as _tr


def _require_shared(in_dims):
    if any(d is not None for d in in_dims):
        raise ValueError("solver topology and configuration must be shared under vmap")


def _flatten(info, in_dims, *tensors):
    """Move mapped dimensions to the front and fold them into the solver batch."""
    V = info.batch_size
    flat = []
    for t, dim in zip(tensors, in_dims):
        t = t.unsqueeze(0).expand(V, *t.shape) if dim is None else t.movedim(dim, 0)
        flat.append(t.reshape(V * t.shape[1], *t.shape[2:]).contiguous())
    return flat


def _restore(x, V):
    return x.reshape(V, x.shape[0] // V, *x.shape[1:])


def _pad_cat(first, rest, axis, lead):
    """[first ; rest] or [rest ; first] along the row axis (tangent band terms)."""
    return torch.cat((first, rest) if lead else (rest, first), dim=axis)


# ---------------------------------------------------------------------------
# tridiagonal (scalar and 3x3 block)
# ---------------------------------------------------------------------------
def _raw_tridiagonal(a, b, c, rhs, block, pcr):
    if block:
        return _sv._block3(a, b, c, rhs, False)
    return _sv._solve(a, b, c, rhs, _lib.PCR if pcr else _lib.THOMAS)


class _Tridiagonal(torch.autograd.Function):
    @staticmethod
    def forward(a, b, c, rhs, block, pcr):
        return _raw_tridiagonal(a, b, c, rhs, block, pcr)

    @staticmethod
    def setup_context(ctx, inputs, output):
        a, b, c, _, ctx.block, ctx.pcr = inputs
        ctx.save_for_backward(a, b, c, output)
        ctx.save_for_forward(a, b, c, output)

    @staticmethod
    def backward(ctx, grad_x):
        a, b, c, x = ctx.saved_tensors
        main = b.transpose(-1, -2).contiguous() if ctx.block else b
        g = _Tridiagonal.apply(c, main, a, grad_x.contiguous(), ctx.block, ctx.pcr)
        axis = -2 if ctx.block else -1
        n = x.shape[axis]
        grad_main = -(g.unsqueeze(-1) * x.unsqueeze(-2)) if ctx.block else -(g * x)
        return (-(g.narrow(axis, 1, n - 1) * x.narrow(axis, 0, n - 1)), grad_main,
                -(g.narrow(axis, 0, n - 1) * x.narrow(axis, 1, n - 1)), g, None, None)

    @staticmethod
    def jvp(ctx, a_t, b_t, c_t, rhs_t, _block_t, _pcr_t):
        a, b, c, x = ctx.saved_tensors
        axis = -2 if ctx.block else -1
        n = x.shape[axis]
        pad = torch.zeros_like(x.narrow(axis, 0, 1))
        tangent = torch.zeros_like(x) if rhs_t is None else rhs_t
        if b_t is not None:
            tangent = tangent - ((b_t @ x.unsqueeze(-1)).squeeze(-1) if ctx.block else b_t * x)
        if a_t is not None:
            tangent = tangent - _pad_cat(pad, a_t * x.narrow(axis, 0, n - 1), axis, True)
        if c_t is not None:
            tangent = tangent - _pad_cat(pad, c_t * x.narrow(axis, 1, n - 1), axis, False)
        return _Tridiagonal.apply(a, b, c, tangent.contiguous(), ctx.block, ctx.pcr)

    @staticmethod
    def vmap(info, in_dims, a, b, c, rhs, block, pcr):
        _require_shared(in_dims[4:])
        flat = _flatten(info, in_dims[:4], a, b, c, rhs)
        return _restore(_Tridiagonal.apply(*flat, block, pcr), info.batch_size), 0


def thomas_solve(a, b, c, rhs):
    """Batched scalar Thomas solve, (B, K-1) bands, (B, K) main and rhs."""
    _sv.validate_tridiagonal(a, b, c, rhs)
    return _Tridiagonal.apply(a, b, c, rhs, False, False)


def pcr_solve(a, b, c, rhs):
    """Batched scalar PCR solve (same system as thomas_solve)."""
    _sv.validate_tridiagonal(a, b, c, rhs)
    return _Tridiagonal.apply(a, b, c, rhs, False, True)


def block_thomas_solve(lower, main, upper, rhs):
    """3x3 block-tridiagonal solve: lower/upper (B, K-1, 3) diagonal blocks,
    main (B, K, 3, 3), rhs (B, K, 3)."""
    _sv.validate_block_tridiagonal(lower, main, upper, rhs)
    return _Tridiagonal.apply(lower, main, upper, rhs, True, False)


# ---------------------------------------------------------------------------
# SPD 3x3 block solve with cached factors
# ---------------------------------------------------------------------------
class _SpdFactorSolve(torch.autograd.Function):
    """Solve with saved SPD block factors (the reference's block_spd_chol
    operator, _cuda_functional.py:101-123): linear in ``rhs`` and symmetric,
    so its reverse and forward rules are the same solve."""

    @staticmethod
    def forward(lower, upper, chol, rhs):
        return _sv._block3_spd_with_chol(lower, upper, chol, rhs)

    @staticmethod
    def setup_context(ctx, inputs, output):
        lower, upper, chol, _ = inputs
        ctx.save_for_backward(lower, upper, chol)
        ctx.save_for_forward(lower, upper, chol)

    @staticmethod
    def backward(ctx, grad):
        lower, upper, chol = ctx.saved_tensors
        return None, None, None, _SpdFactorSolve.apply(lower, upper, chol, grad.contiguous())

    @staticmethod
    def jvp(ctx, _lower_t, _upper_t, _chol_t, rhs_t):
        lower, upper, chol = ctx.saved_tensors
        return _SpdFactorSolve.apply(lower, upper, chol, rhs_t.contiguous())

    @staticmethod
    def vmap(info, in_dims, lower, upper, chol, rhs):
        flat = _flatten(info, in_dims, lower, upper, chol, rhs)
        return _restore(_SpdFactorSolve.apply(*flat), info.batch_size), 0


class _BlockSPD(torch.autograd.Function):
    @staticmethod
    def forward(lower, main, upper, rhs):
        return _sv._block3_spd(lower, main, upper, rhs)

    @staticmethod
    def setup_context(ctx, inputs, output):
        lower, _, upper, _ = inputs
        x, chol = output
        ctx.save_for_backward(lower, upper, x, chol)
        ctx.save_for_forward(lower, upper, x, chol)
        ctx.mark_non_differentiable(chol)
        ctx.set_materialize_grads(False)

    @staticmethod
    def backward(ctx, grad_x, _grad_chol):
        lower, upper, x, chol = ctx.saved_tensors
        if grad_x is None:
            return None, None, None, None
        g = _SpdFactorSolve.apply(lower, upper, chol, grad_x.contiguous())
        return (-(g[:, 1:] * x[:, :-1]), -_sv._symmetric_part(g.unsqueeze(-1) * x.unsqueeze(-2)),
                -(g[:, :-1] * x[:, 1:]), g)

    @staticmethod
    def jvp(ctx, lower_t, main_t, upper_t, rhs_t):
        lower, upper, x, chol = ctx.saved_tensors
        tangent = torch.zeros_like(x) if rhs_t is None else rhs_t
        if main_t is not None:  # the reverse rule's symmetric domain
            tangent = tangent - (_sv._symmetric_part(main_t) @ x.unsqueeze(-1)).squeeze(-1)
        pad = torch.zeros_like(x[:, :1])
        if lower_t is not None:
            tangent = tangent - torch.cat((pad, lower_t * x[:, :-1]), dim=-2)
        if upper_t is not None:
            tangent = tangent - torch.cat((upper_t * x[:, 1:], pad), dim=-2)
        return _SpdFactorSolve.apply(lower, upper, chol, tangent.contiguous()), None

    @staticmethod
    def vmap(info, in_dims, lower, main, upper, rhs):
        flat = _flatten(info, in_dims, lower, main, upper, rhs)
        x, chol = _BlockSPD.apply(*flat)
        return (_restore(x, info.batch_size), _restore(chol, info.batch_size)), (0, 0)


def block_spd_solve(lower, main, upper, rhs):
    """SPD 3x3 block solve (blocks symmetrised, shifted when not positive
    definite); the reverse and forward rules reuse the cached factors."""
    _sv.validate_block_tridiagonal(lower, main, upper, rhs)
    return _BlockSPD.apply(lower, main, upper, rhs)[0]


# ---------------------------------------------------------------------------
# trees (scalar and 3x3 block)
# ---------------------------------------------------------------------------
def _raw_tree(main, edge, rhs, parent, order, layers, block, transpose=False):
    if block:
        return _tr._block_solve(main, edge, rhs, _tr._checked_topology(parent, order, layers),
                                transpose)
    return _tr._solve(main, edge, rhs, _tr._device_topology(parent, order, layers))


def _tree_edge_gradient(x, g, parent, block):
    axis = -2 if block else -1
    safe = parent.clamp_min(0).long()
    root = (parent < 0).reshape((1, -1, 1) if block else (1, -1))
    return torch.where(root, -(g * x),
                       -((g - g.index_select(axis, safe)) * (x - x.index_select(axis, safe))))


def _tree_tangent(main_t, edge_t, rhs_t, x, parent, block):
    tangent = torch.zeros_like(x) if rhs_t is None else rhs_t
    if main_t is not None:
        tangent = tangent - ((main_t @ x.unsqueeze(-1)).squeeze(-1) if block else main_t * x)
    if edge_t is None:
        return tangent
    axis = -2 if block else -1
    shape = (1, -1, 1) if block else (1, -1)
    safe = parent.clamp_min(0).long()
    root = (parent < 0).reshape(shape)
    flow = torch.where(root, torch.zeros_like(x), edge_t * (x - x.index_select(axis, safe)))
    tangent = (tangent - flow).scatter_add(axis, safe.reshape(shape).expand_as(x), flow)
    return tangent - torch.where(root, edge_t * x, torch.zeros_like(x))


class _Tree(torch.autograd.Function):
    @staticmethod
    def forward(main, edge, rhs, parent, order, layers, threads, block):
        return _raw_tree(main, edge, rhs, parent, order, layers, block)

    @staticmethod
    def setup_context(ctx, inputs, output):
        main, edge, _, parent, order, layers, ctx.threads, ctx.block = inputs
        ctx.save_for_backward(main, edge, output, parent, order, layers)
        ctx.save_for_forward(main, edge, output, parent, order, layers)

    @staticmethod
    def backward(ctx, grad_x):
        main, edge, x, parent, order, layers = ctx.saved_tensors
        adj_main = main.transpose(-1, -2).contiguous() if ctx.block else main
        g = _Tree.apply(adj_main, edge, grad_x.contiguous(), parent, order, layers,
                        ctx.threads, ctx.block)
        grad_main = -(g.unsqueeze(-1) * x.unsqueeze(-2)) if ctx.block else -(g * x)
        return (grad_main, _tree_edge_gradient(x, g, parent, ctx.block), g,
                None, None, None, None, None)

    @staticmethod
    def jvp(ctx, main_t, edge_t, rhs_t, *_meta_t):
        main, edge, x, parent, order, layers = ctx.saved_tensors
        tangent = _tree_tangent(main_t, edge_t, rhs_t, x, parent, ctx.block)
        return _Tree.apply(main, edge, tangent.contiguous(), parent, order, layers,
                           ctx.threads, ctx.block)

    @staticmethod
    def vmap(info, in_dims, main, edge, rhs, parent, order, layers, threads, block):
        _require_shared(in_dims[3:])
        flat = _flatten(info, in_dims[:3], main, edge, rhs)
        return _restore(_Tree.apply(*flat, parent, order, layers, threads, block),
                        info.batch_size), 0


def dhs_solve(main, edge, rhs, parent, order, layers, *, threads):
    """Scalar tree solve (B, K): shunt ``main``, edge conductance ``edge``."""
    _tr.validate_tree(main, edge, rhs, parent, order, layers, threads)
    return _Tree.apply(main, edge, rhs, parent, order, layers, threads, False)


def dhs_bt_solve(main, edge, rhs, parent, order, layers, *, threads):
    """3x3 block tree solve: main (B, K, 3, 3), edge and rhs (B, K, 3)."""
    _tr.validate_tree_block(main, edge, rhs, parent, order, layers, threads)
    return _Tree.apply(main, edge, rhs, parent, order, layers, threads, True)


# ---------------------------------------------------------------------------
# row-padded multi-morphology trees
# ---------------------------------------------------------------------------
def _repeat_plan(plan, V, rows):
    """The plan for V stacked copies of a (rows, K_stride) plane."""
    if V == 1:
        return plan
    out = list(plan[:7])
    base, count = plan[7], plan[8]
    out.append(torch.cat([base + v * rows for v in range(V)]))
    out.append(count.repeat(V))
    out[3:7] = [t.repeat(V) for t in out[3:7]]
    return tuple(out)


class _Multi(torch.autograd.Function):
    """``mp`` is the device plan (tree._multi_plan) built from the caller's
    plain index tensors; it travels as a Python object, so transforms never
    wrap the topology."""

    @staticmethod
    def forward(main, edge, rhs, mp):
        return _tr._multi_solve(main, edge, rhs, mp)

    @staticmethod
    def setup_context(ctx, inputs, output):
        main, edge, _, ctx.mp = inputs
        ctx.save_for_backward(main, edge, output)
        ctx.save_for_forward(main, edge, output)

    @staticmethod
    def backward(ctx, grad_x):
        main, edge, x = ctx.saved_tensors
        mp = ctx.mp
        g = _Multi.apply(main, edge, grad_x.contiguous(), mp)
        xf, gf = x.reshape(-1), g.reshape(-1)
        par = mp.parent_flat.clamp_min(0)
        dx = torch.where(mp.has_parent, xf - xf.index_select(0, par), xf)
        dg = torch.where(mp.has_parent, gf - gf.index_select(0, par), gf)
        zero = torch.zeros_like(xf)
        grad_edge = torch.where(mp.node_mask, -(dg * dx), zero).view_as(x)
        grad_main = torch.where(mp.node_mask, -(gf * xf), zero).view_as(x)
        grad_rhs = torch.where(mp.node_mask, gf, zero).view_as(x)
        return grad_main, grad_edge, grad_rhs, None

    @staticmethod
    def jvp(ctx, main_t, edge_t, rhs_t, _mp_t):
        main, edge, x = ctx.saved_tensors
        mp = ctx.mp
        xf = x.reshape(-1)
        tangent = torch.zeros_like(xf) if rhs_t is None else rhs_t.reshape(-1)
        if main_t is not None:
            tangent = tangent - main_t.reshape(-1) * xf
        if edge_t is not None:
            et = edge_t.reshape(-1)
            par = mp.parent_flat.clamp_min(0)
            flow = torch.where(mp.has_parent, et * (xf - xf.index_select(0, par)),
                               torch.zeros_like(xf))
            tangent = (tangent - flow).index_add(0, par, flow)
            root = mp.node_mask & ~mp.has_parent
            tangent = tangent - torch.where(root, et * xf, torch.zeros_like(xf))
        tangent = torch.where(mp.node_mask, tangent, torch.zeros_like(tangent))
        return _Multi.apply(main, edge, tangent.view_as(x).contiguous(), mp)

    @staticmethod
    def vmap(info, in_dims, main, edge, rhs, mp):
        flat = _flatten(info, in_dims[:3], main, edge, rhs)
        V = info.batch_size
        rows = flat[2].shape[0] // V
        plan = _repeat_plan(mp.plan, V, rows)
        big = _tr._multi_plan(plan, V * rows, mp.K_stride, flat[2].device)
        return _restore(_Multi.apply(*flat, big), V), 0


def dhs_multi_solve(main, edge, rhs, *plan, K_stride, L_max, threads, grid_x):
    """Row-padded multi-morphology tree solve (the reference's 12-tensor
    launch plan; see tree.dhs_solve_multi_cuda)."""
    B, _ = _tr.validate_tree_multi(main, edge, rhs, plan, K_stride, L_max, threads, grid_x)
    return _Multi.apply(main, edge, rhs, _tr._multi_plan(tuple(plan), B, K_stride, rhs.device))
