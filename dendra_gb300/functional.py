"""Differentiable functional solvers on the GB300 kernels.

The reference's integrators call functional solvers with reverse, forward and
vmap rules (models/integrators/_cuda_functional.py: ``thomas_solve`` :594,
``pcr_solve`` :599, ``block_thomas_solve`` :604, ``block_spd_solve`` :609,
``dhs_solve`` :615, ``dhs_bt_solve`` :620, ``dhs_multi_solve`` :625; imported
by integrators/implicit.py:16-17 and mechanisms/_spatial.py:837-841, 1980).
The functions below keep those names, signatures and argument checks.

Every one of them is the same mathematical object, a batched linear system
``A(coef) x = rhs``, so a single ``torch.autograd.Function``
(``LinearSolve``) carries all the rules and each solver family contributes
only an *operator*: a plain Python object that knows

* ``solve(coef, rhs)``         -- the CUDA kernel for A x = rhs;
* ``adjoint(coef)``            -- the operator and coefficients of A^T (the
                                  transposed bands or blocks; trees are
                                  symmetric in their edges);
* ``cotangents(coef, x, y)``   -- dL/dcoef given x and y = A^-T dL/dx, i.e.
                                  the entries of -y x^T on A's sparsity pattern;
* ``action(coef, dcoef, x)``   -- (dA) x for coefficient tangents dcoef;
* ``again(coef)``              -- the operator and coefficients that solve the
                                  same system once more (a factored system
                                  reuses its factors);
* ``folded(V, rows)``          -- the operator for V stacked copies of the
                                  batch (vmap).

Reverse mode solves with the adjoint operator through ``LinearSolve`` itself,
forward mode solves ``A dx = drhs - (dA) x`` the same way, so derivatives of
any order compose.  Structure (topology, kernel choice, cached factors) lives
in the operator, never in a tensor argument, so transforms cannot map it.
There is no CPU path: every solve is one of the package's kernels.
"""

from __future__ import annotations

import torch
import torch.nn.functional as nnf

from . import _lib
from . import solvers as _sv
from . import tree as _tr


# ---------------------------------------------------------------------------
# the one autograd function
# ---------------------------------------------------------------------------
def _stack_batch(t, dim, V):
    """Move a vmapped dimension (or a broadcast copy) to the front and merge it
    into the solver's batch dimension."""
    t = t.unsqueeze(0).expand(V, *t.shape) if dim is None else t.movedim(dim, 0)
    return t.reshape(V * t.shape[1], *t.shape[2:]).contiguous()


class LinearSolve(torch.autograd.Function):
    """x = A(coef)^-1 rhs for an operator ``op`` (see the module docstring)."""

    @staticmethod
    def forward(op, rhs, *coef):
        return op.solve(coef, rhs)

    @staticmethod
    def setup_context(ctx, inputs, output):
        ctx.op = inputs[0]
        ctx.save_for_backward(output, *inputs[2:])
        ctx.save_for_forward(output, *inputs[2:])

    @staticmethod
    def backward(ctx, grad_x):
        x, *coef = ctx.saved_tensors
        op_t, coef_t = ctx.op.adjoint(coef)
        y = LinearSolve.apply(op_t, grad_x.contiguous(), *coef_t)
        return (None, y, *ctx.op.cotangents(coef, x, y))

    @staticmethod
    def jvp(ctx, _op_tangent, rhs_tangent, *coef_tangent):
        x, *coef = ctx.saved_tensors
        src = -ctx.op.action(coef, coef_tangent, x)
        if rhs_tangent is not None:
            src = src + rhs_tangent
        op, coef = ctx.op.again(coef)
        return LinearSolve.apply(op, src.contiguous(), *coef)

    @staticmethod
    def vmap(info, in_dims, op, rhs, *coef):
        V = info.batch_size
        flat = [_stack_batch(t, d, V) for t, d in zip((rhs, *coef), in_dims[1:])]
        rows = flat[0].shape[0] // V
        x = LinearSolve.apply(op.folded(V, rows), *flat)
        return x.reshape(V, rows, *x.shape[1:]), 0


def _no_mapped_structure(*tensors):
    """Topology and configuration must be shared by every mapped problem."""
    for t in tensors:
        if isinstance(t, torch.Tensor) and torch._C._functorch.is_batchedtensor(t):
            raise ValueError("solver topology and configuration must be shared under vmap")


def _outer(y, x, block):
    """y x^T restricted to the diagonal entries (scalar) or 3x3 blocks."""
    return y.unsqueeze(-1) * x.unsqueeze(-2) if block else y * x


def _apply_main(m, x, block):
    return (m @ x.unsqueeze(-1)).squeeze(-1) if block else m * x


# ---------------------------------------------------------------------------
# banded systems: scalar tridiagonal and 3x3 block tridiagonal
# ---------------------------------------------------------------------------
class _Banded:
    """Row k: lower[k-1] x[k-1] + main[k] x[k] + upper[k] x[k+1] = rhs[k].

    Scalar rows (B, K), or rows of three unknowns (B, K, 3) with full 3x3
    ``main`` blocks and diagonal coupling blocks given as 3-vectors.
    coef = (lower, main, upper)."""

    def __init__(self, block, method):
        self.block = block
        self.method = method
        self.axis = -2 if block else -1

    def solve(self, coef, rhs):
        lower, main, upper = coef
        if self.block:
            return _sv._block3(lower, main, upper, rhs, False)
        return _sv._solve(lower, main, upper, rhs, self.method)

    def adjoint(self, coef):
        lower, main, upper = coef
        main_t = main.transpose(-1, -2).contiguous() if self.block else main
        return self, (upper, main_t, lower)

    def _rows(self, t, start, count):
        return t.narrow(self.axis, start, count)

    def cotangents(self, coef, x, y):
        n = x.shape[self.axis]
        return (-(self._rows(y, 1, n - 1) * self._rows(x, 0, n - 1)),
                -_outer(y, x, self.block),
                -(self._rows(y, 0, n - 1) * self._rows(x, 1, n - 1)))

    def _pad_row(self, t, first):
        """t with one zero row added at the start (first) or the end."""
        widths = (1, 0) if first else (0, 1)
        return nnf.pad(t, ((0, 0) + widths) if self.block else widths)

    def action(self, coef, dcoef, x):
        d_lower, d_main, d_upper = dcoef
        n = x.shape[self.axis]
        out = torch.zeros_like(x) if d_main is None else _apply_main(d_main, x, self.block)
        if d_lower is not None:
            out = out + self._pad_row(d_lower * self._rows(x, 0, n - 1), first=True)
        if d_upper is not None:
            out = out + self._pad_row(d_upper * self._rows(x, 1, n - 1), first=False)
        return out

    def again(self, coef):
        return self, tuple(coef)

    def folded(self, V, rows):
        return self


class _SymmetricBlocks(_Banded):
    """Symmetric positive definite 3x3 block system (the reference's SPD
    method): main blocks are symmetrised and factored by the kernel, lower ==
    upper.  The factors of the last solve are kept on the operator; the
    adjoint (A is symmetric) and every tangent solve reuse them."""

    def __init__(self):
        super().__init__(block=True, method=None)
        self.factors = None

    def solve(self, coef, rhs):
        lower, main, upper = coef
        x, self.factors = _sv._block3_spd(lower, main, upper, rhs)
        self.bands = (lower, upper)
        return x

    def adjoint(self, coef):
        return _FactoredBlocks(*self.bands, self.factors), ()

    def again(self, coef):
        return self.adjoint(coef)

    def cotangents(self, coef, x, y):
        lower, main, upper = super().cotangents(coef, x, y)
        return lower, _sv._symmetric_part(main), upper

    def action(self, coef, dcoef, x):
        d_lower, d_main, d_upper = dcoef
        d_main = None if d_main is None else _sv._symmetric_part(d_main)
        return super().action(coef, (d_lower, d_main, d_upper), x)

    def folded(self, V, rows):
        return _SymmetricBlocks()


class _FactoredBlocks:
    """A solve with the saved SPD factors (the reference's block_spd_chol,
    _cuda_functional.py:101-123): linear and symmetric in rhs, no
    differentiable coefficients."""

    def __init__(self, lower, upper, factors):
        self.lower, self.upper, self.factors = lower, upper, factors

    def solve(self, coef, rhs):
        return _sv._block3_spd_with_chol(self.lower, self.upper, self.factors, rhs)

    def adjoint(self, coef):
        return self, ()

    def cotangents(self, coef, x, y):
        return ()

    def action(self, coef, dcoef, x):
        return torch.zeros_like(x)

    def again(self, coef):
        return self, ()

    def folded(self, V, rows):
        def rep(t):
            return t.unsqueeze(0).expand(V, *t.shape).reshape(V * t.shape[0], *t.shape[1:])
        return _FactoredBlocks(rep(self.lower), rep(self.upper), rep(self.factors).contiguous())


def thomas_solve(a, b, c, rhs):
    """Batched scalar Thomas solve, (B, K-1) bands, (B, K) main and rhs."""
    _sv.validate_tridiagonal(a, b, c, rhs)
    return LinearSolve.apply(_Banded(False, _lib.THOMAS), rhs, a, b, c)


def pcr_solve(a, b, c, rhs):
    """Batched scalar PCR solve (same system as thomas_solve)."""
    _sv.validate_tridiagonal(a, b, c, rhs)
    return LinearSolve.apply(_Banded(False, _lib.PCR), rhs, a, b, c)


def block_thomas_solve(lower, main, upper, rhs):
    """3x3 block-tridiagonal solve: lower/upper (B, K-1, 3) diagonal blocks,
    main (B, K, 3, 3), rhs (B, K, 3)."""
    _sv.validate_block_tridiagonal(lower, main, upper, rhs)
    return LinearSolve.apply(_Banded(True, None), rhs, lower, main, upper)


def block_spd_solve(lower, main, upper, rhs):
    """SPD 3x3 block solve (blocks symmetrised, shifted when not positive
    definite); the reverse and forward rules reuse the cached factors."""
    _sv.validate_block_tridiagonal(lower, main, upper, rhs)
    return LinearSolve.apply(_SymmetricBlocks(), rhs, lower, main, upper)


# ---------------------------------------------------------------------------
# trees (one shared topology) and row-padded forests of morphologies
# ---------------------------------------------------------------------------
class _Tree:
    """Hines system of a tree in conductance form: every node i has a shunt
    main[i] and an edge conductance edge[i] to parent[i] (a root's edge is a
    second shunt).  A = diag(main) + sum over edges of edge_i (e_i - e_p)
    (e_i - e_p)^T, symmetric; with 3x3 blocks main is a full block and edges
    are diagonal blocks.  coef = (main, edge)."""

    def __init__(self, parent, order, layers, threads, block):
        self.topo = (parent, order, layers)
        self.threads = threads
        self.block = block
        self.axis = -2 if block else -1
        up = parent.clamp_min(0).long()
        self.up = up
        self.is_root = (parent < 0).reshape((1, -1, 1) if block else (1, -1))
        self.scatter_index = up.reshape((1, -1, 1) if block else (1, -1))

    def solve(self, coef, rhs):
        main, edge = coef
        parent, order, layers = self.topo
        if self.block:
            return _tr._block_solve(main, edge, rhs,
                                    _tr._checked_topology(parent, order, layers), False)
        return _tr._solve(main, edge, rhs, _tr._device_topology(parent, order, layers))

    def adjoint(self, coef):
        main, edge = coef
        return self, ((main.transpose(-1, -2).contiguous() if self.block else main), edge)

    def _across_edge(self, v):
        """v[i] - v[parent(i)] on every edge, v[i] at roots."""
        return torch.where(self.is_root, v, v - v.index_select(self.axis, self.up))

    def cotangents(self, coef, x, y):
        return -_outer(y, x, self.block), -(self._across_edge(y) * self._across_edge(x))

    def action(self, coef, dcoef, x):
        d_main, d_edge = dcoef
        out = torch.zeros_like(x) if d_main is None else _apply_main(d_main, x, self.block)
        if d_edge is None:
            return out
        current = d_edge * self._across_edge(x)  # leaves node i, enters its parent
        into_parent = torch.where(self.is_root, torch.zeros_like(current), current)
        out = out + current
        return out.scatter_add(self.axis, self.scatter_index.expand_as(x), -into_parent)

    def again(self, coef):
        return self, tuple(coef)

    def folded(self, V, rows):
        return self


class _Forest:
    """Row-padded planes (rows, K_stride) holding trees of several
    morphologies (the reference's multi-DHS layout); coef = (main, edge).
    Entries outside a tree are ignored on input and zero on output."""

    def __init__(self, plan_tensors, B, K_stride, device):
        self.plan = tuple(plan_tensors)
        self.K_stride = K_stride
        self.mp = _tr._multi_plan(self.plan, B, K_stride, device)

    def solve(self, coef, rhs):
        main, edge = coef
        return _tr._multi_solve(main, edge, rhs, self.mp)

    def adjoint(self, coef):
        return self, tuple(coef)

    def _flat_across_edge(self, v):
        up = self.mp.parent_flat.clamp_min(0)
        return torch.where(self.mp.has_parent, v - v.index_select(0, up), v)

    def cotangents(self, coef, x, y):
        xf, yf = x.reshape(-1), y.reshape(-1)
        keep = self.mp.node_mask
        zero = torch.zeros_like(xf)
        d_main = torch.where(keep, -(yf * xf), zero)
        d_edge = torch.where(keep, -(self._flat_across_edge(yf) * self._flat_across_edge(xf)),
                             zero)
        return d_main.view_as(x), d_edge.view_as(x)

    def action(self, coef, dcoef, x):
        d_main, d_edge = dcoef
        xf = x.reshape(-1)
        out = torch.zeros_like(xf) if d_main is None else d_main.reshape(-1) * xf
        if d_edge is not None:
            current = d_edge.reshape(-1) * self._flat_across_edge(xf)
            keep = self.mp.node_mask
            out = out + torch.where(keep, current, torch.zeros_like(current))
            into_parent = torch.where(self.mp.has_parent, current, torch.zeros_like(current))
            out = out.index_add(0, self.mp.parent_flat.clamp_min(0), -into_parent)
        return torch.where(self.mp.node_mask, out, torch.zeros_like(out)).view_as(x)

    def again(self, coef):
        return self, tuple(coef)

    def folded(self, V, rows):
        if V == 1:
            return self
        # V stacked copies of the planes: the same trees, their rows offset
        plan = list(self.plan[:7])
        base, count = self.plan[7], self.plan[8]
        plan[3:7] = [t.repeat(V) for t in plan[3:7]]
        plan.append(torch.cat([base + v * rows for v in range(V)]))
        plan.append(count.repeat(V))
        return _Forest(plan, V * rows, self.K_stride, base.device)


def dhs_solve(main, edge, rhs, parent, order, layers, *, threads):
    """Scalar tree solve (B, K): shunt ``main``, edge conductance ``edge``."""
    _tr.validate_tree(main, edge, rhs, parent, order, layers, threads)
    _no_mapped_structure(parent, order, layers)
    return LinearSolve.apply(_Tree(parent, order, layers, threads, False), rhs, main, edge)


def dhs_bt_solve(main, edge, rhs, parent, order, layers, *, threads):
    """3x3 block tree solve: main (B, K, 3, 3), edge and rhs (B, K, 3)."""
    _tr.validate_tree_block(main, edge, rhs, parent, order, layers, threads)
    _no_mapped_structure(parent, order, layers)
    return LinearSolve.apply(_Tree(parent, order, layers, threads, True), rhs, main, edge)


def dhs_multi_solve(main, edge, rhs, *plan, K_stride, L_max, threads, grid_x):
    """Row-padded multi-morphology tree solve (the reference's 12-tensor
    launch plan; see tree.dhs_solve_multi_cuda)."""
    B, _ = _tr.validate_tree_multi(main, edge, rhs, plan, K_stride, L_max, threads, grid_x)
    _no_mapped_structure(*plan)
    return LinearSolve.apply(_Forest(plan, B, K_stride, rhs.device), rhs, main, edge)
