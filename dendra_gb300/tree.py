"""Tree (DHS/Hines) solves on the GB300 kernels.

Host-side topology planning restates the reference's helpers:

* :func:`build_morphology`  — integrators/tree.py:414-474 (parent, children, BFS depth)
* :func:`build_dhs_layers`  — integrators/tree.py:615-673 (depth buckets deepest
  first, chunked by ``threads``)

and adds the children CSR the deterministic kernel pulls from.  Solves:

* :func:`dhs_solve_cuda` — reference signature (triton/dhs_kernel.py:634-651),
  B trees sharing one topology, with the reference's gradients
  (DHSSolvePacked.backward, dhs_kernel.py:546-598: the system is symmetric, so
  the adjoint is the same solve).
* :class:`ForestPlan` / :func:`dhs_solve_forest` — trees of different
  topologies packed into one launch (the role of dhs_solve_multi_cuda,
  triton/dhs_kernel_multi.py:831-888).
* :func:`build_chains` — the chain schedule of the same elimination (one lane
  per unbranched chain, one synchronisation per chain level instead of per
  depth layer), the role the reference gives its tree-contraction solver for
  deep trees (triton/tree_contraction.py, segment condensation).
"""

from __future__ import annotations

import ctypes
from collections import deque

import numpy as np
import torch

from . import _lib
from ._cache import TensorKeyedCache
from .solvers import _validate_float_group

_INDEX_DTYPES = (torch.int32, torch.int64)


def build_morphology(parent_idx):
    """Return (parent int32[K], children lists, depth int32[K]) of a rooted tree."""
    K = len(parent_idx)
    if K == 0:
        raise ValueError("parent_idx must contain at least one node")
    roots = [i for i, p in enumerate(parent_idx) if p == -1]
    if len(roots) != 1:
        raise ValueError(f"parent_idx must contain exactly one root; found {len(roots)}")
    children = [[] for _ in range(K)]
    for i, p in enumerate(parent_idx):
        if p == -1:
            continue
        if isinstance(p, bool) or not isinstance(p, (int, np.integer)):
            raise TypeError(f"parent index at node {i} must be an integer; got {p!r}")
        if p < 0 or p >= K:
            raise ValueError(f"parent index at node {i} must be in [0, {K - 1}]; got {p}")
        if p == i:
            raise ValueError(f"node {i} cannot be its own parent")
        children[p].append(i)
    depth = np.zeros(K, dtype=np.int32)
    q = deque([roots[0]])
    visited = set()
    while q:
        u = q.popleft()
        if u in visited:
            raise ValueError("parent_idx contains a cycle")
        visited.add(u)
        for c in children[u]:
            depth[c] = depth[u] + 1
            q.append(c)
    if len(visited) != K:
        raise ValueError("parent_idx contains a cycle or nodes unreachable from the root")
    return torch.as_tensor(np.asarray(parent_idx, dtype=np.int32)), children, torch.as_tensor(depth)


def validate_threads(threads):
    if isinstance(threads, bool) or not isinstance(threads, int):
        raise TypeError("threads must be a positive integer that divides 32")
    if threads <= 0 or threads > 32:
        raise ValueError("threads must be in [1, 32]")
    if 32 % threads != 0:
        raise ValueError("threads must divide 32 (warp size)")
    return threads


def build_dhs_layers(depth, k_threads):
    """Elimination order (deepest depth first) and layer boundaries (chunks <= k_threads)."""
    k_threads = validate_threads(k_threads)
    depth = np.asarray(torch.as_tensor(depth).cpu().numpy())
    if depth.ndim != 1 or depth.size == 0:
        raise ValueError("depth must be a non-empty one-dimensional integer tensor")
    if (depth < 0).any():
        raise ValueError("depth values must be nonnegative")
    bins = [[] for _ in range(int(depth.max()) + 1)]
    for i, d in enumerate(depth):
        bins[int(d)].append(i)
    order, layer_ptr = [], [0]
    for d in range(len(bins) - 1, -1, -1):
        bucket = bins[d]
        for s in range(0, len(bucket), k_threads):
            order.extend(bucket[s:s + k_threads])
            layer_ptr.append(len(order))
    return (torch.as_tensor(order, dtype=torch.int32),
            torch.as_tensor(layer_ptr, dtype=torch.int32))


def children_csr(parent):
    """Children of every node, increasing index order: (child_ptr[K+1], child_idx[max(K-1,1)])."""
    parent = np.asarray(parent, dtype=np.int64)
    K = parent.size
    nonroot = np.nonzero(parent >= 0)[0]
    counts = np.bincount(parent[nonroot], minlength=K)
    ptr = np.zeros(K + 1, dtype=np.int32)
    ptr[1:] = np.cumsum(counts)
    idx = nonroot[np.argsort(parent[nonroot], kind="stable")].astype(np.int32)
    if idx.size == 0:
        idx = np.zeros(1, dtype=np.int32)
    return ptr, idx


def validate_tree(d_mem, a_geom, b, parent_idx, order, layer_ptr, threads):
    """Shape/dtype/device contract of the scalar tree solve (triton/_contracts.py:199-229)."""
    data = (("d_mem", d_mem), ("a_geom", a_geom), ("b", b))
    topo = (("parent_idx", parent_idx), ("order", order), ("layer_ptr", layer_ptr))
    for name, t in data + topo:
        if not isinstance(t, torch.Tensor):
            raise TypeError(f"{name} must be a torch.Tensor")
    if d_mem.ndim != 2:
        raise ValueError(f"d_mem must have shape (B, K), got {tuple(d_mem.shape)}")
    batch, size = map(int, d_mem.shape)
    if batch < 1 or size < 1:
        raise ValueError("B and K must both be >= 1")
    if tuple(a_geom.shape) != (batch, size) or tuple(b.shape) != (batch, size):
        raise ValueError("d_mem, a_geom, and b must have identical (B, K) shapes")
    _validate_float_group(data)
    for name, t in topo:
        if t.ndim != 1:
            raise ValueError(f"{name} must be 1-D")
        if t.dtype not in _INDEX_DTYPES:
            raise TypeError(f"{name} must have dtype int32 or int64")
        if t.device != d_mem.device:
            raise ValueError(f"{name} must be on device {d_mem.device}; got {t.device}")
    if parent_idx.numel() != size or order.numel() != size:
        raise ValueError("parent_idx and order must each contain K entries")
    if layer_ptr.numel() < 2:
        raise ValueError("layer_ptr must contain at least two entries")
    return batch, size, validate_threads(threads)


_topo_cache = TensorKeyedCache(64)


def _device_topology(parent_idx, order, layer_ptr):
    """int32 device copies of the plan plus the children CSR, cached on the
    identity and version of the three plan tensors (the entry holds them)."""

    def build():
        dev = parent_idx.device
        parent_np = parent_idx.detach().cpu().numpy().astype(np.int64)
        cptr, cidx = children_csr(parent_np)
        return tuple(torch.as_tensor(x, dtype=torch.int32, device=dev).contiguous() for x in (
            parent_np, order.detach().cpu().numpy(), layer_ptr.detach().cpu().numpy(),
            cptr, cidx))

    return _topo_cache.get((parent_idx, order, layer_ptr), None, build)


_chain_cache: dict = {}


def _chain_forest(topo, B):
    """Chain-schedule forest of B copies of ``topo``'s tree (cached): the
    elimination runs one lane per unbranched chain with a sync per chain
    level, the same per-node operations as the depth-layer schedule."""
    key = (id(topo), B)
    hit = _chain_cache.get(key)
    if hit is None or hit[0] is not topo:
        if len(_chain_cache) > 64:
            _chain_cache.clear()
        parent = [int(p) for p in topo[0].detach().cpu().numpy()]
        plan = ForestPlan([parent], device=topo[0].device, plan_of=np.zeros(B, dtype=np.int32),
                          chains=True)
        hit = _chain_cache[key] = (topo, plan)
    return hit[1]


def _solve(d, a, b, topo):
    B, K = d.shape
    d, a, b = (t.contiguous() for t in (d, a, b))
    x = torch.empty_like(b)
    f = _chain_forest(topo, B).struct()
    with torch.cuda.device(d.device):
        rc = _lib.load().dgb_dhs_solve_forest(_lib.dtype_code(d.dtype), ctypes.byref(f),
                                              d.data_ptr(), a.data_ptr(), b.data_ptr(),
                                              x.data_ptr(), _lib.stream_ptr(d.device))
    _lib.check(rc, "dgb_dhs_solve_forest")
    return x


class _DHSSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, d_mem, a_geom, b, topo):
        x = _solve(d_mem, a_geom, b, topo)
        ctx.topo = topo
        ctx.save_for_backward(d_mem, a_geom, x)
        return x

    @staticmethod
    def backward(ctx, grad_out):
        d_mem, a_geom, V = ctx.saved_tensors
        g = _solve(d_mem, a_geom, grad_out.contiguous(), ctx.topo)  # symmetric system
        parent_idx = ctx.topo[0].long()
        parent = parent_idx.clamp_min(0)
        Vp = V.index_select(1, parent)
        gp = g.index_select(1, parent)
        root = (parent_idx < 0).view(1, -1)
        grad_a = torch.where(root, -(g * V), -((g - gp) * (V - Vp)))
        return -(g * V), grad_a, g, None


def dhs_solve_cuda(d_mem, a_geom, b, parent_idx, order, layer_ptr, threads=32):
    """Batched tree solve, drop-in for the reference's dhs_solve_cuda.

    All (B, K) tensors are in the solver order that ``order``/``layer_ptr``
    index; ``threads`` is validated like the reference (it sets the layer
    chunking there).  One warp per tree runs the chain schedule of the same
    elimination (one lane per unbranched chain), which gives the depth-layer
    schedule's results bit for bit.
    """
    validate_tree(d_mem, a_geom, b, parent_idx, order, layer_ptr, threads)
    topo = _device_topology(parent_idx, order, layer_ptr)
    return _DHSSolve.apply(d_mem, a_geom, b, topo)


def validate_tree_block(main, edge, rhs, parent_idx, order, layer_ptr, threads):
    """Contract of the 3x3 block tree solve (triton/_contracts.py:232-268)."""
    data = (("main", main), ("edge", edge), ("rhs", rhs))
    topo = (("parent_idx", parent_idx), ("order", order), ("layer_ptr", layer_ptr))
    for name, t in data + topo:
        if not isinstance(t, torch.Tensor):
            raise TypeError(f"{name} must be a torch.Tensor")
    if rhs.ndim != 3 or rhs.shape[-1] != 3:
        raise ValueError(f"rhs must have shape (B, K, 3), got {tuple(rhs.shape)}")
    batch, size, _ = map(int, rhs.shape)
    if batch < 1 or size < 1:
        raise ValueError("B and K must both be >= 1")
    if tuple(edge.shape) != (batch, size, 3):
        raise ValueError(f"edge must have shape {(batch, size, 3)}, got {tuple(edge.shape)}")
    if tuple(main.shape) != (batch, size, 3, 3):
        raise ValueError(
            f"main must have shape {(batch, size, 3, 3)}, got {tuple(main.shape)}")
    _validate_float_group(data)
    for name, t in topo:
        if t.ndim != 1:
            raise ValueError(f"{name} must be 1-D")
        if t.dtype not in _INDEX_DTYPES:
            raise TypeError(f"{name} must have dtype int32 or int64")
        if t.device != rhs.device:
            raise ValueError(f"{name} must be on device {rhs.device}; got {t.device}")
    if parent_idx.numel() != size or order.numel() != size:
        raise ValueError("parent_idx and order must each contain K entries")
    if layer_ptr.numel() < 2:
        raise ValueError("layer_ptr must contain at least two entries")
    return batch, size, validate_threads(threads)


def _checked_topology(parent_idx, order, layer_ptr):
    """Device plan with the children CSR, after checking it indexes K nodes:
    parents in [-1, K), order a permutation, layer_ptr from 0 to K, nondecreasing."""
    K = parent_idx.numel()
    p = parent_idx.detach().cpu().numpy().astype(np.int64)
    o = order.detach().cpu().numpy().astype(np.int64)
    lp = layer_ptr.detach().cpu().numpy().astype(np.int64)
    if (p < -1).any() or (p >= K).any():
        raise ValueError("parent_idx entries must lie in [-1, K)")
    if not np.array_equal(np.sort(o), np.arange(K)):
        raise ValueError("order must be a permutation of range(K)")
    if lp[0] != 0 or lp[-1] != K or (np.diff(lp) < 0).any():
        raise ValueError("layer_ptr must rise from 0 to K")
    return _device_topology(parent_idx, order, layer_ptr)


def _block_solve(main, edge, rhs, topo, transpose):
    parent, order, layer_ptr, cptr, cidx = topo
    B, K = rhs.shape[:2]
    main, edge, rhs = (t.contiguous() for t in (main, edge, rhs))
    x = torch.empty_like(rhs)
    with torch.cuda.device(rhs.device):
        rc = _lib.load().dgb_dhs_block3_solve(
            _lib.dtype_code(rhs.dtype), B, K, main.data_ptr(), edge.data_ptr(), rhs.data_ptr(),
            parent.data_ptr(), order.data_ptr(), layer_ptr.data_ptr(), layer_ptr.numel() - 1,
            cptr.data_ptr(), cidx.data_ptr(), x.data_ptr(), 1 if transpose else 0,
            _lib.stream_ptr(rhs.device))
    _lib.check(rc, "dgb_dhs_block3_solve")
    return x


class _DHSBTSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, main, edge, rhs, topo):
        x = _block_solve(main, edge, rhs, topo, False)
        ctx.topo = topo
        ctx.save_for_backward(main, edge, x)
        return x

    @staticmethod
    def backward(ctx, grad_out):
        main, edge, X = ctx.saved_tensors
        g = _block_solve(main, edge, grad_out.contiguous(), ctx.topo, True)  # A^T
        parent_idx = ctx.topo[0].long()
        parent = parent_idx.clamp_min(0)
        Xp = X.index_select(1, parent)
        gp = g.index_select(1, parent)
        root = (parent_idx < 0).view(1, -1, 1)
        grad_edge = torch.where(root, -(g * X), -((g - gp) * (X - Xp)))
        grad_main = -(g.unsqueeze(-1) * X.unsqueeze(-2))
        return grad_main, grad_edge, g, None


def dhs_bt_solve_cuda(D_blocks, G_vec, b, parent_idx, order, layer_ptr, threads=16):
    """Tree solve for 3-component unknowns (v_i, ve0, ve1) per node, drop-in for
    the reference's dhs_bt_solve_cuda (triton/dhs_kernel_bt.py:465-479): D_blocks
    (B, K, 3, 3), G_vec (B, K, 3) edge conductances to the parent, b (B, K, 3),
    all in solver order.  Differentiable in D_blocks, G_vec and b (the
    reference's DHSBTSolve3.backward formulas; the adjoint is the transposed
    block solve).  ``threads`` is validated like the reference's."""
    validate_tree_block(D_blocks, G_vec, b, parent_idx, order, layer_ptr, threads)
    topo = _checked_topology(parent_idx, order, layer_ptr)
    return _DHSBTSolve.apply(D_blocks, G_vec, b, topo)


def build_chains(parent):
    """Chain schedule of a tree: unbranched chains grouped by level.

    A chain starts at the root or at a child of a branch node and runs down
    through single-child nodes to a leaf or a branch node.  Returns
    ``chain_nodes`` (K, int32: chains one after another, each listed from its
    bottom node to its top), ``chain_ptr`` (n_chains + 1) and ``chain_level``
    (n_levels + 1, offsets into the chains): level 0 holds the chains that end
    in a leaf, level l the chains whose bottom's child chains all lie below l.
    Within a level chains are sorted longest first (lanes take them in turn).
    The elimination may then run level by level, one lane per chain, and the
    back substitution in the reverse order (csrc/dhs.cuh chain_eliminate)."""
    parent = [int(v) for v in parent]
    K = len(parent)
    children = [[] for _ in range(K)]
    root = -1
    for i, pp in enumerate(parent):
        if pp < 0:
            root = i
        else:
            children[pp].append(i)
    chains, bottom_children = [], []
    stack = [root]
    while stack:
        top = stack.pop()
        nodes = [top]
        i = top
        while len(children[i]) == 1:
            i = children[i][0]
            nodes.append(i)
        chains.append(nodes)
        bottom_children.append(children[i])
        stack.extend(children[i])
    chain_of = np.empty(K, dtype=np.int64)
    for c, nodes in enumerate(chains):
        chain_of[nodes] = c
    level = np.zeros(len(chains), dtype=np.int64)
    for c in range(len(chains) - 1, -1, -1):  # child chains were created after their parent
        kids = bottom_children[c]
        if kids:
            level[c] = 1 + max(level[chain_of[k]] for k in kids)
    order = sorted(range(len(chains)), key=lambda c: (level[c], -len(chains[c]), c))
    chain_nodes = np.concatenate([np.asarray(chains[c][::-1], dtype=np.int32) for c in order])
    chain_ptr = np.zeros(len(chains) + 1, dtype=np.int32)
    chain_ptr[1:] = np.cumsum([len(chains[c]) for c in order])
    n_levels = int(level.max()) + 1 if len(chains) else 0
    counts = np.bincount(level, minlength=n_levels)
    chain_level = np.zeros(n_levels + 1, dtype=np.int32)
    chain_level[1:] = np.cumsum(counts)
    return chain_nodes, chain_ptr, chain_level


class DgbForest(ctypes.Structure):
    _fields_ = [
        ("n_trees", ctypes.c_int32), ("max_k", ctypes.c_int32),
        ("node_ptr", ctypes.c_void_p), ("plan_of", ctypes.c_void_p),
        ("plan_node_ptr", ctypes.c_void_p), ("plan_layer_off", ctypes.c_void_p),
        ("parent", ctypes.c_void_p), ("order", ctypes.c_void_p), ("layer_ptr", ctypes.c_void_p),
        ("child_ptr", ctypes.c_void_p), ("child_idx", ctypes.c_void_p),
        ("plan_chain_off", ctypes.c_void_p), ("plan_clevel_off", ctypes.c_void_p),
        ("chain_nodes", ctypes.c_void_p), ("chain_ptr", ctypes.c_void_p),
        ("chain_level", ctypes.c_void_p), ("tree_k", ctypes.c_void_p),
    ]


class ForestPlan:
    """Packed plans of many trees (one topology plan per distinct tree).

    ``parents``: list of parent arrays (local indices, -1 at the root), one per
    tree; trees may share a plan by passing ``plan_of``.
    """

    def __init__(self, parents, device="cuda", threads=32, plan_of=None, chains=True):
        self.n_plans = len(parents)
        node_counts = [len(p) for p in parents]
        plan_node_ptr = np.zeros(self.n_plans + 1, dtype=np.int64)
        plan_node_ptr[1:] = np.cumsum(node_counts)
        par, orders, layers, cptrs, cidxs, layer_off = [], [], [], [], [], [0]
        cnodes, cptrs_c, clevels, chain_off, clevel_off = [], [], [], [0], [0]
        for p in parents:
            if chains:
                cn, cp, cl = build_chains(p)
                cnodes.append(cn)
                cptrs_c.append(cp)
                clevels.append(cl)
                chain_off.append(chain_off[-1] + cp.size)
                clevel_off.append(clevel_off[-1] + cl.size)
            p = [int(v) for v in p]
            _, _, depth = build_morphology(p)
            order, layer_ptr = build_dhs_layers(depth, threads)
            cptr, cidx = children_csr(p)
            par.append(np.asarray(p, dtype=np.int32))
            orders.append(order.numpy())
            layers.append(layer_ptr.numpy())
            layer_off.append(layer_off[-1] + layer_ptr.numel())
            cptrs.append(cptr)
            # K_p entries per plan (K_p - 1 children + one unused) so that plan
            # p's block starts at plan_node_ptr[p], like parent and order
            cidxs.append(np.concatenate([cidx[: max(len(p) - 1, 0)],
                                         np.zeros(1, dtype=np.int32)]))
        if plan_of is None:
            plan_of_np = np.arange(self.n_plans, dtype=np.int32)
        else:
            plan_of_np = np.asarray(plan_of, dtype=np.int32)
        tree_k = np.asarray(node_counts, dtype=np.int64)[plan_of_np]
        node_ptr = np.zeros(plan_of_np.size + 1, dtype=np.int64)
        node_ptr[1:] = np.cumsum(tree_k)
        dev = torch.device(device)

        def t(x, dt):
            return torch.as_tensor(np.concatenate(x) if isinstance(x, list) else x,
                                   dtype=dt, device=dev).contiguous()

        cidx_all = np.concatenate(cidxs)
        assert cidx_all.size == plan_node_ptr[-1]
        self.tensors = dict(
            node_ptr=t(node_ptr, torch.int64), plan_of=t(plan_of_np, torch.int32),
            plan_node_ptr=t(plan_node_ptr, torch.int64),
            plan_layer_off=t(np.asarray(layer_off, dtype=np.int64), torch.int64),
            parent=t(par, torch.int32), order=t(orders, torch.int32),
            layer_ptr=t(layers, torch.int32), child_ptr=t(cptrs, torch.int32),
            child_idx=torch.as_tensor(cidx_all, dtype=torch.int32, device=dev).contiguous(),
        )
        if chains:
            self.tensors.update(
                plan_chain_off=t(np.asarray(chain_off, dtype=np.int64), torch.int64),
                plan_clevel_off=t(np.asarray(clevel_off, dtype=np.int64), torch.int64),
                chain_nodes=t(cnodes, torch.int32), chain_ptr=t(cptrs_c, torch.int32),
                chain_level=t(clevels, torch.int32))
        self.n_trees = int(plan_of_np.size)
        self.n_nodes = int(node_ptr[-1])
        self.max_k = int(tree_k.max()) if tree_k.size else 1
        self.node_ptr = node_ptr
        self.device = dev

    def struct(self):
        f = DgbForest()
        f.n_trees = self.n_trees
        f.max_k = self.max_k
        for k, v in self.tensors.items():
            setattr(f, k, v.data_ptr())
        return f


def dhs_solve_forest(d, a, b, plan: ForestPlan):
    """Solve packed heterogeneous trees: d, a, b are (n_nodes,) packed by tree."""
    if not (d.shape == a.shape == b.shape == (plan.n_nodes,)):
        raise ValueError(f"d, a, b must have shape ({plan.n_nodes},)")
    _validate_float_group((("d", d), ("a", a), ("b", b)))
    d, a, b = (t.contiguous() for t in (d, a, b))
    x = torch.empty_like(b)
    f = plan.struct()
    with torch.cuda.device(d.device):
        rc = _lib.load().dgb_dhs_solve_forest(_lib.dtype_code(d.dtype), ctypes.byref(f),
                                              d.data_ptr(), a.data_ptr(), b.data_ptr(),
                                              x.data_ptr(), _lib.stream_ptr(d.device))
    _lib.check(rc, "dgb_dhs_solve_forest")
    return x


_MULTI_PLAN = ("P_cat", "ORDER_cat", "LAYER_PTR_cat", "WARP_P_OFF", "WARP_ORDER_OFF",
               "WARP_LPTR_OFF", "WARP_L", "WARP_ROW_BASE", "WARP_ROW_COUNT")


def validate_tree_multi(d_mem, a_geom, b, plan, K_stride, L_max, threads, grid_x):
    """The reference's checks of the row-padded multi-morphology launch
    (triton/_contracts.py:271-341); ``plan`` is the nine index tensors in
    signature order."""
    data = (("d_mem", d_mem), ("a_geom", a_geom), ("b", b))
    named = tuple(zip(_MULTI_PLAN, plan))
    for name, t in data + named:
        if not isinstance(t, torch.Tensor):
            raise TypeError(f"{name} must be a torch.Tensor")
    if d_mem.ndim != 2:
        raise ValueError(f"d_mem must have shape (B, K_stride), got {tuple(d_mem.shape)}")
    if a_geom.shape != d_mem.shape or b.shape != d_mem.shape:
        raise ValueError("d_mem, a_geom, and b must have identical shapes")
    batch, width = map(int, d_mem.shape)
    if batch < 1 or width < 1:
        raise ValueError("B and K_stride must both be >= 1")
    if isinstance(K_stride, bool) or not isinstance(K_stride, int):
        raise TypeError("K_stride must be an integer")
    if K_stride != width:
        raise ValueError(f"K_stride must equal the padded row width {width}")
    if isinstance(L_max, bool) or not isinstance(L_max, int):
        raise TypeError("L_max must be an integer")
    if L_max < 1:
        raise ValueError("L_max must be >= 1")
    _validate_float_group(data)
    for name, t in named:
        if t.ndim != 1:
            raise ValueError(f"{name} must be 1-D")
        if t.dtype not in _INDEX_DTYPES:
            raise TypeError(f"{name} must have dtype int32 or int64")
        if t.device != d_mem.device:
            raise ValueError(f"{name} must be on device {d_mem.device}; got {t.device}")
    p_cat, order_cat, lptr_cat = plan[:3]
    if p_cat.numel() != order_cat.numel() or p_cat.numel() < 1:
        raise ValueError("P_cat and ORDER_cat must have the same non-zero length")
    if lptr_cat.numel() < 2:
        raise ValueError("LAYER_PTR_cat must contain at least two entries")
    warp_count = int(plan[7].numel())
    if warp_count < 1:
        raise ValueError("the launch plan must contain at least one warp")
    for name, t in named[3:]:
        if t.numel() != warp_count:
            raise ValueError(f"{name} must contain one entry per warp ({warp_count})")
    if grid_x is not None:
        if isinstance(grid_x, bool) or not isinstance(grid_x, int):
            raise TypeError("grid_x must be an integer or None")
        if grid_x != warp_count:
            raise ValueError(f"grid_x must equal the plan warp count {warp_count}")
    validate_threads(threads)
    return batch, warp_count


_multi_cache = TensorKeyedCache(32)


class _MultiPlan:
    """Device form of a row-padded multi-morphology plan: a forest over the
    covered rows (tree t = one row, its K_t nodes at row * K_stride) and the
    flat parent index of every plane entry for the gradient."""

    def __init__(self, plan, B, K_stride, device):
        self.plan, self.K_stride = tuple(plan), int(K_stride)
        p_cat, _, lptr_cat, p_off, _, l_off, n_l, row_base, row_count = (
            t.detach().cpu().numpy().astype(np.int64) for t in plan)
        morphs, parents, tree_rows, tree_morph = {}, [], [], []
        covered = np.zeros(B, dtype=bool)
        for w in range(row_base.size):
            if n_l[w] < 1 or l_off[w] < 0 or l_off[w] + n_l[w] >= lptr_cat.size:
                raise ValueError(f"warp {w}: layer table out of range")
            k = int(lptr_cat[l_off[w] + n_l[w]])  # the last layer ends at K_g
            if k < 1 or k > K_stride or p_off[w] < 0 or p_off[w] + k > p_cat.size:
                raise ValueError(f"warp {w}: morphology of {k} nodes does not fit")
            key = (int(p_off[w]), k)
            if key not in morphs:
                morphs[key] = len(parents)
                parents.append(p_cat[p_off[w]:p_off[w] + k])
            rows = row_base[w] + np.arange(max(int(row_count[w]), 0))
            if rows.size and (rows.min() < 0 or rows.max() >= B):
                raise ValueError(f"warp {w}: rows out of range")
            if covered[rows].any():
                raise ValueError(f"warp {w}: a row is covered by two warps")
            covered[rows] = True
            tree_rows.extend(rows.tolist())
            tree_morph.extend([morphs[key]] * rows.size)
        self.n_trees = len(tree_rows)
        self.forest = None
        if self.n_trees:
            f = ForestPlan([list(map(int, p)) for p in parents], device=device,
                           plan_of=tree_morph, chains=True)
            rows = np.asarray(tree_rows, dtype=np.int64)
            k_of = np.asarray([len(parents[m]) for m in tree_morph], dtype=np.int32)
            node_ptr = np.append(rows * K_stride, B * K_stride).astype(np.int64)
            f.tensors["node_ptr"] = torch.as_tensor(node_ptr, device=device)
            f.tensors["tree_k"] = torch.as_tensor(k_of, device=device)
            f.max_k = int(k_of.max())
            self.forest = f
        # flat parent of every plane entry (-1: root, padding or uncovered row)
        par = np.full(B * K_stride, -1, dtype=np.int64)
        for r, m in zip(tree_rows, tree_morph):
            p = parents[m]
            base = r * K_stride
            nz = p >= 0
            idx = base + np.flatnonzero(nz)
            par[idx] = base + p[nz]
        self.is_node = np.zeros(B * K_stride, dtype=bool)
        for r, m in zip(tree_rows, tree_morph):
            self.is_node[r * K_stride:r * K_stride + len(parents[m])] = True
        self.parent_flat = torch.as_tensor(par, device=device)
        self.has_parent = self.parent_flat >= 0
        self.node_mask = torch.as_tensor(self.is_node, device=device)


def _multi_plan(plan, B, K_stride, device):
    return _multi_cache.get(tuple(plan), (B, K_stride, str(device)),
                            lambda: _MultiPlan(plan, B, K_stride, device))


def _multi_solve(d, a, b, mp):
    x = torch.zeros_like(b)
    if mp.forest is None:
        return x
    d, a, b = (t.contiguous() for t in (d, a, b))
    f = mp.forest.struct()
    with torch.cuda.device(d.device):
        rc = _lib.load().dgb_dhs_solve_forest(_lib.dtype_code(d.dtype), ctypes.byref(f),
                                              d.data_ptr(), a.data_ptr(), b.data_ptr(),
                                              x.data_ptr(), _lib.stream_ptr(d.device))
    _lib.check(rc, "dgb_dhs_solve_forest")
    return x


class _DHSMultiSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, d_mem, a_geom, b, mp):
        x = _multi_solve(d_mem, a_geom, b, mp)
        ctx.mp = mp
        ctx.save_for_backward(d_mem, a_geom, x)
        return x

    @staticmethod
    def backward(ctx, grad_out):
        d_mem, a_geom, x = ctx.saved_tensors
        mp = ctx.mp
        g = _multi_solve(d_mem, a_geom, grad_out.contiguous(), mp)  # symmetric system
        xf, gf = x.reshape(-1), g.reshape(-1)
        par = mp.parent_flat.clamp_min(0)
        drop_x = torch.where(mp.has_parent, xf - xf.index_select(0, par), xf)
        drop_g = torch.where(mp.has_parent, gf - gf.index_select(0, par), gf)
        grad_a = torch.where(mp.node_mask, -(drop_g * drop_x), torch.zeros_like(xf))
        return -(g * x), grad_a.view_as(x), g, None


def dhs_solve_multi_cuda(d_mem, a_geom, b, P_cat, ORDER_cat, LAYER_PTR_cat, WARP_P_OFF,
                         WARP_ORDER_OFF, WARP_LPTR_OFF, WARP_L, WARP_ROW_BASE, WARP_ROW_COUNT,
                         K_stride: int, L_max: int, threads: int, grid_x: int = None):
    """Row-padded multi-morphology tree solve with the reference's signature
    (triton/dhs_kernel_multi.py:831-888, called at integrators/tree.py:2273-2300).

    ``d_mem``, ``a_geom``, ``b`` are (B_total, K_stride) planes; warp ``w``
    covers rows ``WARP_ROW_BASE[w] ..`` (``WARP_ROW_COUNT[w]`` of them), all
    of the morphology whose parents start at ``P_cat[WARP_P_OFF[w]]`` and
    whose ``WARP_L[w]`` layers start at ``LAYER_PTR_cat[WARP_LPTR_OFF[w]]``
    (the last layer ends at the morphology's node count).  Every covered row
    is one tree in a single dgb_dhs_solve_forest launch (rows read in place);
    entries past a morphology's nodes and uncovered rows return 0.  The
    elimination order is this library's own (deterministic, children pulled in
    index order), so ORDER_cat only has to be a valid plan.  Gradients follow
    DHSSolveMultiPacked.backward (dhs_kernel_multi.py:699-780)."""
    plan = (P_cat, ORDER_cat, LAYER_PTR_cat, WARP_P_OFF, WARP_ORDER_OFF, WARP_LPTR_OFF, WARP_L,
            WARP_ROW_BASE, WARP_ROW_COUNT)
    B, _ = validate_tree_multi(d_mem, a_geom, b, plan, K_stride, L_max, threads, grid_x)
    mp = _multi_plan(plan, B, K_stride, d_mem.device)
    return _DHSMultiSolve.apply(d_mem, a_geom, b, mp)
