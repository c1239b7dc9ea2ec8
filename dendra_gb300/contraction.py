"""Tree contraction solve on the GB300 kernels.

Drop-in for the reference's CUDA tree-contraction solver
(models/integrators/triton/tree_contraction.py: ``prepare`` :651-656,
``solve`` :748-768, autograd/jvp/vmap :596-746) and for the plan object it
takes (``dendra_solvers.TreeContractionPlan``, built at
models/integrators/tree.py:841-867 with ``max_segment_interior_nodes``; the
factory ``tree_contraction`` is integrators/__init__.py:67-96).

The system is the scalar Hines matrix of the tree solve: node ``i`` has a
shunt ``d_i`` to ground and a conductance ``g_i`` to its parent (a root's
``g`` is a second shunt), so

    d_i x_i + g_i (x_i - x_parent(i)) + sum_children g_c (x_i - x_c) = rhs_i.

It is eliminated in conductance form: every step removes a node of degree
at most two and leaves a smaller network of the same kind (shunts, and a
bridge conductance between the two neighbours of a removed chain node).  With
``pivot = shunt + (near + far)`` a neighbour gains the shunt
``small * (large / pivot)`` of the pair (near, shunt) and the right-hand side
``(near / pivot) * value``; the bridge is the same product of (near, far).
Dividing the larger factor keeps shunts and bridges representable and avoids
the subtractive cancellation of the diagonal form
(tree_contraction.py:22-30, the same product).

The plan (host, once per topology):

1. **Segments** (``max_segment_interior_nodes = cap``): maximal runs of
   non-root nodes with exactly one child, cut into pieces of at most ``cap``
   interior nodes (a retained node separates pieces).  Each piece is condensed
   by one thread, top to bottom, into summaries for its two retained endpoints
   and a bridge between them (tree_contraction.py:237-287).  ``cap = None``
   skips this step.
2. **Skeleton contraction**: the retained nodes form a smaller tree that is
   contracted in rounds; a round removes every leaf and a maximal set of
   one-child nodes that are neither adjacent to each other nor to a removed
   leaf (rake and compress, Miller and Reif 1985), so a tree of ``R`` nodes
   takes O(log R) rounds for a balanced shape.  Every surviving neighbour
   gathers the contributions of its removed neighbours in ascending order
   (deterministic, no atomics); results go to fresh state and edge slots, so a
   round never overwrites what another thread of the same round reads.
3. The roots solve ``x = value / (shunt + g_root)``; the rounds are undone in
   reverse (``x = (value + near x_a + far x_c) / pivot``) and finally every
   segment is recovered bottom to top.

The kernel runs one block (32-256 threads) per batch row with all scratch in
shared memory (in a global workspace when a row's scratch does not fit, for
trees of any size) and uses correctly rounded operations only, so the
oracle's numpy restatement of the same plan reproduces it bit for bit.
"""

from __future__ import annotations

import ctypes
from numbers import Integral

import numpy as np
import torch

from . import _lib
from .solvers import _validate_float_group

_P = ctypes.c_void_p
_I32 = ctypes.c_int32


class DgbContractPlan(ctypes.Structure):
    """Mirror of ``dgb_contract_plan`` (field order and types must match)."""

    _fields_ = [
        ("size", _I32), ("n_segments", _I32), ("n_interior", _I32), ("n_retained", _I32),
        ("n_endpoints", _I32), ("n_rounds", _I32), ("n_updates", _I32),
        ("n_incidence", _I32), ("n_eliminated", _I32), ("n_roots", _I32),
        ("n_bridges", _I32), ("threads", _I32),
        ("seg", _P), ("interior", _P), ("retained", _P), ("endpoint", _P),
        ("round_ptr", _P), ("update", _P), ("incidence", _P), ("recovery", _P),
        ("roots", _P),
    ]


_TABLES = ("seg", "interior", "retained", "endpoint", "round_ptr", "update", "incidence",
           "recovery", "roots")


def _validate_cap(cap):
    if cap is None:
        return None
    if isinstance(cap, bool) or not isinstance(cap, Integral):
        raise TypeError("max_segment_interior_nodes must be a positive integer or None")
    if cap <= 0:
        raise ValueError("max_segment_interior_nodes must be positive")
    return int(cap)


def _validate_parent(parent):
    if isinstance(parent, torch.Tensor):
        parent = parent.detach().cpu().numpy()
    parent = np.asarray(parent)
    if parent.ndim != 1 or parent.size == 0:
        raise ValueError("parent must be a non-empty one-dimensional index array")
    if not np.issubdtype(parent.dtype, np.integer):
        raise TypeError("parent must hold integers")
    parent = parent.astype(np.int64)
    K = parent.size
    if K > (1 << 30):
        raise ValueError("tree too large")
    bad = (parent < -1) | (parent >= K)
    if bad.any():
        i = int(np.flatnonzero(bad)[0])
        raise ValueError(f"parent index at node {i} must be in [-1, {K - 1}]; got {parent[i]}")
    if (parent == np.arange(K)).any():
        raise ValueError("a node cannot be its own parent")
    if not (parent < 0).any():
        raise ValueError("parent must contain at least one root (-1)")
    # every node must reach a root: walk up with path marking
    state = np.zeros(K, dtype=np.int8)  # 0 unknown, 1 on stack, 2 reaches a root
    for s in range(K):
        path, n = [], s
        while n >= 0 and state[n] == 0:
            state[n] = 1
            path.append(n)
            n = int(parent[n])
        if n >= 0 and state[n] == 1:
            raise ValueError("parent contains a cycle")
        for p in path:
            state[p] = 2
    return parent


def _preorder(parent, children):
    out = []
    stack = [int(r) for r in np.flatnonzero(parent < 0)[::-1]]
    while stack:
        n = stack.pop()
        out.append(n)
        stack.extend(reversed(children[n]))
    return out


def build_contraction_tables(parent, cap=16):
    """Plan tables (dict of int32 arrays plus counts) for one topology.

    ``parent[i]`` is node i's parent or -1 for a root (any node order; several
    roots make a forest).  Table layout (every row a field):

    * ``seg`` (6, S): ancestor and child (retained indices), interior start,
      end, first interior node, stride (+1 or -1 when the run's node ids are
      consecutive, else 0)
    * ``interior`` (I,): node ids, each segment's run top to bottom
    * ``retained`` (4, R): node, incoming segment (-1), endpoint start, count
    * ``endpoint`` (2, E): segment, side (0 the ancestor end, 1 the child end)
    * ``round_ptr`` (2, P+1): update and recovery offsets per round
    * ``update`` (3, U): target's current state slot, incidence start, count;
      update u writes state slot R + u
    * ``incidence`` (4, Q): removed node's state slot, near edge slot, far
      edge slot (-1), bridge slot written (-1)
    * ``recovery`` (6, N): node (retained index), state slot, ancestor,
      child (-1), near edge slot, far edge slot (-1)
    * ``roots`` (2, n_roots): retained index, final state slot

    State slots 0..R-1 and edge slots 0..R-1 hold the reduced shunt/value and
    the up-edge conductance of every retained node; the root's edge slot holds
    its own ``g``.
    """
    cap = _validate_cap(cap)
    parent = _validate_parent(parent)
    K = parent.size
    children = [[] for _ in range(K)]
    for i in range(K):
        if parent[i] >= 0:
            children[int(parent[i])].append(i)
    order = _preorder(parent, children)

    # 1. segments
    segs = []  # (ancestor, child, [interior top -> bottom])
    is_interior = np.zeros(K, dtype=bool)
    if cap is not None:
        linkable = np.array([parent[i] >= 0 and len(children[i]) == 1 for i in range(K)])
        for n0 in order:
            if not linkable[n0] or linkable[parent[n0]]:
                continue
            run, n = [n0], n0
            while linkable[children[n][0]]:
                n = children[n][0]
                run.append(n)
            bottom = children[n][0]
            anc, pos = int(parent[n0]), 0
            while pos < len(run):
                piece = run[pos:pos + cap]
                nxt = pos + cap
                if nxt < len(run):
                    segs.append((anc, run[nxt], piece))
                    anc, pos = run[nxt], nxt + 1
                else:
                    segs.append((anc, bottom, piece))
                    pos = len(run)
        for _, _, piece in segs:
            is_interior[piece] = True
    # longest first: threads take segments in turn, so this balances them
    segs.sort(key=lambda sg: -len(sg[2]))
    S = len(segs)
    interior = [n for _, _, piece in segs for n in piece]
    seg = np.zeros((6, S), dtype=np.int64)
    start = 0
    for s, (a, c, piece) in enumerate(segs):
        step = np.diff(piece)
        stride = 1 if (step == 1).all() else (-1 if (step == -1).all() else 0)
        seg[:, s] = (a, c, start, start + len(piece), piece[0], stride)
        start += len(piece)

    # 2. retained nodes and their endpoint summaries
    ret_nodes = np.flatnonzero(~is_interior)
    R = ret_nodes.size
    local = np.full(K, -1, dtype=np.int64)
    local[ret_nodes] = np.arange(R)
    incoming = np.full(R, -1, dtype=np.int64)
    ends = [[] for _ in range(R)]
    for s, (a, c, _) in enumerate(segs):
        ends[local[a]].append((s, 0))
        ends[local[c]].append((s, 1))
        incoming[local[c]] = s
    retained = np.zeros((4, R), dtype=np.int64)
    endpoint = []
    for r in range(R):
        e = sorted(ends[r])
        retained[:, r] = (ret_nodes[r], incoming[r], len(endpoint), len(e))
        endpoint.extend(e)
    endpoint = np.asarray(endpoint, dtype=np.int64).reshape(-1, 2).T
    if S:
        seg[:2] = local[seg[:2]]  # endpoints as retained indices
    lpar = np.full(R, -1, dtype=np.int64)
    for r in range(R):
        node = ret_nodes[r]
        if incoming[r] >= 0:
            lpar[r] = local[segs[incoming[r]][0]]
        elif parent[node] >= 0:
            lpar[r] = local[parent[node]]
    roots = np.flatnonzero(lpar < 0)

    # 3. rake/compress rounds on the retained tree
    kids = [set() for _ in range(R)]
    for r in range(R):
        if lpar[r] >= 0:
            kids[lpar[r]].add(r)
    alive = np.ones(R, dtype=bool)
    cur_state = np.arange(R, dtype=np.int64)
    cur_edge = np.arange(R, dtype=np.int64)
    n_edge = R
    updates, incidence, recovery = [], [], []
    round_ptr = [[0], [0]]
    remaining = R - roots.size
    while remaining > 0:
        # top-down order of the live forest
        topo, stack = [], list(roots[::-1])
        while stack:
            n = stack.pop()
            topo.append(n)
            stack.extend(sorted(kids[n], reverse=True))
        sel = set()
        for n in topo:
            if lpar[n] >= 0 and not kids[n]:
                sel.add(n)
        for n in topo:
            if lpar[n] < 0 or len(kids[n]) != 1 or n in sel or lpar[n] in sel:
                continue
            (c,) = tuple(kids[n])
            if c in sel:
                continue
            sel.add(n)
        removed = sorted(sel)
        gathers = {}
        for m in removed:
            a = int(lpar[m])
            c = next(iter(kids[m])) if kids[m] else -1
            far_to_child = int(cur_edge[c]) if c >= 0 else -1
            recovery.append((m, cur_state[m], a, c, cur_edge[m], far_to_child))
            gathers.setdefault(a, []).append((m, int(cur_edge[m]), far_to_child, -1))
            if c >= 0:
                gathers.setdefault(c, []).append((m, int(cur_edge[c]), int(cur_edge[m]), n_edge))
                n_edge += 1
        new_edges = {}
        for t in sorted(gathers):
            recs = sorted(gathers[t])
            updates.append((cur_state[t], len(incidence), len(recs)))
            for m, near, far, dest in recs:
                incidence.append((cur_state[m], near, far, dest))
                if dest >= 0:
                    new_edges[t] = dest
            cur_state[t] = R + len(updates) - 1
        for m in removed:
            a = int(lpar[m])
            alive[m] = False
            kids[a].discard(m)
            for c in kids[m]:
                lpar[c] = a
                kids[a].add(c)
            kids[m] = set()
        for c, dest in new_edges.items():
            cur_edge[c] = dest
        remaining -= len(removed)
        round_ptr[0].append(len(updates))
        round_ptr[1].append(len(recovery))

    def table(rows, width):
        return np.asarray(rows, dtype=np.int64).reshape(-1, width).T.copy()

    tables = dict(
        seg=seg, interior=np.asarray(interior, dtype=np.int64), retained=retained,
        endpoint=endpoint, round_ptr=np.asarray(round_ptr, dtype=np.int64),
        update=table(updates, 3), incidence=table(incidence, 4),
        recovery=table(recovery, 6),
        roots=np.stack([roots, cur_state[roots]]).astype(np.int64))
    tables = {k: v.astype(np.int32) for k, v in tables.items()}
    counts = dict(size=K, n_segments=S, n_interior=len(interior), n_retained=R,
                  n_endpoints=tables["endpoint"].shape[1],
                  n_rounds=len(round_ptr[0]) - 1, n_updates=len(updates),
                  n_incidence=len(incidence), n_eliminated=len(recovery),
                  n_roots=int(roots.size), n_bridges=n_edge - R)
    _check_tables(tables, counts)
    return tables, counts


def _check_tables(t, c):
    """Every index the kernel follows lies inside its table (the kernel
    trusts the plan; a failure here is a planner bug)."""
    K, S, I, R = c["size"], c["n_segments"], c["n_interior"], c["n_retained"]
    U, Q, N, P = c["n_updates"], c["n_incidence"], c["n_eliminated"], c["n_rounds"]
    n_state, n_edge = R + U, R + c["n_bridges"]

    def within(a, lo, hi, what):
        a = np.asarray(a)
        if a.size and (a.min() < lo or a.max() >= hi):
            raise RuntimeError(f"contraction plan: {what} out of range")

    seg, ret, upd, inc, rec = t["seg"], t["retained"], t["update"], t["incidence"], t["recovery"]
    within(seg[:2], 0, R, "segment endpoint")
    within(seg[2:4], 0, I + 1, "segment interior range")
    if S and ((seg[2] >= seg[3]).any()):
        raise RuntimeError("contraction plan: empty segment")
    for s in range(S):
        run = t["interior"][seg[2, s]:seg[3, s]]
        if seg[4, s] != run[0] or (seg[5, s] != 0 and (
                run != seg[4, s] + seg[5, s] * np.arange(run.size)).any()):
            raise RuntimeError("contraction plan: segment stride")
    within(t["interior"], 0, K, "interior node")
    within(ret[0], 0, K, "retained node")
    within(ret[1], -1, S, "incoming segment")
    within(ret[2], 0, c["n_endpoints"] + 1, "endpoint start")
    if R and (ret[2] + ret[3] > c["n_endpoints"]).any():
        raise RuntimeError("contraction plan: endpoint range out of range")
    within(t["endpoint"][0], 0, S, "endpoint segment")
    within(t["endpoint"][1], 0, 2, "endpoint side")
    rp = t["round_ptr"]
    if rp.shape != (2, P + 1) or rp[0, -1] != U or rp[1, -1] != N or (np.diff(rp, axis=1) < 0).any():
        raise RuntimeError("contraction plan: round offsets")
    within(upd[0], 0, n_state, "update source")
    if U and ((upd[1] < 0).any() or (upd[2] < 1).any() or (upd[1] + upd[2] > Q).any()):
        raise RuntimeError("contraction plan: incidence range out of range")
    within(inc[0], 0, n_state, "removed state slot")
    within(inc[1], 0, n_edge, "near edge")
    within(inc[2], -1, n_edge, "far edge")
    within(inc[3], -1, n_edge, "bridge slot")
    within(rec[0], 0, R, "recovered node")
    within(rec[1], 0, n_state, "recovery state slot")
    within(rec[2], 0, R, "recovery ancestor")
    within(rec[3], -1, R, "recovery child")
    within(rec[4], 0, n_edge, "recovery near edge")
    within(rec[5], -1, n_edge, "recovery far edge")
    within(t["roots"][0], 0, R, "root")
    within(t["roots"][1], 0, n_state, "root state slot")
    if c["n_endpoints"] != 2 * S or N != R - c["n_roots"] or R + I != K:
        raise RuntimeError("contraction plan: inconsistent counts")


class TreeContractionPlan:
    """Immutable contraction plan of one topology (the role of
    ``dendra_solvers.TreeContractionPlan``, integrators/tree.py:841-867).

    ``parent``: parent index per node (-1 for a root; any node order).
    ``max_segment_interior_nodes``: the segment cap (default 16, as
    ``dn.tree_contraction``); None contracts every node in rounds.
    """

    def __init__(self, parent, max_segment_interior_nodes=16, threads=0):
        self.max_segment_interior_nodes = _validate_cap(max_segment_interior_nodes)
        if threads not in (0, 32, 64, 128, 256):
            raise ValueError("threads must be 0 (automatic), 32, 64, 128 or 256")
        self.threads = int(threads)
        self.tables, self.counts = build_contraction_tables(
            parent, self.max_segment_interior_nodes)
        self.size = self.counts["size"]
        p = _validate_parent(parent)
        self.parent = p.astype(np.int32)
        self._devices = {}

    def prepare(self, device):
        """Upload the tables once per device (before CUDA-graph capture)."""
        device = torch.device(device)
        if device.type != "cuda":
            raise ValueError("CUDA tree contraction requires a CUDA device")
        if device.index is None:
            device = torch.device("cuda", torch.cuda.current_device())
        hit = self._devices.get(device)
        if hit is None:
            parts, offsets, off = [], {}, 0
            for k in _TABLES:
                a = _device_layout(k, self.tables[k], self.tables)
                offsets[k] = off
                pad = (-a.size) % 4  # every table starts on 16 bytes
                parts += [a, np.zeros(pad, dtype=np.int32)]
                off += a.size + pad
            packed = torch.as_tensor(np.concatenate(parts + [np.zeros(4, dtype=np.int32)])).to(
                device)
            parent = torch.as_tensor(self.parent, dtype=torch.int64).to(device)
            is_root = parent < 0
            hit = (packed, offsets, parent.clamp_min(0), is_root)
            self._devices[device] = hit
        return hit

    def struct(self, device):
        packed, offsets, _, _ = self.prepare(device)
        s = DgbContractPlan()
        for k, v in self.counts.items():
            setattr(s, k, v)
        s.threads = self.threads
        base = packed.data_ptr()
        for k in _TABLES:
            setattr(s, k, base + 4 * offsets[k])
        return s

    def smem_values(self):
        """Scratch values per batch row the kernel keeps in shared memory."""
        c = self.counts
        return (3 * c["size"] + c["n_interior"] + 5 * c["n_segments"]
                + 2 * (c["n_retained"] + c["n_updates"]) + 2 * c["n_retained"] + c["n_bridges"])


def _device_layout(name, table, tables):
    """Device form of a plan table: records of 16 bytes (one vector load
    each) except ``interior`` and ``roots``, stored field after field."""
    if name == "seg":         # {ancestor, child, start, end}, {first, stride, child, ancestor nodes}
        ret_node = tables["retained"][0]
        ends = ret_node[table[:2]] if table.shape[1] else np.zeros((2, 0), np.int32)
        return np.vstack([table, ends[1:2], ends[0:1]]).T.ravel().copy()
    if name == "retained":    # {node, incoming, endpoint start, count}, 4 endpoint codes
        ep = tables["endpoint"]
        codes = np.full((4, table.shape[1]), -1, np.int32)
        for r in range(table.shape[1]):
            e0, ne = table[2, r], table[3, r]
            for k in range(min(ne, 4)):
                codes[k, r] = 2 * ep[0, e0 + k] + ep[1, e0 + k]
        return np.vstack([table, codes]).T.ravel().copy()
    if name == "endpoint":    # {segment, side}
        return table.T.ravel().copy()
    if name == "update":      # {source, incidence start, count, 0}
        return np.vstack([table, np.zeros((1, table.shape[1]), np.int32)]).T.ravel().copy()
    if name == "incidence":   # {removed, near, far, bridge}
        return table.T.ravel().copy()
    if name == "recovery":    # {node, state, ancestor, child}, {near, far, 0, 0}
        z = np.zeros((2, table.shape[1]), np.int32)
        return np.vstack([table, z]).T.ravel().copy()
    return table.ravel()


def prepare(plan, device):
    """Upload the plan's tables to ``device`` (tree_contraction.py:651-656)."""
    device = torch.device(device)
    if device.type != "cuda":
        raise ValueError("CUDA tree contraction requires a CUDA device")
    plan.prepare(device)
    return plan


def _launch(d, g, rhs, plan):
    B, K = d.shape
    out = torch.empty_like(rhs, memory_format=torch.contiguous_format)
    if B == 0:
        return out
    d, g, rhs = (v.contiguous() for v in (d, g, rhs))
    s = plan.struct(d.device)
    L = _lib.load()
    code = _lib.dtype_code(d.dtype)
    with torch.cuda.device(d.device):
        nwork = L.dgb_tree_contract_work_size(code, ctypes.byref(s), B)
        work = torch.empty(nwork, dtype=torch.uint8, device=d.device) if nwork else None
        rc = L.dgb_tree_contract_solve(
            code, B, ctypes.byref(s), d.data_ptr(), g.data_ptr(), rhs.data_ptr(),
            out.data_ptr(), None if work is None else work.data_ptr(), nwork,
            _lib.stream_ptr(d.device))
    _lib.check(rc, "dgb_tree_contract_solve")
    return out


def _gradients(adjoint, x, plan, needs):
    """Reference gradients (tree_contraction.py:596-609)."""
    _, _, parent, is_root = plan.prepare(x.device)
    need_d, need_g, need_rhs = needs
    grad_g = None
    if need_g:
        x_drop = torch.where(is_root, x, x - x.index_select(-1, parent))
        a_drop = torch.where(is_root, adjoint, adjoint - adjoint.index_select(-1, parent))
        grad_g = -(x_drop * a_drop)
    return (-(adjoint * x) if need_d else None, grad_g, adjoint if need_rhs else None)


class _TreeContraction(torch.autograd.Function):
    """Solve with the symmetric-system adjoint, forward-mode tangent and vmap
    (tree_contraction.py:698-735)."""

    @staticmethod
    def forward(d, g, rhs, plan):
        return _launch(d, g, rhs, plan)

    @staticmethod
    def setup_context(ctx, inputs, output):
        d, g, _, plan = inputs
        ctx.plan = plan
        ctx.save_for_backward(d, g, output)
        ctx.save_for_forward(d, g, output)

    @staticmethod
    def backward(ctx, cotangent):
        d, g, x = ctx.saved_tensors
        adjoint = _TreeContraction.apply(d, g, cotangent.contiguous(), ctx.plan)
        return (*_gradients(adjoint, x, ctx.plan, ctx.needs_input_grad[:3]), None)

    @staticmethod
    def jvp(ctx, d_tangent, g_tangent, rhs_tangent, _plan_tangent):
        d, g, x = ctx.saved_tensors
        _, _, parent, is_root = ctx.plan.prepare(x.device)
        tangent = torch.zeros_like(x) if rhs_tangent is None else rhs_tangent
        if d_tangent is not None:
            tangent = tangent - d_tangent * x
        if g_tangent is not None:
            flow = torch.where(is_root, torch.zeros_like(x),
                               g_tangent * (x - x.index_select(-1, parent)))
            tangent = (tangent - flow).scatter_add(
                -1, parent.unsqueeze(0).expand_as(flow), flow)
            tangent = tangent - torch.where(is_root, g_tangent * x, torch.zeros_like(x))
        return _TreeContraction.apply(d, g, tangent.contiguous(), ctx.plan)

    @staticmethod
    def vmap(info, in_dims, d, g, rhs, plan):
        if in_dims[3] is not None:
            raise ValueError("tree contraction topology must be shared under vmap")
        size = info.batch_size
        flat = []
        for t, dim in zip((d, g, rhs), in_dims[:3]):
            t = t.unsqueeze(0).expand(size, *t.shape) if dim is None else t.movedim(dim, 0)
            flat.append(t.reshape(-1, t.shape[-1]))
        out = _TreeContraction.apply(*flat, plan)
        return out.reshape(size, -1, out.shape[-1]), 0


def validate_contraction(d, g, rhs, plan):
    """The reference's checks (tree_contraction.py:750-766) plus the kernel's limits."""
    if not isinstance(plan, TreeContractionPlan):
        raise TypeError("plan must be a TreeContractionPlan")
    for name, t in (("d", d), ("g", g), ("rhs", rhs)):
        if not isinstance(t, torch.Tensor):
            raise TypeError(f"{name} must be a torch.Tensor")
    if d.ndim != 2 or d.shape[1] != plan.size:
        raise ValueError("tree contraction inputs must have shape (B, K) matching the plan")
    if d.dtype not in (torch.float32, torch.float64):
        raise ValueError("CUDA tree contraction requires float32 or float64")
    for t in (d, g, rhs):
        if (t.shape != d.shape or t.device != d.device or t.device.type != "cuda"
                or t.dtype != d.dtype or t.layout != torch.strided):
            raise ValueError("tree contraction inputs must be same-shaped strided CUDA "
                             "tensors with matching dtypes")
    _validate_float_group((("d", d), ("g", g), ("rhs", rhs)))


def solve(d, g, rhs, plan):
    """Solve a batch of scalar Hines systems sharing ``plan``'s topology
    (drop-in for tree_contraction.solve, :748-768): ``d``, ``g``, ``rhs`` are
    (B, K) float32/float64 CUDA tensors in the plan's node order."""
    validate_contraction(d, g, rhs, plan)
    return _TreeContraction.apply(d, g, rhs, plan)


def tree_contraction_solve(d_mem, a_geom, rhs, parent, order, layers, *, plan):
    """Tree-integrator solver signature (integrators/tree.py:186-190)."""
    return solve(d_mem, a_geom, rhs, plan)
