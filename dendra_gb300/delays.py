"""Interpolated (differentiable) delay transport on the GB300 kernels.

Host mirrors of the reference's interpolated-delay pieces, every per-step
operation on the GPU and deterministic (one thread owns one ring column and
adds in the reference's order; no floating-point atomics):

* :func:`linear_delay_taps`, :func:`delay_interpolation` — positions
  ``max(delay / dt, 1)`` split into offsets and shares
  (networks/_event_delivery.py:202-226); elementwise, once per rollout
* :func:`ordered_two_tap_enqueue`, :func:`ordered_two_tap_enqueue_from_source`
  and the in-place ``..._`` forms — the ordered two-tap op
  (networks/_two_tap_enqueue_cpu.cpp:61-152, 317-342) with its adjoint
  (networks/_two_tap_enqueue.py:94-150) as a ``torch.autograd.Function``
* :func:`delay_ring_gather_two_tap`, :func:`delay_ring_two_tap_vjp`
  (_two_tap_enqueue_cpu.cpp:206-315)
* :func:`dense_interpolated_delay_transition` — the two- and three-tap
  transition (networks/_event_delivery.py:229-308)
* :func:`two_tap_rollout` — many steps of the two-tap transition in one
  launch, each block's ring columns held in shared memory for the whole
  rollout, with a hand-written reverse sweep (the adjoint the reference takes
  by autograd through its per-step loop)

Ring layout: ``queue[depth][width]`` (row = delivery step, column = target
slot).  Two-tap addresses are flat and relative to the start of row ``slot``:
destination ``(slot*width + address) mod (depth*width)``.
"""

from __future__ import annotations

from typing import NamedTuple

import torch

from . import _lib
from ._cache import TensorKeyedCache

ERR_SLOT, ERR_ADDRESS, ERR_SOURCE, ERR_PLAN = 1, 2, 3, 4


class DenseTransition(NamedTuple):
    """Result of one transition (the reference's networks/_event_delivery.py:25-29)."""

    queue: torch.Tensor
    slot: torch.Tensor
    global_step: torch.Tensor
    event_queue: torch.Tensor | None


# ---------------------------------------------------------------------------
# delay positions
# ---------------------------------------------------------------------------
def linear_delay_taps(positions):
    """(lower offset as int64, upper-tap share) of positions in steps."""
    lower = torch.floor(positions)
    return lower.to(torch.int64), positions - lower


def delay_interpolation(delays, dt, *, dtype, taps, sigma):
    """Offsets and shares of physical delays.

    Positions are ``max(delay / dt, 1)`` steps.  Two taps: the floor and the
    upper share (the fractional part).  Three taps: offsets ``floor - 1,
    floor, floor + 1`` with Gaussian weights ``softmax(-((pos - centre) /
    (sigma + 1e-6))**2 / 2)`` (the reference's 1e-6 denominator offset).
    """
    pos = (delays.to(dtype) / dt.to(dtype).reshape(1)).clamp_min(1.0)
    if taps == 2:
        return linear_delay_taps(pos)
    base = torch.floor(pos).to(torch.int64)
    offsets = torch.stack([base - 1, base, base + 1], dim=-1)
    z = (pos.unsqueeze(-1) - offsets.to(dtype)) / (sigma + 1e-6)
    return offsets, torch.softmax(-0.5 * z ** 2, dim=-1)


# ---------------------------------------------------------------------------
# column plans
# ---------------------------------------------------------------------------
def _column_lists(keys, n):
    """(ptr[n+1], edge ids grouped by key, ascending within a key)."""
    order = torch.argsort(keys, stable=True)
    ptr = torch.zeros(n + 1, dtype=torch.int64, device=keys.device)
    if keys.numel():
        torch.cumsum(torch.bincount(keys, minlength=n), 0, out=ptr[1:])
    return ptr, order.to(torch.int64).contiguous()


class TapPlan:
    """Per-column edge lists of a set of two-tap addresses.

    ``lower_ptr/lower_edge`` list, for every ring column, the edges whose
    lower address lies in it (ascending), ``upper_ptr/upper_edge`` the same for
    upper addresses.  ``consistent`` is true when every edge's two taps share a
    column; then ``col_ptr/col_edge`` serve both (the multi-step kernels need
    this).  With source indices, ``src_ptr/src_edge`` list each source's edges.
    """

    def __init__(self, depth, width, lower, upper, pre_idx=None, n_sources=0,
                 post_idx=None):
        self.depth, self.width = int(depth), int(width)
        size = self.depth * self.width
        self.n_edges = int(lower.numel() if lower is not None else post_idx.numel())
        if post_idx is not None:
            # both taps in column post_idx[e] (the transition's own addresses)
            if self.n_edges and not bool(((post_idx >= 0) & (post_idx < self.width)).all()):
                raise IndexError("post_idx is outside the delivery ring width")
            self.lower_ptr, self.lower_edge = _column_lists(post_idx, self.width)
            self.upper_ptr, self.upper_edge = self.lower_ptr, self.lower_edge
            self.consistent = True
        else:
            if self.n_edges and not bool(
                ((lower >= 0) & (lower < size) & (upper >= 0) & (upper < size)).all()):
                raise RuntimeError("Two-tap address is outside the delivery ring")
            lo_col = lower.remainder(self.width) if self.width else lower
            up_col = upper.remainder(self.width) if self.width else upper
            self.lower_ptr, self.lower_edge = _column_lists(lo_col, self.width)
            self.consistent = bool(torch.equal(lo_col, up_col))
            if self.consistent:
                self.upper_ptr, self.upper_edge = self.lower_ptr, self.lower_edge
            else:
                self.upper_ptr, self.upper_edge = _column_lists(up_col, self.width)
        self.col_ptr = self.lower_ptr if self.consistent else None
        self.col_edge = self.lower_edge if self.consistent else None
        self.src_ptr = self.src_edge = None
        self.n_sources = int(n_sources)
        if pre_idx is not None:
            if self.n_edges and not bool(((pre_idx >= 0) & (pre_idx < self.n_sources)).all()):
                raise IndexError("Two-tap source index is out of range")
            self.src_ptr, self.src_edge = _column_lists(pre_idx, self.n_sources)


_plans = TensorKeyedCache(16)


def _cached_plan(key_tensors, depth, width, n_sources, build):
    """Plan cache keyed on tensor identity and version (entries hold the tensors)."""
    return _plans.get(key_tensors, (depth, width, n_sources), build)


def two_tap_plan(depth, width, lower, upper, pre_idx=None, n_sources=0):
    """Cached :class:`TapPlan` of flat two-tap addresses."""
    keys = (lower, upper, pre_idx)
    return _cached_plan(keys, int(depth), int(width), int(n_sources),
                        lambda: TapPlan(depth, width, lower, upper, pre_idx, n_sources))


def post_plan(depth, width, post_idx, pre_idx=None, n_sources=0):
    """Cached :class:`TapPlan` for taps in column ``post_idx[e]``."""
    keys = (post_idx, pre_idx)
    return _cached_plan(keys, int(depth), int(width), int(n_sources),
                        lambda: TapPlan(depth, width, None, None, pre_idx, n_sources,
                                        post_idx=post_idx))


# ---------------------------------------------------------------------------
# argument checks (the reference's TORCH_CHECK messages, _two_tap_enqueue_cpu.cpp:12-100)
# ---------------------------------------------------------------------------
def _ptr(t):
    return None if t is None else t.data_ptr()


def _check_queue(queue):
    if not (isinstance(queue, torch.Tensor) and queue.is_cuda and queue.dim() == 2
            and queue.size(0) > 0 and queue.dtype in (torch.float32, torch.float64)):
        raise RuntimeError(
            "Two-tap queue must be a CUDA float32 or float64 matrix with positive depth")


def _check_vec(t, dtype, n, name, device):
    if not (isinstance(t, torch.Tensor) and t.device == device and t.dim() == 1
            and t.dtype == dtype and t.numel() == n and t.is_contiguous()):
        raise RuntimeError(f"{name} must be a contiguous CUDA tensor of the required dtype "
                           "and size")


def _slot_tensor(slot, depth, device):
    """Slot as a one-element int64 device tensor; host values are range-checked here,
    device values by the kernels (``delay_status``)."""
    if isinstance(slot, torch.Tensor) and slot.is_cuda:
        if slot.numel() != 1 or slot.dtype != torch.int64:
            raise RuntimeError("slot must be a one-element int64 tensor")
        return slot.reshape(1)
    value = int(slot.reshape(-1)[0]) if isinstance(slot, torch.Tensor) else int(slot)
    if not 0 <= value < depth:
        raise RuntimeError("Two-tap slot is outside the delivery ring")
    return torch.tensor([value], dtype=torch.int64, device=device)


def delay_status() -> int:
    """First device-side index error of the delay kernels (0 = none), cleared."""
    rc = _lib.load().dgb_delay_status(_lib.stream_ptr())
    if rc < 0:
        _lib.check(rc, "dgb_delay_status")
    return rc


# ---------------------------------------------------------------------------
# raw launches
# ---------------------------------------------------------------------------
def _enqueue_into(ring, slot_t, weights, gates, fraction, lower, upper, pre_idx, plan,
                  payload=None):
    L = _lib.load()
    depth, width = ring.shape
    _lib.check(L.dgb_two_tap_enqueue(
        _lib.dtype_code(ring.dtype), ring.data_ptr(), depth, width, slot_t.data_ptr(),
        plan.n_edges, _ptr(weights), _ptr(gates), _ptr(pre_idx), plan.n_sources,
        _ptr(fraction), _ptr(lower), _ptr(upper), plan.lower_ptr.data_ptr(),
        _ptr(plan.lower_edge), plan.upper_ptr.data_ptr(), _ptr(plan.upper_edge),
        _ptr(payload), _lib.stream_ptr(ring.device)), "dgb_two_tap_enqueue")


def _vjp(ring, offset_t, weights, gates, fraction, lower, upper, pre_idx, plan):
    L = _lib.load()
    dw = torch.empty_like(weights)
    dg = torch.empty_like(gates)
    df = torch.empty_like(fraction)
    _lib.check(L.dgb_two_tap_vjp(
        _lib.dtype_code(ring.dtype), ring.data_ptr(), ring.numel(), offset_t.data_ptr(),
        weights.numel(), _ptr(weights), _ptr(gates), _ptr(pre_idx),
        plan.n_sources if pre_idx is not None else 0, _ptr(fraction), _ptr(lower),
        _ptr(upper), _ptr(plan.src_ptr), _ptr(plan.src_edge), dw.data_ptr(), dg.data_ptr(),
        df.data_ptr(), _lib.stream_ptr(ring.device)), "dgb_two_tap_vjp")
    return dw, dg, df


def _prepare(queue, weights, gates, fraction, lower, upper, pre_idx):
    _check_queue(queue)
    dev, dt = queue.device, queue.dtype
    for name, t in (("weights", weights), ("gates", gates), ("fraction", fraction),
                    ("lower", lower), ("upper", upper)):
        if not isinstance(t, torch.Tensor) or t.dim() != 1:
            raise RuntimeError("Two-tap edge inputs must be vectors")
    n = weights.numel()
    if queue.numel() == 0 and n:
        raise RuntimeError("Empty ring cannot receive edges")
    _check_vec(weights, dt, n, "weights", dev)
    _check_vec(gates, dt, gates.numel() if pre_idx is not None else n, "gates", dev)
    _check_vec(fraction, dt, n, "fraction", dev)
    _check_vec(lower, torch.int64, n, "lower", dev)
    _check_vec(upper, torch.int64, n, "upper", dev)
    if pre_idx is not None:
        _check_vec(pre_idx, torch.int64, n, "source indices", dev)
    return n


# ---------------------------------------------------------------------------
# autograd operators
# ---------------------------------------------------------------------------
class _TwoTapEnqueue(torch.autograd.Function):
    """queue -> new queue (row slot cleared, two taps added); linear in queue."""

    @staticmethod
    def forward(ctx, queue, slot_t, weights, gates, fraction, lower, upper, pre_idx, plan):
        out = queue.clone(memory_format=torch.contiguous_format)
        _enqueue_into(out, slot_t, weights, gates, fraction, lower, upper, pre_idx, plan)
        ctx.save_for_backward(slot_t, weights, gates, fraction, lower, upper,
                              *(() if pre_idx is None else (pre_idx,)))
        ctx.plan = plan
        ctx.width = queue.shape[1]
        return out

    @staticmethod
    def backward(ctx, grad_out):
        slot_t, weights, gates, fraction, lower, upper, *rest = ctx.saved_tensors
        pre_idx = rest[0] if rest else None
        need_q, _, need_w, need_g, need_f = ctx.needs_input_grad[:5]
        grad_out = grad_out.contiguous()
        gq = grad_out.index_fill(0, slot_t, 0) if need_q else None
        dw = dg = df = None
        if need_w or need_g or need_f:
            offset_t = slot_t * ctx.width
            dw, dg, df = _vjp(grad_out, offset_t, weights, gates, fraction, lower, upper,
                              pre_idx, ctx.plan)
            dw, dg, df = (dw if need_w else None, dg if need_g else None,
                          df if need_f else None)
        return gq, None, dw, dg, df, None, None, None, None


class _ThreeTapEnqueue(torch.autograd.Function):
    @staticmethod
    def forward(ctx, queue, slot_t, weights, gates, coeff, offsets, post_idx, plan):
        out = queue.clone(memory_format=torch.contiguous_format)
        L = _lib.load()
        depth, width = out.shape
        n = weights.numel()
        _lib.check(L.dgb_three_tap_enqueue(
            _lib.dtype_code(out.dtype), out.data_ptr(), depth, width, slot_t.data_ptr(), n,
            _ptr(weights), _ptr(gates), None, 0, _ptr(coeff), _ptr(offsets), _ptr(post_idx),
            plan.lower_ptr.data_ptr(), _ptr(plan.lower_edge), None,
            _lib.stream_ptr(out.device)), "dgb_three_tap_enqueue")
        ctx.save_for_backward(slot_t, weights, gates, coeff, offsets, post_idx)
        return out

    @staticmethod
    def backward(ctx, grad_out):
        slot_t, weights, gates, coeff, offsets, post_idx = ctx.saved_tensors
        grad_out = grad_out.contiguous()
        gq = grad_out.index_fill(0, slot_t, 0) if ctx.needs_input_grad[0] else None
        dw = torch.empty_like(weights)
        dg = torch.empty_like(gates)
        dc = torch.empty_like(coeff)
        depth, width = grad_out.shape
        _lib.check(_lib.load().dgb_three_tap_vjp(
            _lib.dtype_code(grad_out.dtype), grad_out.data_ptr(), depth, width,
            slot_t.data_ptr(), weights.numel(), _ptr(weights), _ptr(gates), _ptr(coeff),
            _ptr(offsets), _ptr(post_idx), dw.data_ptr(), dg.data_ptr(), dc.data_ptr(),
            _lib.stream_ptr(grad_out.device)), "dgb_three_tap_vjp")
        need = ctx.needs_input_grad
        return (gq, None, dw if need[2] else None, dg if need[3] else None,
                dc if need[4] else None, None, None, None)


def ordered_two_tap_enqueue(queue, slot, weights, gates, fraction, lower, upper):
    """New queue: row ``slot`` cleared, then ``(w g)(1-f)`` at every lower address
    (edge order) and ``(w g) f`` at every upper address (edge order)."""
    _prepare(queue, weights, gates, fraction, lower, upper, None)
    slot_t = _slot_tensor(slot, queue.shape[0], queue.device)
    plan = two_tap_plan(queue.shape[0], queue.shape[1], lower, upper)
    return _TwoTapEnqueue.apply(queue, slot_t, weights, gates, fraction, lower, upper, None,
                                plan)


def ordered_two_tap_enqueue_from_source(queue, slot, weights, gates, fraction, lower, upper,
                                        pre_idx):
    """As :func:`ordered_two_tap_enqueue` with edge e's gate ``gates[pre_idx[e]]``."""
    _prepare(queue, weights, gates, fraction, lower, upper, pre_idx)
    slot_t = _slot_tensor(slot, queue.shape[0], queue.device)
    plan = two_tap_plan(queue.shape[0], queue.shape[1], lower, upper, pre_idx, gates.numel())
    return _TwoTapEnqueue.apply(queue, slot_t, weights, gates, fraction, lower, upper, pre_idx,
                                plan)


def ordered_two_tap_enqueue_(queue, slot, weights, gates, fraction, lower, upper,
                             pre_idx=None, payload=None):
    """In-place form (no autograd).  ``payload`` (optional, ``width``) receives
    row ``slot`` before it is cleared."""
    _prepare(queue, weights, gates, fraction, lower, upper, pre_idx)
    if not queue.is_contiguous():
        raise RuntimeError("The private two-tap queue must be contiguous")
    slot_t = _slot_tensor(slot, queue.shape[0], queue.device)
    plan = two_tap_plan(queue.shape[0], queue.shape[1], lower, upper, pre_idx,
                        gates.numel() if pre_idx is not None else 0)
    with torch.no_grad():
        _enqueue_into(queue, slot_t, weights, gates, fraction, lower, upper, pre_idx, plan,
                      payload)
    return queue


def ordered_two_tap_enqueue_from_source_(queue, slot, weights, gates, fraction, lower, upper,
                                         pre_idx, payload=None):
    return ordered_two_tap_enqueue_(queue, slot, weights, gates, fraction, lower, upper,
                                    pre_idx, payload)


def delay_ring_gather_two_tap(ring, offset, lower, upper):
    """(ring[(lower + offset) mod size], ring[(upper + offset) mod size])."""
    if not (ring.is_cuda and ring.dim() == 2 and ring.numel() > 0 and ring.is_contiguous()
            and ring.dtype in (torch.float32, torch.float64)):
        raise RuntimeError("Two-tap gather requires a nonempty contiguous CUDA float matrix")
    off = offset if isinstance(offset, torch.Tensor) and offset.is_cuda else torch.tensor(
        [int(offset)], dtype=torch.int64, device=ring.device)
    lo = torch.empty(lower.numel(), dtype=ring.dtype, device=ring.device)
    hi = torch.empty_like(lo)
    _lib.check(_lib.load().dgb_two_tap_gather(
        _lib.dtype_code(ring.dtype), ring.data_ptr(), ring.numel(), off.data_ptr(),
        lower.numel(), _ptr(lower), _ptr(upper), lo.data_ptr(), hi.data_ptr(),
        _lib.stream_ptr(ring.device)), "dgb_two_tap_gather")
    return lo, hi


def delay_ring_two_tap_vjp(ring, offset, weights, gates, fraction, lower, upper,
                           source_indices=None):
    """(grad_weights, grad_gates, grad_fraction) at ring cotangent ``ring``."""
    if not (ring.is_cuda and ring.dim() == 2 and ring.numel() > 0 and ring.is_contiguous()):
        raise RuntimeError("Two-tap VJP requires a nonempty contiguous CUDA float matrix")
    _prepare(ring, weights, gates, fraction, lower, upper, source_indices)
    off = offset if isinstance(offset, torch.Tensor) and offset.is_cuda else torch.tensor(
        [int(offset)], dtype=torch.int64, device=ring.device)
    plan = two_tap_plan(ring.shape[0], ring.shape[1], lower, upper, source_indices,
                        gates.numel() if source_indices is not None else 0)
    return _vjp(ring, off.reshape(1), weights, gates, fraction, lower, upper, source_indices,
                plan)


def dense_interpolated_delay_transition(queue, slot, global_step, weights, connection_gates,
                                        delays, dt, *, post_idx, depth, width, taps, sigma,
                                        delay_taps=None, _clone_once=False):
    """One interpolated transition: the returned queue has row ``slot`` cleared
    and every connection's ``w g`` split over its taps (two: floor / floor+1 by
    the fractional position; three: Gaussian weights around the floor).  Today's
    row must be read (``queue[slot]``) before this call.  Returns a
    :class:`DenseTransition` with the slot and step advanced by one."""
    if delay_taps is None:
        delay_taps = delay_interpolation(delays, dt, dtype=queue.dtype, taps=taps, sigma=sigma)
    offsets, shares = delay_taps
    _check_queue(queue)
    if tuple(queue.shape) != (depth, width):
        raise RuntimeError("queue must have shape (depth, width)")
    slot_t = _slot_tensor(slot, depth, queue.device)
    plan = post_plan(depth, width, post_idx)
    if taps == 2:
        lower = offsets.remainder(depth) * width + post_idx
        upper = (lower + width).remainder(depth * width)
        _check_vec(weights, queue.dtype, lower.numel(), "weights", queue.device)
        _check_vec(connection_gates, queue.dtype, lower.numel(), "gates", queue.device)
        frac = shares.contiguous()
        nxt = _TwoTapEnqueue.apply(queue, slot_t, weights, connection_gates, frac,
                                   lower.contiguous(), upper.contiguous(), None, plan)
    else:
        nxt = _ThreeTapEnqueue.apply(queue, slot_t, weights, connection_gates,
                                     shares.contiguous(), offsets.contiguous(), post_idx, plan)
    gs = global_step + 1 if isinstance(global_step, torch.Tensor) else int(global_step) + 1
    return DenseTransition(nxt, (slot_t + 1).remainder(depth), gs, None)


# ---------------------------------------------------------------------------
# multi-step rollout
# ---------------------------------------------------------------------------
# Optional launch timing: while ``launch_events`` is a list, every rollout
# launch appends (name, start event, end event) recorded on its stream (the
# reverse launch covers the sweep and the per-source sum).
launch_events = None


class _Timed:
    def __init__(self, name, dev):
        self.name, self.dev = name, dev

    def __enter__(self):
        if launch_events is not None:
            self.e0 = torch.cuda.Event(enable_timing=True)
            self.e0.record(torch.cuda.current_stream(self.dev))
        return self

    def __exit__(self, *exc):
        if launch_events is not None:
            e1 = torch.cuda.Event(enable_timing=True)
            e1.record(torch.cuda.current_stream(self.dev))
            launch_events.append((self.name, self.e0, e1))


# gate-cotangent scratch per reverse-sweep launch (the sweep is split into
# launches of at most this many bytes of per-edge gate cotangents)
_SCRATCH_BYTES = 4 << 30
# DGB_ROLLOUT_* flags
ONE_EDGE, EMPTY_START, NO_FINAL, CHAINED, GATES_BY_SOURCE = 1, 2, 4, 8, 16


class RolloutPlan:
    """Tap rows per list position of a consistent plan, for the rollout kernels.

    ``lo_row/hi_row[j]`` are the row distances of the two taps of the edge at
    position j of the column lists; ``src_pos`` lists each source's edges
    (ascending by edge) as list positions; ``flags`` marks plans with at most
    one edge per column.
    """

    def __init__(self, plan, lower, upper):
        W, E = plan.width, plan.n_edges
        dev = plan.col_ptr.device
        edge = plan.col_edge
        self.lo_row = (lower[edge] // W).to(torch.int32).contiguous()
        self.hi_row = (upper[edge] // W).to(torch.int32).contiguous()
        counts = plan.col_ptr[1:] - plan.col_ptr[:-1]
        self.flags = ONE_EDGE if (E == 0 or int(counts.max()) <= 1) else 0
        # every edge's taps at lo and lo + 1 with 1 <= lo <= depth - 2: each
        # delivered value is a closed form of two gates (the direct kernels)
        D = plan.depth
        if self.flags & ONE_EDGE and (E == 0 or bool(
                ((self.lo_row >= 1) & (self.lo_row <= D - 2)
                 & (self.hi_row == self.lo_row + 1)).all())):
            self.flags |= CHAINED
        self.src_ptr = self.src_pos = None
        if plan.src_ptr is not None:
            pos = torch.empty(E, dtype=torch.int64, device=dev)
            pos[edge] = torch.arange(E, device=dev)
            self.src_ptr = plan.src_ptr
            self.src_pos = pos[plan.src_edge].contiguous()


class _TwoTapRollout(torch.autograd.Function):
    """(payload[n][width], final queue) of n two-tap steps from ``queue0``
    (None: an empty ring)."""

    @staticmethod
    def forward(ctx, queue0, slot_t, weights, gates, fraction, pre_idx, plan, rp, shape):
        n = gates.shape[0]
        depth, width = shape
        dev, dt = weights.device, weights.dtype
        flags = rp.flags
        if queue0 is None:
            ring = torch.empty(depth, width, dtype=dt, device=dev)
            flags |= EMPTY_START
        else:
            ring = queue0.clone(memory_format=torch.contiguous_format)
        payload = torch.empty(n, width, dtype=dt, device=dev)
        g_use, g_row, gates_t = gates, 0, None
        if pre_idx is not None and flags & CHAINED and gates.numel():
            # per-source rows: a column's consecutive steps share cache sectors
            g_row = (n + 7) // 8 * 8
            gates_t = torch.empty(gates.shape[1], g_row, dtype=dt, device=dev)
            _lib.check(_lib.load().dgb_gates_by_source(
                _lib.dtype_code(dt), n, gates.shape[1], gates.data_ptr(), gates_t.data_ptr(),
                g_row, _lib.stream_ptr(dev)), "dgb_gates_by_source")
            g_use, flags = gates_t, flags | GATES_BY_SOURCE
        with _Timed("two_tap_rollout", dev):
            _lib.check(_lib.load().dgb_two_tap_rollout(
                _lib.dtype_code(dt), ring.data_ptr(), depth, width, slot_t.data_ptr(), n,
                plan.n_edges, _ptr(weights), _ptr(g_use), g_row, _ptr(pre_idx),
                plan.n_sources if pre_idx is not None else 0, _ptr(fraction),
                plan.col_ptr.data_ptr(), _ptr(plan.col_edge), _ptr(rp.lo_row),
                _ptr(rp.hi_row), flags, payload.data_ptr(), _lib.stream_ptr(dev)),
                "dgb_two_tap_rollout")
        ctx.save_for_backward(slot_t, weights, gates, fraction,
                              *(() if pre_idx is None else (pre_idx,)))
        ctx.plan, ctx.rp = plan, rp
        ctx.gates_t, ctx.g_row = gates_t, g_row
        ctx.has_queue0 = queue0 is not None
        # an unused output's cotangent stays None (no zero ring to read back)
        ctx.set_materialize_grads(False)
        return payload, ring

    @staticmethod
    def backward(ctx, grad_payload, grad_final):
        slot_t, weights, gates, fraction, *rest = ctx.saved_tensors
        pre_idx = rest[0] if rest else None
        plan, rp = ctx.plan, ctx.rp
        n = gates.shape[0]
        depth, width = plan.depth, plan.width
        dev, dt = weights.device, weights.dtype
        flags = rp.flags
        if grad_final is None:
            R = torch.empty(depth, width, dtype=dt, device=dev)
            empty = True
        else:
            R = grad_final.clone(memory_format=torch.contiguous_format)
            empty = False
        gp = None if grad_payload is None else grad_payload.contiguous()
        dw = torch.zeros_like(weights)
        df = torch.zeros_like(fraction)
        dgates = torch.empty_like(gates)
        E = plan.n_edges
        chunk = n
        scratch = None
        if pre_idx is not None and E:
            chunk = max(8, min(n, _SCRATCH_BYTES // (E * weights.element_size())) // 8 * 8)
            # one row of chunk (rounded up to 8) steps per list position
            scratch = torch.empty(E * ((chunk + 7) // 8 * 8), dtype=dt, device=dev)
        L = _lib.load()
        stream = _lib.stream_ptr(dev)
        gates_t, g_row = ctx.gates_t, ctx.g_row
        if gates_t is not None:
            flags |= GATES_BY_SOURCE
        hi = n
        while hi > 0:  # newest chunk first; the cotangent ring carries between chunks
            lo = max(0, hi - chunk)
            s_lo = (slot_t + lo).remainder(depth)
            g_ptr = (gates_t.data_ptr() + lo * gates_t.element_size() if gates_t is not None
                     else gates[lo:hi].data_ptr())
            with _Timed("two_tap_rollout_vjp", dev):
                _lib.check(L.dgb_two_tap_rollout_vjp(
                    _lib.dtype_code(dt), R.data_ptr(), depth, width, s_lo.data_ptr(), hi - lo, E,
                    _ptr(weights), g_ptr, g_row, _ptr(pre_idx),
                    plan.n_sources if pre_idx is not None else 0, _ptr(fraction),
                    plan.col_ptr.data_ptr(), _ptr(plan.col_edge), _ptr(rp.lo_row), _ptr(rp.hi_row),
                    flags | (EMPTY_START if empty else 0), _ptr(rp.src_ptr), _ptr(rp.src_pos),
                    None if gp is None else gp[lo:hi].data_ptr(), 0 if hi == n else 1,
                    dw.data_ptr(), dgates[lo:hi].data_ptr(), df.data_ptr(), _ptr(scratch), stream),
                    "dgb_two_tap_rollout_vjp")
            empty = False
            hi = lo
        if n == 0 and empty:
            R.zero_()
        return (R if ctx.has_queue0 else None), None, dw, dgates, df, None, None, None, None


def two_tap_rollout(queue0, slot, weights, gates, fraction, lower, upper, pre_idx=None,
                    depth=None, width=None):
    """``n = gates.shape[0]`` two-tap steps from row ``slot`` in one launch.

    ``gates[k]`` are step k's gates (per source with ``pre_idx``, else per
    edge); returns ``(payload, queue)``: ``payload[k]`` is the row delivered at
    step k (``queue[slot_k]`` before the step), ``queue`` the ring after the
    last step.  ``queue0=None`` starts from an empty ring of shape
    ``(depth, width)``.  Differentiable in queue0, weights, gates and
    fraction; the backward runs the reverse sweep on the GPU.  Both taps of
    every edge must lie in one column (true for transition addresses
    ``off*width + post``).
    """
    if queue0 is not None:
        _check_queue(queue0)
        depth, width = queue0.shape
    elif depth is None or width is None:
        raise RuntimeError("two_tap_rollout needs queue0 or depth and width")
    depth, width = int(depth), int(width)
    if gates.dim() != 2:
        raise RuntimeError("rollout gates must be (n_steps, n_sources or n_edges)")
    n = weights.numel()
    dev, dt = weights.device, weights.dtype
    if not (weights.is_cuda and dt in (torch.float32, torch.float64)):
        raise RuntimeError("rollout weights must be a CUDA float32 or float64 vector")
    if queue0 is not None and (queue0.device != dev or queue0.dtype != dt):
        raise RuntimeError("queue0 must match the weights' device and dtype")
    _check_vec(weights, dt, n, "weights", dev)
    _check_vec(fraction, dt, n, "fraction", dev)
    _check_vec(lower, torch.int64, n, "lower", dev)
    _check_vec(upper, torch.int64, n, "upper", dev)
    if pre_idx is not None:
        _check_vec(pre_idx, torch.int64, n, "source indices", dev)
    elif gates.shape[1] != n:
        raise RuntimeError("gates must have one column per edge without pre_idx")
    if not (gates.device == dev and gates.dtype == dt):
        raise RuntimeError("gates must match the weights' device and dtype")
    gates = gates.contiguous()
    slot_t = _slot_tensor(slot, depth, dev)
    plan = two_tap_plan(depth, width, lower, upper, pre_idx,
                        gates.shape[1] if pre_idx is not None else 0)
    if not plan.consistent:
        raise RuntimeError("two_tap_rollout needs both taps of every edge in one column")
    if getattr(plan, "rollout", None) is None:
        plan.rollout = RolloutPlan(plan, lower, upper)
    return _TwoTapRollout.apply(queue0, slot_t, weights, gates, fraction, pre_idx, plan,
                                plan.rollout, (depth, width))


def transition_addresses(offsets, post_idx, depth, width):
    """Flat (lower, upper) addresses of the two-tap transition."""
    lower = offsets.remainder(depth) * width + post_idx
    return lower.contiguous(), (lower + width).remainder(depth * width).contiguous()
