"""Event transport (NetCon) on the GB300 kernels.

Host mirrors of the reference's NetCon pieces, with every per-step operation
on the GPU and deterministic (no floating-point atomics):

* :func:`inference_delay_steps` — delay quantisation, round-half-even with a
  one-step minimum (networks/netcon.py:2760-2795)
* :func:`pack_source_spikes`, :func:`build_delivery` — the bit-packed history
  path (networks/netcon_bitpack_ops.py:590-712, netcon_bitpack_kernel.cpp:145-149);
  connections are re-ordered by target once (cached) so each target is summed
  by one thread in connection order
* :class:`DenseRing` — the dense delay ring of dense_fixed_delay_transition
  (networks/_event_delivery.py:30-199): deliver today's row, clear it,
  enqueue weight * gate at (slot + delay) % depth, advance the slot
* :func:`detect_spikes` — rising-edge detection (networks/spiking.py:7-73)
* :func:`exp2syn_factor` — Exp2Syn peak normalisation (mod/EXP2SYN.py:112-144)
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib
from ._cache import TensorKeyedCache

BITS_PER_WORD = 63


def inference_delay_steps(delay_ms, dt_ms):
    """(delay_steps, inference_delay_steps): round-half-even of delay/dt, then >= 1."""
    ratio = torch.as_tensor(delay_ms, dtype=torch.float64) / float(dt_ms)
    steps = torch.round(ratio).to(torch.int64)  # torch.round is round-half-even
    return steps, steps.clamp_min(1)


def exp2syn_factor(tau1, tau2):
    """Exp2Syn weight normalisation with tau1/tau2 clamped to [1e-9, 0.9999]."""
    tau1 = torch.as_tensor(tau1, dtype=torch.float64)
    tau2 = torch.as_tensor(tau2, dtype=torch.float64)
    if not bool((torch.isfinite(tau1) & torch.isfinite(tau2) & (tau1 > 0) & (tau2 > 0)).all()):
        raise ValueError("exp2syn tau1 and tau2 must be positive and finite.")
    ratio = (tau1 / tau2).clamp(1.0e-9, 0.9999)
    log_den = torch.log1p(-ratio) + ratio / (1 - ratio) * torch.log(ratio)
    return torch.exp(-log_den)


def n_words_for(n_source: int) -> int:
    return max(1, -(-int(n_source) // BITS_PER_WORD))


def source_word_and_mask(pre_idx):
    """Word index and bit mask of each connection's source in the packed history."""
    pre = torch.as_tensor(pre_idx, dtype=torch.int64)
    return pre // BITS_PER_WORD, torch.ones_like(pre) << (pre % BITS_PER_WORD)


def detect_spikes(v, below, thr=0.0, comp=None):
    """spikes = (v[comp] >= thr) & below; below <- ~(v[comp] >= thr).  uint8 tensors."""
    n = below.numel()
    spikes = torch.empty(n, dtype=torch.uint8, device=v.device)
    with torch.cuda.device(v.device):
        rc = _lib.load().dgb_detect_spikes(
            _lib.dtype_code(v.dtype), v.data_ptr(), None if comp is None else comp.data_ptr(), n,
            float(thr), below.data_ptr(), spikes.data_ptr(), _lib.stream_ptr(v.device))
    _lib.check(rc, "dgb_detect_spikes")
    return spikes


def pack_source_spikes(source_spikes, packed_history, current_time_step):
    """Write the source-spike bits into row current_time_step[0] of packed_history."""
    src = source_spikes.to(torch.uint8).contiguous()
    if packed_history.dtype != torch.int64 or not packed_history.is_contiguous():
        raise TypeError("packed_history must be a contiguous int64 CUDA tensor")
    n_words = packed_history.shape[-1]
    with torch.cuda.device(src.device):
        rc = _lib.load().dgb_pack_source_spikes(src.data_ptr(), src.numel(),
                                                packed_history.data_ptr(), n_words,
                                                current_time_step.data_ptr(),
                                                _lib.stream_ptr(src.device))
    _lib.check(rc, "dgb_pack_source_spikes")
    return packed_history


class TargetCSR:
    """Connections re-ordered by target (stable: connection order kept per target)."""

    def __init__(self, post_idx, n_post: int):
        post = torch.as_tensor(post_idx, dtype=torch.int64).cpu()
        self.perm = torch.argsort(post, stable=True)
        counts = torch.bincount(post, minlength=n_post)
        self.ptr = torch.zeros(n_post + 1, dtype=torch.int64)
        self.ptr[1:] = torch.cumsum(counts, 0)
        self.n_post = int(n_post)

    def to(self, device):
        self.perm = self.perm.to(device)
        self.ptr = self.ptr.to(device)
        return self


_csr_cache = TensorKeyedCache(32)


def _target_csr(post_idx, n_post):
    """Target CSR of a connection list, cached on the identity and version of
    ``post_idx`` (the entry holds it, so its address cannot be reused)."""
    return _csr_cache.get((post_idx,), int(n_post),
                          lambda: TargetCSR(post_idx, n_post).to(post_idx.device))


def build_delivery(packed_history, current_time_step, delay_steps, conn_word_idx,
                   conn_bit_mask, post_idx, weight, delivery_out):
    """Add each connection's delayed event weight to delivery_out[post_idx] (in place)."""
    csr = _target_csr(post_idx, delivery_out.numel())
    perm = csr.perm
    d = delay_steps.index_select(0, perm).contiguous()
    w_idx = conn_word_idx.index_select(0, perm).contiguous()
    mask = conn_bit_mask.index_select(0, perm).contiguous()
    w = weight.index_select(0, perm).contiguous()
    depth, n_words = packed_history.shape
    with torch.cuda.device(delivery_out.device):
        rc = _lib.load().dgb_build_delivery(
            _lib.dtype_code(delivery_out.dtype), packed_history.data_ptr(),
            current_time_step.data_ptr(), d.data_ptr(), w_idx.data_ptr(), mask.data_ptr(),
            csr.ptr.data_ptr(), csr.n_post, w.data_ptr(), delivery_out.data_ptr(), w.numel(),
            depth, n_words, _lib.stream_ptr(delivery_out.device))
    _lib.check(rc, "dgb_build_delivery")
    return delivery_out


def build_delivery_uniform(packed_history, current_time_step, delay_step, conn_word_idx,
                           conn_bit_mask, post_idx, weight, delivery_out):
    """build_delivery with the same delay (an int, in steps) for every connection
    (the reference's build_delivery_uniform, netcon_bitpack_ops.py:669-712)."""
    depth, n_words = packed_history.shape
    delay_step = int(delay_step)
    if not 0 <= delay_step < depth:
        raise ValueError(f"delay_step must lie in [0, {depth}) for this history")
    csr = _target_csr(post_idx, delivery_out.numel())
    perm = csr.perm
    w_idx = conn_word_idx.index_select(0, perm).contiguous()
    mask = conn_bit_mask.index_select(0, perm).contiguous()
    w = weight.index_select(0, perm).contiguous()
    with torch.cuda.device(delivery_out.device):
        rc = _lib.load().dgb_build_delivery_uniform(
            _lib.dtype_code(delivery_out.dtype), packed_history.data_ptr(),
            current_time_step.data_ptr(), delay_step, w_idx.data_ptr(), mask.data_ptr(),
            csr.ptr.data_ptr(), csr.n_post, w.data_ptr(), delivery_out.data_ptr(), w.numel(),
            depth, n_words, _lib.stream_ptr(delivery_out.device))
    _lib.check(rc, "dgb_build_delivery_uniform")
    return delivery_out


class DenseRing:
    """Dense delay ring [depth, width] with fixed per-connection delays.

    ``pre_idx`` (source of each connection), ``post_idx`` (target column),
    ``delay_steps`` (>= 1) and ``weight`` are fixed at construction; the
    connections are stored sorted by target once.
    """

    def __init__(self, depth, width, pre_idx, post_idx, delay_steps, weight, device="cuda",
                 dtype=torch.float64):
        self.depth, self.width = int(depth), int(width)
        dev = torch.device(device)
        post = torch.as_tensor(post_idx, dtype=torch.int64)
        csr = TargetCSR(post, self.width)
        perm = csr.perm
        d = torch.as_tensor(delay_steps, dtype=torch.int64)
        if d.numel() and (int(d.min()) < 1 or int(d.max()) >= self.depth):
            raise ValueError("delay_steps must lie in [1, depth)")
        self.ptr = csr.ptr.to(dev)
        self.pre = torch.as_tensor(pre_idx, dtype=torch.int64)[perm].to(dev).contiguous()
        self.delay = d[perm].to(dev).contiguous()
        self.weight = torch.as_tensor(weight, dtype=dtype)[perm].to(dev).contiguous()
        self.ring = torch.zeros(self.depth, self.width, dtype=dtype, device=dev)
        self.slot = torch.zeros(1, dtype=torch.int64, device=dev)
        self.dtype = dtype
        self.device = dev

    def due(self):
        """Today's row (a copy)."""
        return self.ring.index_select(0, self.slot).squeeze(0)

    def transition(self, source_gates):
        """Clear today's row, enqueue the gated events, advance the slot."""
        gates = source_gates.to(torch.uint8).contiguous()
        self.ring.index_fill_(0, self.slot, 0)
        with torch.cuda.device(self.device):
            rc = _lib.load().dgb_ring_enqueue(
                _lib.dtype_code(self.dtype), self.ring.data_ptr(), self.depth, self.width,
                self.slot.data_ptr(), self.ptr.data_ptr(), self.width, None,
                self.pre.data_ptr(), gates.data_ptr(), self.delay.data_ptr(),
                self.weight.data_ptr(), _lib.stream_ptr(self.device))
        _lib.check(rc, "dgb_ring_enqueue")
        self.slot.add_(1).remainder_(self.depth)
