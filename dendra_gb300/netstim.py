"""NetStim renewal generators on the GPU.

Mirror of the reference's NetStim (networks/netstim.py) for the renewal
process that drives network background input: ``N`` independent generators
with mean interval ``interval`` (ms), ``noise`` mixing periodic and Poisson
intervals (``(1 - noise) interval + noise interval E``, E unit exponential),
a first clock ``start + noise interval E`` (or ``start`` when no generator
has noise) and at most ``number`` spikes.  Every step applies the reference's
transition (networks/_netstim_renewal.py:94-159): a generator whose clock is
due (``t >= next``) and below its cap fires and advances its clock by a fresh
interval; a draw is consumed every step.  Time is ``t0 + step * dt`` in the
state dtype, the network's exact clock.

Draws come from a counter-based generator on the device (Philox4x32-10 keyed
by ``seed``, counter = step and generator), so a run split at any step
continues identically and needs no stored generator state; a table of draws
may be supplied instead (how the parity tests reproduce the reference).  The
surrogate gradient of the reference's straight-through gate is not provided:
these generators produce events.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib


class NetStim:
    """``N`` renewal generators.

    Parameters broadcast to ``(N,)``: ``interval`` (ms), ``noise`` in
    [0, 1], ``start`` (ms), ``number`` (spike cap; None = unlimited).
    """

    def __init__(self, N, interval=10.0, noise=0.0, start=0.0, number=None, seed=0,
                 dtype=torch.float32, device="cuda"):
        self.N = int(N)
        self.dtype, self.device = dtype, torch.device(device)

        def vec(x, dt):
            return torch.broadcast_to(torch.as_tensor(x, dtype=dt), (self.N,)).to(
                self.device).contiguous()

        self.interval = vec(interval, dtype)
        self.noise = vec(noise, dtype)
        self.start = vec(start, dtype)
        self.number = None if number is None else vec(number, torch.int64)
        if bool((self.noise < 0).any()) or bool((self.noise > 1).any()):
            raise ValueError("noise must lie in [0, 1]")
        self.seed = int(seed) & ((1 << 64) - 1)
        self.next_stoch_time = torch.empty(self.N, dtype=dtype, device=self.device)
        self.spike_counts = torch.zeros(self.N, dtype=torch.int64, device=self.device)
        self.step = 0
        self.initialize()

    def initialize(self, draws=None):
        """Reset clocks (netstim_initial_state) and counts; step 0."""
        any_noise = int(bool((self.noise > 0).any()))
        d = None if draws is None else torch.as_tensor(draws, dtype=self.dtype).to(
            self.device).contiguous()
        _lib.check(_lib.load().dgb_netstim_init(
            _lib.dtype_code(self.dtype), self.N, self.interval.data_ptr(),
            self.noise.data_ptr(), self.start.data_ptr(), any_noise, self.seed,
            None if d is None else d.data_ptr(), self.next_stoch_time.data_ptr(),
            self.spike_counts.data_ptr(), _lib.stream_ptr(self.device)), "dgb_netstim_init")
        self.step = 0
        return self

    def run(self, n_steps, dt, t0=0.0, draws=None, spikes=True, bits=False):
        """Advance ``n_steps`` steps of ``dt`` ms from the current step.

        Returns ``spikes`` (uint8 ``(n_steps, N)``) and/or ``bits`` (int64
        ``(n_steps, ceil(N/64))``, bit ``g % 64`` of word ``g // 64``) as
        requested; ``draws`` (optional) is a ``(n_steps, N)`` table of unit
        exponentials used instead of the device generator.
        """
        n_steps = int(n_steps)
        words = max(1, -(-self.N // 64))
        spk = (torch.empty(n_steps, self.N, dtype=torch.uint8, device=self.device)
               if spikes else None)
        bit = (torch.empty(n_steps, words, dtype=torch.int64, device=self.device)
               if bits else None)
        d = None
        if draws is not None:
            d = torch.as_tensor(draws, dtype=self.dtype).to(self.device).contiguous()
            if tuple(d.shape) != (n_steps, self.N):
                raise ValueError("draws must have shape (n_steps, N)")
        _lib.check(_lib.load().dgb_netstim_run(
            _lib.dtype_code(self.dtype), self.N, n_steps, self.step, float(t0), float(dt),
            self.interval.data_ptr(), self.noise.data_ptr(),
            None if self.number is None else self.number.data_ptr(), self.seed,
            None if d is None else d.data_ptr(), self.next_stoch_time.data_ptr(),
            self.spike_counts.data_ptr(), None if spk is None else spk.data_ptr(),
            None if bit is None else bit.data_ptr(), words, _lib.stream_ptr(self.device)),
            "dgb_netstim_run")
        self.step += n_steps
        if spikes and bits:
            return spk, bit
        return spk if spikes else bit


def spike_steps(spikes):
    """Per generator, the steps at which it fired (host lists)."""
    s = spikes.cpu().numpy() if isinstance(spikes, torch.Tensor) else np.asarray(spikes)
    return [np.flatnonzero(s[:, g]) for g in range(s.shape[1])]
