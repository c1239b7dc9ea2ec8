"""Gradients of recorded cable traces through the hand-written adjoint kernels.

The reference differentiates a cable run with torch autograd through every
step of its eager update (integrators/implicit.py:569-664, the cnexp gate
step mechanisms/_cnexp.py:96-132, the HH rates mod/HH.py:24-40 and current
:109-116) and, on the GPU, the transpose solve of ThomasSolve.backward
(triton/t_kernel_thomas.py:147-189).  Here the same gradient comes from two
kernels per segment of ``checkpoint_every`` steps:

* ``dgb_cable_run_taped`` recomputes the segment from its checkpoint and
  writes the state tape (v, m, h, n after every step);
* ``dgb_cable_adjoint`` walks the segment backwards: transposed chunked
  tridiagonal solve, reverse of the membrane assembly and of the gate advance,
  accumulating dLoss/d(gnabar, gkbar, gl) per compartment and the axial term.

The forward pass keeps only the checkpoints (state every ``checkpoint_every``
steps) and the recorded trace.  ``cable_traces`` wraps both passes in a
``torch.autograd.Function`` whose inputs are per-cable gnabar, gkbar, gl and
Ra (the parameters a fit recovers) and whose output is the somatic trace.
"""

from __future__ import annotations

import ctypes

import torch

from . import _lib
from .cable import CablePopulation


class CableGradient:
    """Checkpointed forward and adjoint of a recorded trace of ``pop``.

    pop: an initialized CablePopulation (its state is the initial state of
    every forward; it is not modified).  rec_idx: local compartment recorded
    per cable (int or per-cable sequence).  The trace has one sample per step,
    (B, n_steps + 1), sample 0 being the initial state.  overlap: recompute
    the next segment on a side stream while the adjoint of the current one
    runs (two tapes in memory instead of one).  Off by default: with the
    bulk-staged adjoint the two kernels compete for shared memory on the SMs,
    and the serial order measured faster (1,024 cables × 201 compartments,
    20,000 steps: 247 vs 308 ms per backward pass).  A float32 population built
    with fast_math runs the forward, the recompute and the adjoint's gate
    partials and solve with the fast-math arithmetic.  tune: pick the
    forward and recompute runs' launch shape (cables per CTA or the
    split-gate run) by timing a short taped recompute, once per population
    shape (cached); this sets pop.warps_per_block and pop.split_gates.
    """

    def __init__(self, pop: CablePopulation, n_steps: int, rec_idx=0, checkpoint_every=500,
                 overlap=False, tune=True):
        if pop.dt is None:
            raise RuntimeError("Model must be initialized before running.")
        if n_steps < 1 or checkpoint_every < 1:
            raise ValueError("n_steps and checkpoint_every must be >= 1")
        self.pop = pop
        self.n_steps = int(n_steps)
        self.seg = int(min(checkpoint_every, n_steps))
        dev = pop.device
        kk = torch.as_tensor(pop.n_comp, dtype=torch.int32)
        rec = torch.as_tensor(rec_idx, dtype=torch.int32).expand(pop.B).contiguous()
        if bool(((rec < 0) | (rec >= kk)).any()):
            raise ValueError("rec_idx out of range for some cable")
        self.rec = rec.to(dev)
        self.state0 = tuple(t.clone() for t in (pop.v, pop.m, pop.h, pop.n))
        if tune:
            self._tune_launch()
        self.counts = torch.as_tensor(pop.n_comp, device=dev)
        self.comp_cable = pop._dev["comp_cable"].long()
        self.base_axial = (pop._dev["g_right"].clone(), pop._dev["g_left"].clone())
        first = torch.as_tensor(pop.cable_ptr_np[:-1], device=dev)
        self.rhoa0 = pop.rhoa.to(dev, torch.float64)[first]
        self.ra = self.rhoa0.clone()
        self.checkpoints = []
        self._tapes = []
        self.overlap = bool(overlap)
        if self.overlap:
            self._side = torch.cuda.Stream(dev)
            self._side_scratch = torch.zeros(4, dtype=torch.int32, device=dev)

    def _tune_launch(self):
        """Cables per CTA or the split-gate run for the forward and recompute
        runs, timed on what dominates them: a taped recompute of
        min(checkpoint_every, 50) steps from the initial state (cached per
        population shape)."""
        from .autotune import CABLE_RUN_SPLIT, tune

        pop = self.pop
        steps = min(self.seg, 50)
        L = _lib.load()
        bufs = {}  # tape and work state, made at the first timing (none when cached)

        def apply(c):
            pop.warps_per_block = max(int(c[0]), 0)
            pop.split_gates = int(c[0]) < 0

        def run(c):
            apply(c)
            if not bufs:
                bufs["tape"] = torch.empty((steps + 1, 4, pop.N), dtype=pop.dtype,
                                           device=pop.device)
                bufs["work"] = tuple(torch.empty_like(t) for t in self.state0)
            for w, s in zip(bufs["work"], self.state0):
                w.copy_(s)
            _lib.check(L.dgb_cable_run_taped(self._args(steps, 0, bufs["work"]),
                                             bufs["tape"].data_ptr(),
                                             _lib.stream_ptr(pop.device)), "dgb_cable_run_taped")

        cands = ((2, 0, 0), (4, 0, 0), CABLE_RUN_SPLIT)
        parts = (str(pop.dtype), pop.B, max(pop.n_comp), pop.N, pop.fast_math,
                 pop.uniform_geometry and pop.uniform_channels,
                 "ve" if pop.field is not None else "-", steps)
        with torch.cuda.device(pop.device):
            best, _ = tune("cable_gradient_launch", parts, cands, run, pop.device)
        apply(best)

    # -- parameters -------------------------------------------------------
    def set_params(self, gnabar=None, gkbar=None, gl=None, ra=None):
        """Per-cable values (B,) of the fitted parameters (None keeps the current)."""
        d = self.pop._dev
        for name, val in (("gnabar", gnabar), ("gkbar", gkbar), ("gl", gl)):
            if val is not None:
                d[name] = self._per_cable(val).to(self.pop.dtype)
        if ra is not None:
            ra = torch.as_tensor(ra, device=self.pop.device).to(torch.float64).reshape(-1)
            if ra.numel() != self.pop.B or bool((ra <= 0).any()):
                raise ValueError("ra must hold one positive value per cable")
            self.ra = ra.clone()
            kappa = (self.rhoa0 / ra)[self.comp_cable]
            gr0, gl0 = self.base_axial
            same = bool((ra == self.rhoa0).all())
            d["g_right"] = gr0.clone() if same else (gr0.double() * kappa).to(self.pop.dtype)
            d["g_left"] = gl0.clone() if same else (gl0.double() * kappa).to(self.pop.dtype)

    def _per_cable(self, val):
        val = torch.as_tensor(val, device=self.pop.device).reshape(-1)
        if val.numel() != self.pop.B:
            raise ValueError(f"expected {self.pop.B} per-cable values")
        return torch.repeat_interleave(val, self.counts)

    # -- passes -----------------------------------------------------------
    def _args(self, steps, step0, state, trace=None):
        a = self.pop._args(steps, 1)
        a.rec_idx = self.rec.data_ptr()
        a.trace = None if trace is None else trace.data_ptr()
        a.v, a.m, a.h, a.n = (t.data_ptr() for t in state)
        a.step0 = int(step0)
        return a

    def _segments(self):
        return [(k * self.seg, min(self.seg, self.n_steps - k * self.seg))
                for k in range((self.n_steps + self.seg - 1) // self.seg)]

    def forward(self):
        """Run all steps, keep the checkpoints, return the trace (B, n_steps + 1)."""
        pop = self.pop
        dev = pop.device
        L = _lib.load()
        state = tuple(t.clone() for t in self.state0)
        trace = torch.empty((pop.B, self.n_steps + 1), dtype=pop.dtype, device=dev)
        seg_trace = torch.empty((pop.B, self.seg + 1), dtype=pop.dtype, device=dev)
        self.checkpoints = []
        with torch.cuda.device(dev):
            for step0, steps in self._segments():
                self.checkpoints.append(tuple(t.clone() for t in state))
                buf = seg_trace[:, :steps + 1]
                if steps != self.seg:
                    buf = torch.empty((pop.B, steps + 1), dtype=pop.dtype, device=dev)
                args = self._args(steps, step0, state, buf)
                # the taped kernel without a tape: the checkpoints lie on the
                # trajectory the recompute reproduces bit for bit
                _lib.check(L.dgb_cable_run_taped(args, None, _lib.stream_ptr(dev)),
                           "dgb_cable_run_taped")
                trace[:, step0:step0 + steps + 1] = buf
        return trace

    def backward(self, grad_trace):
        """Per-cable gradients {gnabar, gkbar, gl, ra} for dLoss/dtrace (B, n_steps + 1)."""
        if not self.checkpoints:
            raise RuntimeError("backward() needs a forward() first")
        pop = self.pop
        dev = pop.device
        N, B = pop.N, pop.B
        gt = grad_trace.to(device=dev, dtype=pop.dtype).contiguous()
        if tuple(gt.shape) != (B, self.n_steps + 1):
            raise ValueError(f"grad_trace must be ({B}, {self.n_steps + 1})")
        segs = self._segments()
        nbuf = 2 if (self.overlap and len(segs) > 1) else 1
        if len(self._tapes) != nbuf or self._tapes[0].dtype != pop.dtype:
            self._tapes = [torch.empty((self.seg + 1, 4, N), dtype=pop.dtype, device=dev)
                           for _ in range(nbuf)]
        lam = torch.zeros((4, N), dtype=pop.dtype, device=dev)
        gcomp = torch.zeros((3, N), dtype=pop.dtype, device=dev)
        gax = torch.zeros(N, dtype=pop.dtype, device=dev)
        works = [tuple(torch.empty_like(t) for t in self.state0) for _ in range(nbuf)]
        adj = _lib.CableAdjointArgs()
        adj.trace_grad = gt.data_ptr()
        adj.trace_len = self.n_steps + 1
        adj.lam_v, adj.lam_m, adj.lam_h, adj.lam_n = (lam[i].data_ptr() for i in range(4))
        adj.grad_gnabar, adj.grad_gkbar, adj.grad_gl = (gcomp[i].data_ptr() for i in range(3))
        adj.grad_axial = gax.data_ptr()
        L = _lib.load()
        main = torch.cuda.current_stream(dev)
        # recompute runs on a side stream with its own work counter, so the
        # recompute of segment k - 1 overlaps the adjoint of segment k (each
        # kernel alone keeps only one warp per cable busy)
        side = self._side if nbuf == 2 else main
        rec_done = [torch.cuda.Event() for _ in range(nbuf)]
        adj_done = [torch.cuda.Event() for _ in range(nbuf)]
        used = [False] * nbuf
        err = torch.zeros(1, dtype=torch.int32, device=dev)
        scratch = pop._dev["scratch"]
        side_err = [torch.zeros(1, dtype=torch.int32, device=dev) for _ in range(nbuf)]

        def recompute(k):
            b = k % nbuf
            step0, steps = segs[k]
            with torch.cuda.stream(side):
                if used[b]:
                    side.wait_event(adj_done[b])
                for w, c in zip(works[b], self.checkpoints[k]):
                    w.copy_(c)
                args = self._args(steps, step0, works[b])
                if nbuf == 2:
                    args.scratch = self._side_scratch.data_ptr()
                _lib.check(L.dgb_cable_run_taped(args, self._tapes[b].data_ptr(),
                                                 side.cuda_stream), "dgb_cable_run_taped")
                if nbuf == 2:
                    side_err[b].copy_(self._side_scratch[1:2])
                else:
                    err.bitwise_or_(scratch[1:2])
                rec_done[b].record(side)

        with torch.cuda.device(dev):
            if nbuf == 2:
                side.wait_stream(main)
            last = len(segs) - 1
            if nbuf == 2:
                recompute(last)
            for k in range(last, -1, -1):
                b = k % nbuf
                if nbuf == 2 and k >= 1:
                    recompute(k - 1)
                elif nbuf == 1:
                    recompute(k)
                main.wait_event(rec_done[b])
                step0, steps = segs[k]
                adj.tape = self._tapes[b].data_ptr()
                args = self._args(steps, step0, works[b])
                _lib.check(L.dgb_cable_adjoint(args, ctypes.byref(adj), main.cuda_stream),
                           "dgb_cable_adjoint")
                err.bitwise_or_(scratch[1:2])
                if nbuf == 2:
                    err.bitwise_or_(side_err[b])
                adj_done[b].record(main)
                used[b] = True
            if nbuf == 2:
                main.wait_stream(side)
        # a cable the kernels could not process, or a tape-stage wait that gave
        # up, leaves error bits in the launch's work counter (each launch resets
        # it): they were gathered after every launch, checked once here
        bits = int(err.item())
        if bits:
            raise RuntimeError(f"dgb_cable_adjoint / dgb_cable_run_taped reported error bits "
                               f"{bits:#x}")
        # per-compartment results, kept for inspection: adjoint of the initial
        # state (v, m, h, n), dLoss/d(gnabar, gkbar, gl) and the axial term
        self.lam0, self.grad_comp, self.grad_axial = lam, gcomp, gax
        per = self._per_cable_sum(torch.cat([gcomp, gax[None]]))
        return {"gnabar": per[0], "gkbar": per[1], "gl": per[2], "ra": -per[3] / self.ra}

    def _per_cable_sum(self, x):
        """Deterministic float64 sums of (R, N) per-compartment rows over each cable."""
        x = x.double()
        ks = self.pop.n_comp
        if min(ks) == max(ks):
            return x.reshape(x.shape[0], self.pop.B, ks[0]).sum(dim=2)
        cs = torch.nn.functional.pad(torch.cumsum(x, dim=1), (1, 0))
        ptr = torch.as_tensor(self.pop.cable_ptr_np, device=x.device)
        return cs[:, ptr[1:]] - cs[:, ptr[:-1]]


class _TraceFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, gnabar, gkbar, gl, ra, runner):
        runner.set_params(gnabar.detach(), gkbar.detach(), gl.detach(), ra.detach())
        ctx.runner = runner
        ctx.dtypes = tuple(t.dtype for t in (gnabar, gkbar, gl, ra))
        return runner.forward()

    @staticmethod
    def backward(ctx, grad_trace):
        g = ctx.runner.backward(grad_trace)
        out = tuple(g[k].to(dt) for k, dt in zip(("gnabar", "gkbar", "gl", "ra"), ctx.dtypes))
        return (*out, None)


def cable_traces(runner: CableGradient, gnabar, gkbar, gl, ra):
    """Recorded traces (B, n_steps + 1) as a differentiable function of the
    per-cable gnabar, gkbar, gl (S/cm^2) and Ra (ohm cm)."""
    return _TraceFunction.apply(gnabar, gkbar, gl, ra, runner)
