"""Unbranched Hodgkin–Huxley cable populations on the GB300 kernels.

The host side of the reference path

    dn.Unmyelinated(diameters, L, dx, ...)  .insert(hh)  integrator=dn.bwd_euler_ub()
    model[..., i].inject(dn.mono_rect(...));  model.run(extra=(point_field, mono_rect))

restated for a packed ragged population: cables of different compartment
counts are stored back to back (``cable_ptr``), and one ``run`` call advances
every cable by ``n_steps`` backward-Euler steps in a single persistent kernel
launch (``dgb_cable_run``).  ``step_plain`` advances one step through the
unfused kernel pair (``dgb_cable_assemble`` + ``dgb_cable_solve_update``).

Workspace preparation follows the reference arithmetic in the state dtype:
  area      models/core.py:2028           diam*1e-4*pi*dx*1e-4
  g_edge    integrators/cable.py:18-29    2/(R_i + R_{i+1}),  R = Ra*L/(pi r^2)
  workspace integrators/implicit.py:484-522
  gates     mod/HH.py:42-56               steady state at v_init
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib

# mod/HH.py:100 defaults.  The reference stores mechanism GLOBALs as float32
# values (widened in float64 models), so the effective defaults are the
# float32-rounded numbers in both precisions.
HH_DEFAULTS = {k: float(np.float32(v)) for k, v in
               dict(gnabar=0.12, gkbar=0.036, gl=0.0003, ena=50.0, ek=-77.0, el=-54.3).items()}
# gate rate constants am1, ah1, an1 (HH.py:20), float32-rounded for the same reason
AM1, AH1, AN1 = (float(np.float32(x)) for x in (0.1, 0.07, 0.01))


def q10_of(celsius: float) -> float:
    """Temperature factor 3**((celsius - 6.3)/10) (mod/HH.py:21-22)."""
    return 3.0 ** ((celsius - 6.3) / 10.0)


def dt_seconds(dt_ms: float, dtype) -> float:
    """dt*1e-3 rounded in the state dtype, as the reference forms it."""
    if dtype == torch.float32:
        return float(np.float32(np.float32(dt_ms) * np.float32(1.0e-3)))
    return float(np.float64(dt_ms) * 1.0e-3)


def membrane_area(diam, dx):
    """Lateral cylinder area in cm^2 (models/core.py:2028)."""
    return diam * 1e-4 * torch.pi * dx * 1e-4


def cylindrical_edge_conductance(diam, dx, rhoa):
    """Centre-to-centre conductance of adjoining cylinders (cable.py:18-29)."""
    radius_cm = 1.0e-4 * diam / 2.0
    length_cm = 1.0e-4 * dx
    seg = rhoa * length_cm / (torch.pi * radius_cm.square())
    return 2.0 / (seg[:-1] + seg[1:])


def point_source_field(x_um, y_um, z_um, src=(0.0, 0.0, 0.0), rhoe=300.0):
    """Isotropic point-source lead field in mV/mA (fields/analytic.py:60-62)."""
    r = torch.sqrt((x_um - src[0]) ** 2 + (y_um - src[1]) ** 2 + (z_um - src[2]) ** 2) * 1e-4
    return rhoe / (4 * torch.pi * r)


def unmyelinated_positions(K: int, dx: float, dtype=torch.float32):
    """Compartment centres of an Unmyelinated cable (models/core.py:10950-10953)."""
    length = (K - 1) * dx
    return torch.linspace(-length / 2, length / 2, K, dtype=dtype)


def waveform_param(x):
    """A waveform parameter as the reference holds it.

    Python numbers given to a waveform (``mono_rect(delay=1.0, pw=0.1)``) are
    stored by the reference as float32 values and widened on use, so a pulse
    of pw=0.1 ms ends at 1.0 + float32(0.1) even in a float64 model.  Tensors
    keep their own values.
    """
    if isinstance(x, (bool, int, float, np.floating, np.integer)):
        return torch.tensor(float(np.float32(x)), dtype=torch.float64)
    return torch.as_tensor(x)


@dataclass
class RasterState:
    """Upward threshold crossings at checked compartments (Raster/APCount).

    idx (B, R) int32 local compartments (-1: none); below (B, R) int32 latch
    (1 = below threshold); count (B, R) int32 crossings counted so far; steps
    (B, R, cap) int64 absolute step index (1-based, counted from
    initialize) of each crossing while its ordinal is below cap, -1 after.
    A count above cap means later crossings were counted but not stored.
    Pass it back as ``raster_state`` to continue counting in a later run."""

    idx: torch.Tensor
    below: torch.Tensor
    count: torch.Tensor
    steps: torch.Tensor

    @property
    def overflow(self) -> bool:
        return bool((self.count > self.steps.shape[-1]).any())

    def spike_steps(self, cable: int, q: int = 0):
        """The stored crossing steps of one cable's check q (a numpy array)."""
        c = int(self.count[cable, q])
        return self.steps[cable, q, :min(c, self.steps.shape[-1])].cpu().numpy()


@dataclass
class RunResult:
    trace: torch.Tensor | None
    spk_count: torch.Tensor | None
    spk_first: torch.Tensor | None
    trace_all: torch.Tensor | None = None
    raster: RasterState | None = None


class CablePopulation:
    """A packed population of unbranched HH cables.

    Parameters
    ----------
    n_comp : sequence of int
        Compartments per cable (each 1..512).
    diam, dx : float or sequence
        Per-cable diameter (um) and compartment length (um), or per-compartment
        packed arrays of length ``sum(n_comp)``.
    rhoa : float or sequence
        Axial resistivity (ohm cm): scalar, per cable or per compartment.
    cm : float or sequence
        Specific capacitance (uF/cm^2), scalar or per compartment.
    celsius, v_init : float
    dtype : torch.float32 or torch.float64
    hh : dict, optional
        Per-compartment or scalar overrides of gnabar, gkbar, gl, el (ena and
        ek are scalars).
    """

    def __init__(self, n_comp, diam, dx, *, rhoa=100.0, cm=1.0, celsius=6.3, v_init=-65.0,
                 dtype=torch.float32, device="cuda", hh=None, fast_math=False,
                 compress_uniform=True):
        n_comp = [int(k) for k in n_comp]
        if not n_comp:
            raise ValueError("a population needs at least one cable")
        if min(n_comp) < 1 or max(n_comp) > 1024:
            raise ValueError("compartments per cable must be in [1, 1024]")
        if dtype not in (torch.float32, torch.float64):
            raise TypeError("state dtype must be float32 or float64")
        self.dtype = dtype
        self.device = torch.device(device)
        self.n_comp = n_comp
        self.B = len(n_comp)
        self.N = int(sum(n_comp))
        ptr = np.zeros(self.B + 1, dtype=np.int64)
        ptr[1:] = np.cumsum(n_comp)
        self.cable_ptr_np = ptr
        self.celsius = float(celsius)
        self.v_init = float(v_init)
        self._diam = self._per_comp(diam)
        self.rhoa = self._per_comp(rhoa)
        self.cm = self._per_comp(cm)
        self._dx = self._per_comp(dx)
        hh = {**HH_DEFAULTS, **(hh or {})}
        self.ena = float(hh["ena"])
        self.ek = float(hh["ek"])
        self._chan = {k: self._per_comp(hh[k]) for k in ("gnabar", "gkbar", "gl", "el")}
        if fast_math and dtype != torch.float32:
            raise ValueError("fast_math applies to float32 state only")
        self.fast_math = bool(fast_math)
        self.compress_uniform = bool(compress_uniform)
        # cables in flight per CTA of the persistent kernels (0 = library
        # default); dendra_gb300.autotune.tune_cable_run picks it
        self.warps_per_block = 0
        # Thomas/PCR split of the persistent run: None = 32 lanes per cable;
        # (k16, k8) = cables with K <= k8 run on 8 lanes, K <= k16 on 16
        # lanes, longer ones on 32 (rows per lane on 16 or 8 lanes may not
        # exceed max(8, those of the longest cable on 32)).  tune_cable_run
        # picks it.
        self.lanes_split = None
        # True: one cable per CTA of 4 warps, the gate advance of its rows
        # spread over the SM's four sub-partitions (the same operations:
        # float32 results bit for bit, float64 up to last-bit contraction).
        # With warps_per_block 0 and no lanes split the library also chooses
        # it for a population of at most one cable per SM.
        self.split_gates = False
        self.field = None
        self.ve = None
        self.intra = None
        self.t = 0.0
        # time origin of the stimulus grid: step k of a run sees
        # t0_ms + (step_index + k) dt, in binary64, cast to the state dtype
        self.t0_ms = 0.0
        self.dt = None
        self._dev = {}

    # -- geometry --------------------------------------------------------
    def _per_comp(self, value):
        """Expand a scalar / per-cable / per-compartment value to (N,) in dtype (CPU)."""
        t = torch.as_tensor(value, dtype=self.dtype)
        if t.ndim == 0:
            return t.expand(self.N).clone()
        if t.numel() == self.B and self.B != self.N:
            return torch.repeat_interleave(t, torch.as_tensor(self.n_comp))
        if t.numel() == self.N:
            return t.reshape(self.N).clone()
        raise ValueError(f"expected a scalar, {self.B} per-cable or {self.N} per-compartment values")

    def positions(self):
        """Packed compartment centres (um) of Unmyelinated-style cables."""
        ks = np.asarray(self.n_comp)
        first = self.cable_ptr_np[:-1]
        dx = self._dx.double().numpy()[first]
        local = np.arange(self.N) - np.repeat(first, ks)
        half = np.repeat((ks - 1) * dx / 2.0, ks)
        step = np.repeat(np.where(ks > 1, (ks - 1) * dx / np.maximum(ks - 1, 1), 0.0), ks)
        return torch.as_tensor(-half + local * step)

    def _workspace(self, dt):
        """Per-compartment g_right, g_left, scale, cm_inv (implicit.py:484-522).

        Element-wise identical to the reference's per-cable (B, K) arithmetic;
        edges are the adjacent compartment pairs inside one cable.
        """
        dt_s = dt_seconds(dt, self.dtype)
        cm = torch.as_tensor(self.cm, dtype=self.dtype)
        diam, dx = self._diam, self._dx
        area = membrane_area(diam, dx)
        capacitance = 1.0e-6 * (cm * torch.ones_like(area)) * area
        cm_inv = capacitance.reciprocal()
        scale = area * cm_inv
        g_edge = cylindrical_edge_conductance(diam, dx, self.rhoa)
        cab = torch.as_tensor(np.repeat(np.arange(self.B), self.n_comp))
        inner = cab[1:] == cab[:-1]  # edge (i, i+1) lies inside one cable
        zero = torch.zeros_like(g_edge)
        g_right = torch.zeros(self.N, dtype=self.dtype)
        g_left = torch.zeros(self.N, dtype=self.dtype)
        g_right[:-1] = torch.where(inner, g_edge / capacitance[:-1], zero)
        g_left[1:] = torch.where(inner, g_edge / capacitance[1:], zero)
        return dict(g_right=g_right, g_left=g_left, scale=scale, cm_inv=cm_inv, dt_s=dt_s)

    # -- stimuli ---------------------------------------------------------
    def set_extracellular(self, field, amp, delay, pw):
        """ve(t) = field * amp on [delay, delay+pw) per cable (mono_rect x point field).

        amp, delay, pw: scalars (held as float32 values, like the reference's
        waveform parameters) or per-cable tensors."""
        self.field = self._per_comp(field)
        self.ve = tuple(waveform_param(x).to(self.dtype).expand(self.B).clone()
                        for x in (amp, delay, pw))
        self._dev.pop("field", None)

    def inject(self, comp_idx, amp, delay, pw):
        """Current clamp (mA) at local compartment comp_idx per cable (-1: none)."""
        idx = torch.as_tensor(comp_idx, dtype=torch.int32).expand(self.B).clone()
        if bool(((idx >= torch.as_tensor(self.n_comp, dtype=torch.int32)) | (idx < -1)).any()):
            raise ValueError("injection compartment out of range")
        self.intra = (idx,) + tuple(waveform_param(x).to(self.dtype).expand(self.B).clone()
                                    for x in (amp, delay, pw))

    # -- lifecycle -------------------------------------------------------
    def initialize(self, dt):
        """Build the workspace, set v_init and steady-state gates, upload."""
        self.dt = float(dt)
        ws = self._workspace(self.dt)
        self.dt_s = ws.pop("dt_s")
        v = torch.full((self.N,), self.v_init, dtype=self.dtype)
        m, h, n = hh_steady_state(v)
        dev = self.device
        d = {k: t.to(dev) for k, t in ws.items()}
        d.update({k: t.to(dev) for k, t in self._chan.items()})
        d["cable_ptr"] = torch.as_tensor(self.cable_ptr_np, device=dev)
        order = np.argsort(-np.asarray(self.n_comp), kind="stable").astype(np.int32)
        d["order"] = torch.as_tensor(order, device=dev)
        d["comp_cable"] = torch.as_tensor(
            np.repeat(np.arange(self.B, dtype=np.int32), self.n_comp), device=dev)
        d["scratch"] = torch.zeros(4, dtype=torch.int32, device=dev)
        if self.field is not None:
            d["field"] = self.field.to(dev)
            d["ve_amp"], d["ve_delay"], d["ve_pw"] = (x.to(dev) for x in self.ve)
        if self.intra is not None:
            d["in_idx"], d["in_amp"], d["in_delay"], d["in_pw"] = (x.to(dev) for x in self.intra)
        self._dev = d
        self.uniform_channels = self.compress_uniform and self._channels_uniform()
        self.uniform_geometry = self.compress_uniform and self._geometry_uniform(ws)
        self.v = v.to(dev)
        self.m, self.h, self.n = m.to(dev), h.to(dev), n.to(dev)
        self.t = 0.0
        self.step_index = 0
        return self

    def _channels_uniform(self):
        """True when gnabar, gkbar, gl, el are constant inside every cable."""
        cab = torch.as_tensor(np.repeat(np.arange(self.B), self.n_comp))
        same_cable = cab[1:] == cab[:-1]
        for t in self._chan.values():
            if bool(((t[1:] != t[:-1]) & same_cable).any()):
                return False
        return True

    def _geometry_uniform(self, ws):
        """True when g_right / g_left (interior edges) and scale are constant per cable."""
        cab = torch.as_tensor(np.repeat(np.arange(self.B), self.n_comp))
        same = cab[1:] == cab[:-1]
        gr, gl, sc = ws["g_right"], ws["g_left"], ws["scale"]
        # g_right on compartments i < K-1 and g_left on i > 0 are the interior edges
        gr_in = gr[:-1][same]
        gl_in = gl[1:][same]
        cab_edges = cab[:-1][same]
        for t in (gr_in, gl_in):
            if t.numel() > 1 and bool(((t[1:] != t[:-1]) & (cab_edges[1:] == cab_edges[:-1])).any()):
                return False
        if bool(((sc[1:] != sc[:-1]) & same).any()):
            return False
        return True

    def _args(self, n_steps=0, rec_every=1, rec_idx=None, trace=None, spk=None, spk_thr=0.0):
        d = self._dev
        a = _lib.CableArgs()
        a.dtype = _lib.dtype_code(self.dtype)
        a.n_cables = self.B
        a.n_steps = int(n_steps)
        a.rec_every = int(rec_every)
        a.cable_ptr = d["cable_ptr"].data_ptr()
        a.order = d["order"].data_ptr()
        a.v, a.m, a.h, a.n = (t.data_ptr() for t in (self.v, self.m, self.h, self.n))
        for k in ("g_right", "g_left", "scale", "cm_inv", "gnabar", "gkbar", "gl", "el"):
            setattr(a, k, d[k].data_ptr())
        if "field" in d:
            a.field = d["field"].data_ptr()
            a.ve_amp, a.ve_delay, a.ve_pw = (d[k].data_ptr() for k in ("ve_amp", "ve_delay", "ve_pw"))
        if "in_idx" in d:
            a.in_idx, a.in_amp, a.in_delay, a.in_pw = (
                d[k].data_ptr() for k in ("in_idx", "in_amp", "in_delay", "in_pw"))
        a.ena, a.ek, a.q10 = self.ena, self.ek, q10_of(self.celsius)
        a.dt_ms, a.dt_s, a.t0_ms = self.dt, self.dt_s, float(self.t0_ms)
        a.step0 = self.step_index
        if rec_idx is not None:
            a.rec_idx = rec_idx.data_ptr()
            a.trace = trace.data_ptr()
        if spk is not None:
            a.spk_idx, a.spk_below, a.spk_count, a.spk_first = (t.data_ptr() for t in spk)
            a.spk_thr = float(spk_thr)
        a.max_k = max(self.n_comp)
        a.flags = ((_lib.CABLE_UNIFORM_CHANNELS if self.uniform_channels else 0)
                   | (_lib.CABLE_UNIFORM_GEOMETRY if self.uniform_geometry else 0)
                   | (_lib.CABLE_FAST_MATH if self.fast_math else 0)
                   | (_lib.CABLE_SPLIT_GATES if self.split_gates else 0))
        a.n_comp = self.N
        a.comp_cable = d["comp_cable"].data_ptr()
        a.scratch = d["scratch"].data_ptr()
        a.warps_per_block = int(self.warps_per_block)
        if self.lanes_split is not None:
            n32, n16 = self._lane_counts(self.lanes_split)
            a.lanes_mode, a.n_lanes32, a.n_lanes16 = 1, n32, n16
        return a

    def _lane_counts(self, split):
        """Cables on 32 and on 16 lanes for split (k16, k8); the work order
        lists cables by non-increasing K, so each class is one contiguous run."""
        k16, k8 = (int(x) for x in split)
        # rows per lane of the launch: those of the longest cable on 32 lanes, at least 8
        ch = max(-(-max(self.n_comp) // 32), 8)
        if not (0 <= k8 <= 8 * ch and 0 <= k16 <= 16 * ch):
            raise ValueError(f"lanes_split (k16, k8) needs k16 <= {16 * ch} and k8 <= {8 * ch} "
                             "for this population")
        k8 = min(k8, k16)
        ks = np.asarray(self.n_comp)
        n32 = int((ks > k16).sum())
        n16 = int(((ks > k8) & (ks <= k16)).sum())
        return n32, n16

    def run(self, n_steps, *, rec_idx=None, rec_every=1, spk_idx=None, spk_thr=0.0,
            spk_state=None, spk_idx2=None, stop_on_spike=False, cables=None,
            record_all=False, raster=None, raster_cap=64, raster_state=None):
        """Advance every cable by n_steps in one persistent launch.

        rec_idx / spk_idx: per-cable local compartment (int, sequence or
        tensor; -1 disables).  Returns a RunResult with the trace
        (B, 1 + n_steps//rec_every), spike counts and first crossing steps
        (1-based step index within this call, -1 if none).  spk_idx2: an
        optional second detection compartment (an edge at either counts).
        stop_on_spike: a cable stops after the step of its first spike.
        cables: optional int32 device tensor of the cables to advance (others
        are left untouched).
        record_all: also record v of every compartment every rec_every steps
        (``trace_all``, shape (1 + n_steps//rec_every, N), packed like the
        state; Recorder(("v",)) of the reference).
        raster: up to 4 checked compartments per cable (a sequence of local
        indices applied to every cable, negative counting from the far end like
        Raster's node_check, or a (B, R) tensor); every upward crossing of
        spk_thr is counted and its step stored (``raster``, a RasterState,
        at most raster_cap steps per check).  raster_state continues an
        earlier run's raster (its idx is reused).
        """
        if self.dt is None:
            raise RuntimeError("Model must be initialized before running.")
        dev = self.device
        kk = torch.as_tensor(self.n_comp, dtype=torch.int32)
        for name, idx in (("rec_idx", rec_idx), ("spk_idx", spk_idx), ("spk_idx2", spk_idx2)):
            if idx is not None:
                ii = torch.as_tensor(idx, dtype=torch.int32).expand(self.B).cpu()
                if bool(((ii < -1) | (ii >= kk)).any()):
                    raise ValueError(f"{name} out of range for some cable")
        trace = rec = None
        if rec_idx is not None:
            rec = torch.as_tensor(rec_idx, dtype=torch.int32).expand(self.B).contiguous().to(dev)
            trace = torch.full((self.B, 1 + int(n_steps) // int(rec_every)), float("nan"),
                               dtype=self.dtype, device=dev)
        spk = None
        if spk_idx is not None:
            si = torch.as_tensor(spk_idx, dtype=torch.int32).expand(self.B).contiguous().to(dev)
            below = (torch.ones(self.B, dtype=torch.int32, device=dev) if spk_state is None
                     else spk_state)
            spk = (si, below, torch.zeros(self.B, dtype=torch.int32, device=dev),
                   torch.full((self.B,), -1, dtype=torch.int32, device=dev))
        args = self._args(n_steps, rec_every, rec, trace, spk, spk_thr)
        if spk_idx2 is not None:
            si2 = torch.as_tensor(spk_idx2, dtype=torch.int32).expand(self.B).contiguous().to(dev)
            b2 = torch.ones(self.B, dtype=torch.int32, device=dev)
            self._keep = (si2, b2)
            args.spk_idx2, args.spk_below2 = si2.data_ptr(), b2.data_ptr()
        if stop_on_spike:
            args.flags |= _lib.CABLE_STOP_ON_SPIKE
        if cables is not None:
            args.order = cables.data_ptr()
            args.n_cables = int(cables.numel())
            args.lanes_mode = 0  # the lane classes are positions of the full order
        trace_all = None
        if record_all:
            trace_all = torch.full((1 + int(n_steps) // int(rec_every), self.N), float("nan"),
                                   dtype=self.dtype, device=dev)
            args.trace_all = trace_all.data_ptr()
        rs = None
        if raster is not None or raster_state is not None:
            rs = raster_state if raster_state is not None else self._raster(raster, raster_cap)
            args.n_rast = int(rs.idx.shape[1])
            args.rast_idx, args.rast_below, args.rast_count = (
                t.data_ptr() for t in (rs.idx, rs.below, rs.count))
            args.rast_steps = rs.steps.data_ptr()
            args.rast_cap = int(rs.steps.shape[2])
            args.spk_thr = float(spk_thr)
        with torch.cuda.device(dev):
            rc = _lib.load().dgb_cable_run(args, _lib.stream_ptr(dev))
        _lib.check(rc, "dgb_cable_run")
        self.t = self.t + int(n_steps) * self.dt
        self.step_index += int(n_steps)
        return RunResult(trace, spk[2] if spk else None, spk[3] if spk else None, trace_all, rs)

    def _raster(self, raster, cap):
        """A fresh RasterState for the checked compartments ``raster``."""
        kk = torch.as_tensor(self.n_comp, dtype=torch.int64)
        idx = torch.as_tensor(raster, dtype=torch.int64)
        if idx.ndim == 1:
            idx = idx.reshape(1, -1).expand(self.B, -1)
        if idx.ndim != 2 or idx.shape[0] != self.B or not 1 <= idx.shape[1] <= 4:
            raise ValueError("raster takes 1 to 4 checked compartments per cable")
        idx = torch.where(idx < 0, idx + kk.reshape(-1, 1), idx)
        if bool(((idx < 0) | (idx >= kk.reshape(-1, 1))).any()):
            raise ValueError("raster compartment out of range for some cable")
        if int(cap) < 0:
            raise ValueError("raster_cap must be >= 0")
        dev = self.device
        R = idx.shape[1]
        return RasterState(idx.to(torch.int32).contiguous().to(dev),
                           torch.ones((self.B, R), dtype=torch.int32, device=dev),
                           torch.zeros((self.B, R), dtype=torch.int32, device=dev),
                           torch.full((self.B, R, max(int(cap), 0)), -1, dtype=torch.int64,
                                      device=dev))

    def check_status(self):
        """Raise if the last persistent run flagged a cable it could not advance."""
        err = int(self._dev["scratch"][1].item())
        if err:
            raise RuntimeError(f"dgb_cable_run reported error bits {err:#x}")

    def step_plain(self, bands=None):
        """One step through the unfused assemble + solve/update kernels."""
        if bands is None:
            bands = torch.empty((4, self.N), dtype=self.dtype, device=self.device)
        args = self._args(1)
        L = _lib.load()
        st = _lib.stream_ptr(self.device)
        p = [bands[i].data_ptr() for i in range(4)]
        with torch.cuda.device(self.device):
            rc = L.dgb_cable_assemble(args, 0, p[0], p[1], p[2], p[3], st)
            _lib.check(rc, "dgb_cable_assemble")
            rc = L.dgb_cable_solve_update(args, p[0], p[1], p[2], p[3], st)
            _lib.check(rc, "dgb_cable_solve_update")
        self.t = self.t + self.dt
        self.step_index += 1
        return bands

    # -- oracle interchange ---------------------------------------------
    def problem_dict(self):
        """Host numpy copy of the packed problem (used by tests and baselines)."""
        d = {k: v.detach().cpu().numpy() for k, v in self._dev.items()
             if k not in ("scratch", "order", "comp_cable")}
        d.update(v=self.v.cpu().numpy().copy(), m=self.m.cpu().numpy().copy(),
                 h=self.h.cpu().numpy().copy(), n=self.n.cpu().numpy().copy())
        d.update(ena=self.ena, ek=self.ek, q10=q10_of(self.celsius), dt_ms=self.dt,
                 dt_s=self.dt_s)
        return d


def hh_steady_state(v):
    """Steady-state m, h, n at v in v's dtype (mod/HH.py:42-56)."""
    def vtrap(x, y):
        q = x / y
        thr = 1.0 if v.dtype == torch.float32 else 0.5
        small = q.abs() <= thr
        sq = torch.where(small, q, torch.zeros_like(q))
        sx = torch.where(small, x, torch.zeros_like(q))
        sy = torch.where(small, y, torch.zeros_like(q))
        q2 = sq * sq
        if v.dtype == torch.float64:
            val = q2 * (43867 / 5109094217170944000) - 3617 / 10670622842880000
            val = val * q2 + 1 / 74724249600
            val = val * q2 - 691 / 1307674368000
            val = val * q2 + 1 / 47900160
        else:
            val = q2 * (-691 / 1307674368000) + 1 / 47900160
        val = val * q2 - 1 / 1209600
        val = val * q2 + 1 / 30240
        val = val * q2 - 1 / 720
        val = val * q2 + 1 / 12
        approx = torch.addcmul(sy - sx / 2, sx, sq * val)
        q_safe = torch.where(small, torch.ones_like(q), q)
        return torch.where(small, approx, x / (torch.exp(q_safe) - 1))

    ten = torch.full_like(v, 10.0)
    alpha_m = AM1 * vtrap(-(v + 40), ten)
    beta_m = 4.0 * torch.exp(-(v + 65) / 18)
    alpha_h = AH1 * torch.exp(-(v + 65) / 20)
    beta_h = 1.0 / (torch.exp(-(v + 35) / 10) + 1)
    alpha_n = AN1 * vtrap(-(v + 55), ten)
    beta_n = 0.125 * torch.exp(-(v + 65) / 80)
    return (alpha_m / (alpha_m + beta_m), alpha_h / (alpha_h + beta_h),
            alpha_n / (alpha_n + beta_n))


def unmyelinated_K(L_um: float, dx_um: float) -> int:
    """Compartment count of dn.Unmyelinated(L, dx): ceil(L/dx)//2*2+1 (core.py:10937-10940)."""
    return math.ceil(L_um / dx_um) // 2 * 2 + 1
