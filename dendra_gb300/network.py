"""Spiking networks of branched cells on the GB300 kernels.

Host side of the reference's Network path for HH-soma / passive-dendrite
trees with Exp2Syn synapses and NetCon connections:

* tree workspace — integrators/tree.py:477-612 (axial conductance from
  half-segment resistances) and :1010-1044 (cm/dt, area);
* synapses — mod/EXP2SYN.py (A, B states; factor and tau1_effective from
  derive_buffers :112-144; exact decay of A' = -A/tau1_effective);
* connections — NetCon with delays rounded half-even to steps, at least one
  (netcon.py:2760-2795), weights in uS;
* the step loop — Network.run phase order (networks/net.py:214-240).

A run advances the network in windows of W steps (W = the smallest delay, at
most 64): ``dgb_net_window`` advances every cell W steps with its state in
shared memory, then ``dgb_net_enqueue`` scatters the window's spikes into the
delay ring.  Background (NetStim-like) events are generated on the host from
a seeded Poisson process and fed to one synapse per cell, identically to the
oracle.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .cable import HH_DEFAULTS, dt_seconds, hh_steady_state, q10_of
from .netcon import TargetCSR, exp2syn_factor, inference_delay_steps
from .tree import ForestPlan


class NetArgs(ctypes.Structure):
    """Mirror of dgb_net_args."""

    from .tree import DgbForest as _F

    _fields_ = [
        ("dtype", ctypes.c_int32), ("n_cells", ctypes.c_int32), ("n_steps", ctypes.c_int32),
        ("bg_syn", ctypes.c_int32), ("step0", ctypes.c_int64), ("depth", ctypes.c_int64),
        ("slot0", ctypes.c_int64), ("n_syn", ctypes.c_int64), ("forest", _F),
        ("v", ctypes.c_void_p), ("area", ctypes.c_void_p), ("cm_dt", ctypes.c_void_p),
        ("a_geom", ctypes.c_void_p), ("gl", ctypes.c_void_p), ("el", ctypes.c_void_p),
        ("m", ctypes.c_void_p), ("h", ctypes.c_void_p), ("n", ctypes.c_void_p),
        ("gnabar", ctypes.c_double), ("gkbar", ctypes.c_double), ("ena", ctypes.c_double),
        ("ek", ctypes.c_double), ("q10", ctypes.c_double), ("dt_ms", ctypes.c_double),
        ("spk_thr", ctypes.c_double),
        ("syn_ptr", ctypes.c_void_p), ("node_syn_ptr", ctypes.c_void_p),
        ("syn_A", ctypes.c_void_p), ("syn_B", ctypes.c_void_p), ("syn_factor", ctypes.c_void_p),
        ("syn_decay_A", ctypes.c_void_p), ("syn_decay_B", ctypes.c_void_p),
        ("e_syn", ctypes.c_double), ("ring", ctypes.c_void_p),
        ("bg_bits", ctypes.c_void_p), ("bg_words", ctypes.c_int64), ("bg_weight", ctypes.c_double),
        ("below", ctypes.c_void_p), ("spike_bits", ctypes.c_void_p),
        ("spike_count", ctypes.c_void_p),
        ("warps_per_block", ctypes.c_int32), ("threads_per_cell", ctypes.c_int32),
        ("ve_field", ctypes.c_void_p), ("ve_amp", ctypes.c_void_p), ("ve_delay", ctypes.c_void_p),
        ("ve_pw", ctypes.c_void_p), ("in_node", ctypes.c_void_p), ("in_amp", ctypes.c_void_p),
        ("in_delay", ctypes.c_void_p), ("in_pw", ctypes.c_void_p), ("t0_ms", ctypes.c_double),
        ("cell_list", ctypes.c_void_p), ("n_list", ctypes.c_int32), ("list_max_k", ctypes.c_int32),
    ]


@dataclass
class Cell:
    """One branched cell: parent (-1 at the soma node 0), compartment lengths
    and diameters (um); node 0 carries HH, the rest the passive leak."""

    parent: np.ndarray
    length: np.ndarray
    diam: np.ndarray


def axial_conductance(parent, length_um, diam_um, ra):
    """Conductance (S) of each node to its parent from half-segment resistances
    (integrators/tree.py:560-583); 0 at the root."""
    L = np.asarray(length_um, dtype=np.float64) * 1e-4
    r = np.asarray(diam_um, dtype=np.float64) * 1e-4 * 0.5
    half = ra * (L / 2) / (np.pi * r ** 2)
    parent = np.asarray(parent)
    a = np.zeros(parent.size)
    nz = parent >= 0
    a[nz] = 1.0 / (half[nz] + half[parent[nz]])
    return a


def random_cell(rng, k_target, max_depth=12, soma_len=20.0, soma_diam=20.0):
    """Random binary-branching tree with ~k_target compartments.

    Branch lengths U[20, 200] um, diameters 2 um at the soma, times U[0.7, 0.95]
    per branch point, branch points at most max_depth deep; compartments of
    equal length inside each branch, their number scaled to reach k_target."""
    branches = [(-1, 0, 2.0)]  # (parent branch, depth, diameter)
    frontier = [0]
    while frontier and len(branches) < max(3, k_target // 6):
        b = frontier.pop(int(rng.integers(len(frontier))))
        _, depth, diam = branches[b]
        if depth >= max_depth:
            continue
        for _ in range(2):
            branches.append((b, depth + 1, diam * rng.uniform(0.7, 0.95)))
            frontier.append(len(branches) - 1)
    blen = rng.uniform(20.0, 200.0, len(branches))
    total = blen.sum()
    nseg = np.maximum(1, np.round(blen / total * (k_target - 1)).astype(int))
    parent, length, diam = [-1], [soma_len], [soma_diam]
    last = {}
    for bi, (pb, _, d) in enumerate(branches):
        prev = 0 if pb < 0 else last[pb]
        for _ in range(nseg[bi]):
            parent.append(prev)
            length.append(blen[bi] / nseg[bi])
            diam.append(d)
            prev = len(parent) - 1
        last[bi] = prev
    return Cell(np.asarray(parent), np.asarray(length), np.asarray(diam))


class TreeNetwork:
    """A network of branched cells with Exp2Syn synapses and fixed-delay NetCons.

    cells: list of Cell.  syn_node: per cell, local nodes of its synapses (the
    first synapse of every cell is its background synapse).  Connections:
    pre cell, post synapse (global index), delay (ms), weight (uS).
    """

    def __init__(self, cells, syn_node, conn_pre, conn_post, conn_delay_ms, conn_weight, *,
                 dt=0.025, dtype=torch.float32, device="cuda", ra=100.0, cm=1.0, celsius=6.3,
                 v_init=-65.0, g_pas=0.001, e_pas=-70.0, tau1=0.5, tau2=5.0, e_syn=0.0,
                 spk_thr=0.0, bg_steps=None, bg_weight=0.0, window=None, chains=True,
                 bg_netstim=None, extracellular=None, clamp=None, size_classes=False):
        self.dtype = dtype
        self.device = torch.device(device)
        self.dt = float(dt)
        self.n_cells = len(cells)
        dev = self.device
        # chains=True: the window kernel eliminates one unbranched chain per
        # lane (tree.build_chains); False: the depth-layer schedule.  Same results.
        self.plan = ForestPlan([c.parent for c in cells], device=dev, chains=chains)
        node_ptr = self.plan.node_ptr
        N = int(node_ptr[-1])
        self.N = N
        hh = HH_DEFAULTS
        area = np.concatenate([np.pi * c.diam * c.length * 1e-8 for c in cells])  # cm^2
        a_geom = np.concatenate([axial_conductance(c.parent, c.length, c.diam, ra) for c in cells])
        dt_s = dt_seconds(dt, dtype)
        gl = np.full(N, g_pas)
        el = np.full(N, e_pas)
        gl[node_ptr[:-1]] = hh["gl"]
        el[node_ptr[:-1]] = hh["el"]
        t = lambda x: torch.as_tensor(np.asarray(x), dtype=dtype)  # noqa: E731
        area_t = t(area)
        cap = 1.0e-6 * (torch.as_tensor(cm, dtype=dtype) * torch.ones_like(area_t)) * area_t
        self.nodes = dict(area=area_t, cm_dt=cap / torch.as_tensor(dt_s, dtype=dtype),
                          a_geom=t(a_geom), gl=t(gl), el=t(el))
        # synapses: sorted by node inside each cell
        syn_ptr = np.zeros(self.n_cells + 1, dtype=np.int64)
        node_syn_ptr = np.zeros(N + self.n_cells, dtype=np.int32)
        self.syn_perm = []
        for c, nodes in enumerate(syn_node):
            nodes = np.asarray(nodes, dtype=np.int64)
            perm = np.argsort(nodes, kind="stable")
            self.syn_perm.append(perm)
            syn_ptr[c + 1] = syn_ptr[c] + nodes.size
            K = node_ptr[c + 1] - node_ptr[c]
            cnt = np.bincount(nodes, minlength=K)
            node_syn_ptr[node_ptr[c] + c + 1: node_ptr[c] + c + K + 1] = np.cumsum(cnt)
        # the background synapse (local index 0 before sorting) after sorting
        self.bg_syn_sorted = np.array([int(np.nonzero(p == 0)[0][0]) for p in self.syn_perm])
        if len(set(self.bg_syn_sorted.tolist())) != 1:
            raise ValueError("the background synapse must keep the same local slot in every cell")
        self.n_syn = int(syn_ptr[-1])
        ratio = torch.clamp(torch.tensor(tau1 / tau2, dtype=torch.float64), 1e-9, 0.9999)
        tau1_eff = float(ratio * tau2)
        factor = float(exp2syn_factor(tau1, tau2))
        self.syn = dict(
            factor=torch.full((self.n_syn,), factor, dtype=dtype),
            decay_A=torch.full((self.n_syn,), float(np.exp(-dt / tau1_eff)), dtype=dtype),
            decay_B=torch.full((self.n_syn,), float(np.exp(-dt / tau2)), dtype=dtype),
        )
        # global synapse index of (cell, original local index)
        self.syn_global = [syn_ptr[c] + np.argsort(p, kind="stable") for c, p in
                           enumerate(self.syn_perm)]
        post = np.asarray(conn_post, dtype=np.int64)
        cell_of_post = np.searchsorted(syn_ptr, post, side="right") - 1
        local = post - syn_ptr[cell_of_post]
        post_sorted = np.array([self.syn_global[c][k] for c, k in zip(cell_of_post, local)],
                               dtype=np.int64) if post.size else post
        _, dsteps = inference_delay_steps(torch.as_tensor(conn_delay_ms), dt)
        dsteps = dsteps.numpy()
        self.depth = int(dsteps.max()) + 1 if dsteps.size else 2
        self.window = int(min(64, dsteps.min() if dsteps.size else 64)) if window is None \
            else int(window)
        if dsteps.size and self.window > dsteps.min():
            raise ValueError("the window must not exceed the smallest delay")
        # cells in flight per CTA of dgb_net_window (0 = library default);
        # dendra_gb300.autotune.tune_network picks it
        self.warps_per_block = 0
        # threads advancing one cell (0 = library default 128); the autotuner's
        # other knob
        self.threads_per_cell = 0
        csr = TargetCSR(torch.as_tensor(post_sorted), self.n_syn)
        perm = csr.perm.numpy()
        self.conn = dict(
            pre=np.asarray(conn_pre, dtype=np.int64), post=post_sorted, delay=dsteps,
            weight=np.asarray(conn_weight, dtype=np.float64))
        self.csr = dict(ptr=csr.ptr, pre=torch.as_tensor(self.conn["pre"][perm]),
                        delay=torch.as_tensor(dsteps[perm]),
                        weight=torch.as_tensor(self.conn["weight"][perm], dtype=dtype))
        # background events: bit (step, cell), from host lists or generated on
        # the device by a NetStim with one generator per cell
        if bg_netstim is not None and bg_netstim.N != self.n_cells:
            raise ValueError("bg_netstim needs one generator per cell")
        if bg_netstim is not None and bg_steps is not None:
            raise ValueError("give bg_steps or bg_netstim, not both")
        self.bg_steps = bg_steps
        self.bg_netstim = bg_netstim
        self.bg_weight = float(bg_weight)
        self.params = dict(gnabar=hh["gnabar"], gkbar=hh["gkbar"], ena=hh["ena"], ek=hh["ek"],
                           q10=q10_of(celsius), dt_ms=float(dt), spk_thr=float(spk_thr),
                           e_syn=float(e_syn))
        self.v_init = float(v_init)
        # optional drive of the tree step: extracellular (field per node in mV
        # per unit amplitude; amp, delay, pw per cell, a rectangular pulse) and
        # an injected current (local node, amp in mA, delay, pw per cell)
        self.drive = {}
        per_cell = lambda x: torch.as_tensor(x, dtype=dtype).reshape(-1).expand(  # noqa: E731
            self.n_cells).clone()
        if extracellular is not None:
            field, amp, delay, pw = extracellular
            field = torch.as_tensor(field, dtype=dtype).reshape(-1)
            if field.numel() != N:
                raise ValueError(f"the extracellular field needs one value per node ({N})")
            self.drive.update(ve_field=field, ve_amp=per_cell(amp), ve_delay=per_cell(delay),
                              ve_pw=per_cell(pw))
        if clamp is not None:
            node, amp, delay, pw = clamp
            node = torch.as_tensor(node, dtype=torch.int32).reshape(-1).expand(self.n_cells)
            kk = torch.as_tensor(np.diff(node_ptr), dtype=torch.int32)
            if bool(((node < -1) | (node >= kk)).any()):
                raise ValueError("clamp node out of range for some cell")
            self.drive.update(in_node=node.clone(), in_amp=per_cell(amp),
                              in_delay=per_cell(delay), in_pw=per_cell(pw))
        self._syn_ptr = syn_ptr
        self._node_syn_ptr = node_syn_ptr
        # size classes (off by default): cells of at most half the largest
        # cell's compartments are advanced by their own window launch, whose
        # shared memory per cell is sized for them (about twice as many cells
        # per SM); same results.  On the 4,096-cell network the two launches run one after
        # the other and each ends in a tail: 2.36e10 vs 2.44e10 in one launch.
        self.classes = None
        kk = np.diff(node_ptr)
        half = int(kk.max()) // 2
        small = np.nonzero(kk <= half)[0]
        large = np.nonzero(kk > half)[0]
        if size_classes and small.size and large.size:
            self.classes = [(torch.as_tensor(ix, dtype=torch.int32, device=dev),
                             int(kk[ix].max())) for ix in (large, small)]
        self._upload()

    @property
    def _has_bg(self):
        return self.bg_steps is not None or self.bg_netstim is not None

    def _bg_device(self, n_steps):
        """Background bits of steps [0, n_steps) as a device tensor: generated
        by the NetStim (counter-based draws: the same bits for any split of the
        run) or uploaded from the host lists."""
        if self.bg_netstim is not None:
            ns = self.bg_netstim.initialize()
            bits = ns.run(n_steps, self.params["dt_ms"], spikes=False, bits=True)
            return bits, bits.shape[1]
        bits_np, words = self._bg_bits(n_steps)
        return torch.as_tensor(bits_np.view(np.int64), device=self.device), words

    def _bg_bits(self, n_steps):
        if self.bg_netstim is not None:
            bits, words = self._bg_device(n_steps)
            return bits.cpu().numpy().view(np.uint64), words
        words = max(1, -(-self.n_cells // 64))
        bits = np.zeros((n_steps, words), dtype=np.uint64)
        if self.bg_steps is not None:
            for c, steps in enumerate(self.bg_steps):
                steps = np.asarray(steps, dtype=np.int64)
                steps = steps[(steps >= 0) & (steps < n_steps)]
                bits[steps, c >> 6] |= np.uint64(1) << np.uint64(c & 63)
        return bits, words

    def _upload(self):
        dev = self.device
        self.d = {k: v.to(dev) for k, v in self.nodes.items()}
        self.d.update({f"syn_{k}": v.to(dev) for k, v in self.syn.items()})
        self.d["syn_ptr"] = torch.as_tensor(self._syn_ptr, device=dev)
        self.d["node_syn_ptr"] = torch.as_tensor(self._node_syn_ptr, device=dev)
        self.d.update({f"csr_{k}": v.to(dev).contiguous() for k, v in self.csr.items()})
        self.d.update({f"drive_{k}": v.to(dev).contiguous() for k, v in self.drive.items()})
        self.reset()

    def reset(self):
        """Initial state (v_init, steady-state soma gates, empty synapses and
        ring).  Tensors are refilled in place once they exist, so a captured
        run (``capture``) stays bound to them."""
        dev, dt = self.device, self.dtype
        m, h, n = (x.to(dev) for x in hh_steady_state(
            torch.full((self.n_cells,), self.v_init, dtype=dt)))
        if getattr(self, "v", None) is None:
            self.v = torch.empty((self.N,), dtype=dt, device=dev)
            self.m, self.h, self.n = (torch.empty_like(x) for x in (m, h, n))
            self.A = torch.empty(self.n_syn, dtype=dt, device=dev)
            self.B = torch.empty(self.n_syn, dtype=dt, device=dev)
            self.ring = torch.empty(self.depth, self.n_syn, dtype=dt, device=dev)
            self.below = torch.empty(self.n_cells, dtype=torch.uint8, device=dev)
            self.spike_count = torch.empty(self.n_cells, dtype=torch.int32, device=dev)
        self.v.fill_(self.v_init)
        for dst, src in zip((self.m, self.h, self.n), (m, h, n)):
            dst.copy_(src)
        for t in (self.A, self.B, self.ring, self.spike_count):
            t.zero_()
        self.below.fill_(1)
        self.step = 0
        self.slot = 0

    def _windows(self, n_steps):
        W = self.window
        return [W] * (n_steps // W) + ([n_steps % W] if n_steps % W else [])

    def _prepare(self, n_steps):
        """Device inputs of a run of n_steps from the current step: background
        event bits and the per-window spike masks."""
        windows = self._windows(n_steps)
        bg, words = self._bg_device(self.step + n_steps)
        masks = torch.zeros(len(windows), self.n_cells, dtype=torch.int64, device=self.device)
        return windows, bg, words, masks

    def _launch(self, windows, bg, words, masks):
        """Enqueue the window loop on the current stream (no host synchronisation)."""
        L = _lib.load()
        st = _lib.stream_ptr(self.device)
        a = self._args()
        a.bg_bits = bg.data_ptr() if self._has_bg else None
        a.bg_words = words
        d = self.d
        for w, wl in enumerate(windows):
            a.n_steps = wl
            a.step0 = self.step
            a.slot0 = self.slot
            a.spike_bits = masks[w].data_ptr()
            with torch.cuda.device(self.device):
                for lst, kmax in self.classes or [(None, 0)]:
                    a.cell_list = None if lst is None else lst.data_ptr()
                    a.n_list = 0 if lst is None else lst.numel()
                    a.list_max_k = kmax
                    rc = L.dgb_net_window(ctypes.byref(a), st)
                    _lib.check(rc, "dgb_net_window")
                rc = L.dgb_net_enqueue(a.dtype, self.ring.data_ptr(), self.depth, self.n_syn,
                                       self.slot, d["csr_ptr"].data_ptr(), self.n_syn, None,
                                       d["csr_pre"].data_ptr(), d["csr_delay"].data_ptr(),
                                       d["csr_weight"].data_ptr(), masks[w].data_ptr(), st)
                _lib.check(rc, "dgb_net_enqueue")
            self.step += wl
            self.slot = (self.slot + wl) % self.depth

    def _raster(self, windows, masks, n_steps):
        W = self.window
        shifts = torch.arange(W, device=self.device, dtype=torch.int64)
        rows = ((masks[:, None, :] >> shifts[None, :, None]) & 1).to(torch.uint8)
        return rows.reshape(-1, self.n_cells)[:n_steps] if n_steps % W == 0 else \
            torch.cat([rows[i, :wl] for i, wl in enumerate(windows)])

    def run(self, n_steps):
        """Advance n_steps; returns the spike raster as a (n_steps, n_cells) uint8 tensor.

        Steps run in windows of at most ``self.window`` (the smallest delay);
        each window is one dgb_net_window launch plus one dgb_net_enqueue."""
        n_steps = int(n_steps)
        windows, bg, words, masks = self._prepare(n_steps)
        self._launch(windows, bg, words, masks)
        return self._raster(windows, masks, n_steps)

    def capture(self, n_steps):
        """Capture run(n_steps) from the current step as one CUDA graph.

        The graph holds every window launch and enqueue of the run (their step,
        slot and buffer arguments fixed at capture); ``CapturedRun.replay()``
        replays it from the same starting step, e.g. after ``reset()``.  Only
        kernels are captured: the host does nothing between windows."""
        n_steps = int(n_steps)
        start = (self.step, self.slot)
        windows, bg, words, masks = self._prepare(n_steps)
        dev = self.device
        _lib.load()
        graph = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.device(dev), torch.cuda.stream(side):
            with torch.cuda.graph(graph, stream=side, capture_error_mode="relaxed"):
                self._launch(windows, bg, words, masks)
        torch.cuda.current_stream(dev).wait_stream(side)
        self.step, self.slot = start  # capturing ran nothing
        return CapturedRun(self, graph, start, n_steps, windows, (bg, masks))

    def _args(self):
        a = NetArgs()
        a.dtype = _lib.dtype_code(self.dtype)
        a.n_cells = self.n_cells
        a.bg_syn = int(self.bg_syn_sorted[0])
        a.depth = self.depth
        a.n_syn = self.n_syn
        a.forest = self.plan.struct()
        d = self.d
        a.v = self.v.data_ptr()
        for k in ("area", "cm_dt", "a_geom", "gl", "el"):
            setattr(a, k, d[k].data_ptr())
        a.m, a.h, a.n = self.m.data_ptr(), self.h.data_ptr(), self.n.data_ptr()
        for k, val in self.params.items():
            setattr(a, k, val)
        a.syn_ptr = d["syn_ptr"].data_ptr()
        a.node_syn_ptr = d["node_syn_ptr"].data_ptr()
        a.syn_A, a.syn_B = self.A.data_ptr(), self.B.data_ptr()
        a.syn_factor = d["syn_factor"].data_ptr()
        a.syn_decay_A = d["syn_decay_A"].data_ptr()
        a.syn_decay_B = d["syn_decay_B"].data_ptr()
        a.ring = self.ring.data_ptr()
        a.bg_weight = self.bg_weight
        a.below = self.below.data_ptr()
        a.spike_count = self.spike_count.data_ptr()
        a.warps_per_block = int(self.warps_per_block)
        a.threads_per_cell = int(self.threads_per_cell)
        for k in self.drive:
            setattr(a, k, d[f"drive_{k}"].data_ptr())
        a.t0_ms = 0.0
        return a

    # -- oracle interchange ----------------------------------------------
    def problem_dict(self, n_steps):
        """Host copies of everything the oracle needs for n_steps from now."""
        T = self.plan.tensors
        bits, words = self._bg_bits(self.step + n_steps)
        c = lambda x: x.detach().cpu().numpy().copy()  # noqa: E731
        return dict(
            plan={k: c(v) for k, v in T.items()}, v=c(self.v), m=c(self.m), h=c(self.h),
            n=c(self.n), A=c(self.A), B=c(self.B), ring=c(self.ring), below=c(self.below),
            spike_count=c(self.spike_count), nodes={k: c(v) for k, v in self.nodes.items()},
            syn={k: c(v) for k, v in self.syn.items()}, syn_ptr=self._syn_ptr.copy(),
            node_syn_ptr=self._node_syn_ptr.copy(), conn=self.conn, params=self.params,
            bg_bits=bits if self._has_bg else None, bg_words=words,
            bg_syn=int(self.bg_syn_sorted[0]), bg_weight=self.bg_weight, depth=self.depth,
            slot=self.slot, step=self.step, n_syn=self.n_syn, n_cells=self.n_cells,
            t0_ms=0.0, **{k: c(v) for k, v in self.drive.items()})


class CapturedRun:
    """A network run captured as a CUDA graph (``TreeNetwork.capture``)."""

    def __init__(self, net, graph, start, n_steps, windows, buffers):
        self.net, self.graph, self.start = net, graph, start
        self.n_steps, self.windows = n_steps, windows
        self.bg, self.masks = buffers
        self.launches = (1 + len(net.classes or [None])) * len(windows)

    def replay(self):
        """Run the captured steps; returns the spike raster like ``run``."""
        net = self.net
        if (net.step, net.slot) != self.start:
            raise RuntimeError(f"the graph was captured at step/slot {self.start}, the network "
                               f"is at {(net.step, net.slot)} (reset() first)")
        self.masks.zero_()
        self.graph.replay()
        net.step += self.n_steps
        net.slot = (net.slot + self.n_steps) % net.depth
        return net._raster(self.windows, self.masks, self.n_steps)


def random_network(n_cells, k_range=(200, 2000), syn_per_cell=100, seed=0, dt=0.025,
                   rate_hz=5.0, t_stop_ms=200.0, bg_weight=0.05, delay_range=(1.0, 5.0),
                   bg="host", **kw):
    """A network like the 4,096-cell benchmark: random trees, syn_per_cell Exp2Syn inputs from random
    pre cells (lognormal(-7, 0.5) uS, delays U[1,5] ms), one background synapse at
    the soma driven by a seeded 5 Hz Poisson process: event times drawn on the
    host (bg="host") or a NetStim per cell on the device (bg="netstim":
    interval 1000/rate_hz ms, noise 1)."""
    rng = np.random.default_rng(seed)
    cells = [random_cell(rng, int(rng.integers(k_range[0], k_range[1] + 1)))
             for _ in range(n_cells)]
    syn_node, post, pre = [], [], []
    base = 0
    for c, cell in enumerate(cells):
        K = cell.parent.size
        nodes = np.concatenate([[0], rng.integers(1, max(2, K), syn_per_cell) % K])
        syn_node.append(nodes)
        post.extend(base + 1 + np.arange(syn_per_cell))  # synapse 0 is the background one
        pre.extend(rng.integers(0, n_cells, syn_per_cell))
        base += nodes.size
    n_conn = len(post)
    weight = rng.lognormal(-7.0, 0.5, n_conn)
    delay = rng.uniform(delay_range[0], delay_range[1], n_conn)
    n_steps = int(round(t_stop_ms / dt))
    bg_steps = []
    for _ in range(n_cells):
        isi = rng.exponential(1000.0 / rate_hz, int(3 + 2 * rate_hz * t_stop_ms / 1000.0))
        times = np.cumsum(isi)
        bg_steps.append(np.floor(times[times < t_stop_ms] / dt).astype(np.int64))
    if bg == "netstim":
        from .netstim import NetStim

        ns = NetStim(n_cells, interval=1000.0 / rate_hz, noise=1.0, start=0.0, seed=seed,
                     dtype=kw.get("dtype", torch.float32), device=kw.get("device", "cuda"))
        return TreeNetwork(cells, syn_node, pre, post, delay, weight, dt=dt, bg_netstim=ns,
                           bg_weight=bg_weight, **kw), n_steps
    return TreeNetwork(cells, syn_node, pre, post, delay, weight, dt=dt, bg_steps=bg_steps,
                       bg_weight=bg_weight, **kw), n_steps
