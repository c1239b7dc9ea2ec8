"""ctypes bindings of the C oracle — TEST INFRASTRUCTURE ONLY.

Builds ``oracle.c`` with gcc into ``oracle/_build/liboracle.so`` on first use
(the build is plain C with OpenMP; no reference sources are compiled).
"""

from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_SO = os.path.join(_BUILD, "liboracle.so")
_SRC = [os.path.join(_HERE, "oracle.c"), os.path.join(_HERE, "oracle_impl.h")]
_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle shared library if it is missing or stale."""
    os.makedirs(_BUILD, exist_ok=True)
    stale = not os.path.exists(_SO) or any(
        os.path.getmtime(s) > os.path.getmtime(_SO) for s in _SRC
    )
    if force or stale:
        tmp = _SO + f".tmp{os.getpid()}"
        cmd = [
            "gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
            "-fno-fast-math", "-o", tmp, _SRC[0], "-lm",
        ]
        subprocess.run(cmd, check=True)
        os.replace(tmp, _SO)
    return _SO


def lib():
    global _lib
    with _lock:
        if _lib is None:
            _lib = ctypes.CDLL(build())
            _declare(_lib)
    return _lib


_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I32 = ctypes.c_int32
_D = ctypes.c_double


def _declare(L):
    for sfx, real in (("_f64", ctypes.c_double), ("_f32", ctypes.c_float)):
        getattr(L, "orc_vtrap" + sfx).restype = real
        getattr(L, "orc_vtrap" + sfx).argtypes = [real, real]
        getattr(L, "orc_phi1" + sfx).restype = real
        getattr(L, "orc_phi1" + sfx).argtypes = [real]
        getattr(L, "orc_cnexp" + sfx).restype = real
        getattr(L, "orc_cnexp" + sfx).argtypes = [real, real, real, real]
        getattr(L, "orc_hh_rates" + sfx).argtypes = [real, real, _P]
        getattr(L, "orc_hh_steady" + sfx).argtypes = [real, _P]
        getattr(L, "orc_thomas_batched" + sfx).argtypes = [_I64, _I64, _P, _P, _P, _P, _P]
        getattr(L, "orc_pcr" + sfx).argtypes = [_I64, _P, _P, _P, _P, _P]
        getattr(L, "orc_dhs_solve_batched" + sfx).argtypes = [
            _I64, _I64, _P, _P, _P, _P, _P, _P, _I32, _P]
        getattr(L, "orc_cable_run" + sfx).argtypes = (
            [_I32, _I32, _I32, _P] + [_P] * 4 + [_P] * 9 + [_D] * 6
            + [_P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _D, _P, _P, _P, _I32, _P, _P]
            + [_P, _I32, _P, _P, _P, _I32, _P, _I64]
        )
        getattr(L, "orc_block3_thomas" + sfx).argtypes = [_I64, _I64, _P, _P, _P, _P, _P]
        getattr(L, "orc_cable_grad" + sfx).argtypes = (
            [_I32, _I32, _I32, _P] + [_P] * 4 + [_P] * 9 + [_D] * 6
            + [_P, _P, _P, _P, _P, _P, _P, _P, _P, _I32] + [_P] * 8
        )
        getattr(L, "orc_net_run" + sfx).argtypes = (
            [_I32, _I32, _I64, _I64, _P, _I64] + [_P] * 9 + [_P] * 9 + [_D] * 7
            + [_P, _P, _P, _P, _P, _P, _P, _D, _P, _P, _I64, _I32, _D, _I64, _P, _P, _P, _P, _P,
               _P, _P] + [_P] * 8 + [_D])
        getattr(L, "orc_two_tap_enqueue" + sfx).restype = ctypes.c_int
        getattr(L, "orc_two_tap_enqueue" + sfx).argtypes = (
            [_I64, _I64, _P, _I64, _I64, _P, _P, _P, _I64, _P, _P, _P, _P])
        getattr(L, "orc_three_tap_enqueue" + sfx).restype = ctypes.c_int
        getattr(L, "orc_three_tap_enqueue" + sfx).argtypes = (
            [_I64, _I64, _P, _I64, _I64, _P, _P, _P, _I64, _P, _P, _P, _P])
        getattr(L, "orc_two_tap_vjp" + sfx).argtypes = (
            [_I64, _P, _I64, _I64, _P, _P, _P, _I64, _P, _P, _P, _P, _P, _P])
        getattr(L, "orc_two_tap_rollout" + sfx).restype = ctypes.c_int
        getattr(L, "orc_two_tap_rollout" + sfx).argtypes = (
            [_I64, _I64, _P, _I64, _I64, _I64, _P, _P, _P, _I64, _P, _P, _P, _P])
        getattr(L, "orc_two_tap_rollout_vjp" + sfx).argtypes = (
            [_I64, _I64, _P, _I64, _I64, _I64, _P, _P, _P, _I64, _P, _P, _P, _P, _P, _P, _P])
        getattr(L, "orc_philox4x32_10" + sfx).argtypes = [_P, _P, _P]
        getattr(L, "orc_series_log" + sfx).restype = ctypes.c_double
        getattr(L, "orc_series_log" + sfx).argtypes = [ctypes.c_double]
        getattr(L, "orc_unit_exponential" + sfx).restype = real
        getattr(L, "orc_unit_exponential" + sfx).argtypes = [
            ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32]
        getattr(L, "orc_netstim_init" + sfx).argtypes = [
            _I64, _P, _P, _P, _I32, ctypes.c_uint64, _P, _P, _P]
        getattr(L, "orc_netstim_run" + sfx).argtypes = [
            _I64, _I64, _I64, _D, _D, _P, _P, _P, ctypes.c_uint64, _P, _P, _P, _P]
    L.orc_num_threads.restype = ctypes.c_int


def _sfx(dtype) -> str:
    dtype = np.dtype(dtype)
    if dtype == np.float64:
        return "_f64"
    if dtype == np.float32:
        return "_f32"
    raise TypeError(f"oracle supports float32/float64, got {dtype}")


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def num_threads() -> int:
    return int(lib().orc_num_threads())


def vtrap(x, y, dtype=np.float64):
    f = getattr(lib(), "orc_vtrap" + _sfx(dtype))
    return np.array([f(float(a), float(b)) for a, b in np.broadcast(x, y)], dtype=dtype)


def phi1(z, dtype=np.float64):
    f = getattr(lib(), "orc_phi1" + _sfx(dtype))
    return np.array([f(float(a)) for a in np.ravel(z)], dtype=dtype)


def hh_rates(v, q10=1.0, dtype=np.float64):
    """Return (len(v), 6) rates m_a, m_b, h_a, h_b, n_a, n_b."""
    f = getattr(lib(), "orc_hh_rates" + _sfx(dtype))
    v = np.ravel(np.asarray(v, dtype=dtype))
    out = np.empty((v.size, 6), dtype=dtype)
    for i, vi in enumerate(v):
        f(float(vi), float(q10), out[i].ctypes.data_as(ctypes.c_void_p))
    return out


def hh_steady(v, dtype=np.float64):
    f = getattr(lib(), "orc_hh_steady" + _sfx(dtype))
    v = np.ravel(np.asarray(v, dtype=dtype))
    out = np.empty((v.size, 3), dtype=dtype)
    for i, vi in enumerate(v):
        f(float(vi), out[i].ctypes.data_as(ctypes.c_void_p))
    return out


def cnexp(x, a, b, dt, dtype=np.float64):
    f = getattr(lib(), "orc_cnexp" + _sfx(dtype))
    return np.array(
        [f(float(xi), float(ai), float(bi), float(dt)) for xi, ai, bi in np.broadcast(x, a, b)],
        dtype=dtype,
    )


def thomas(a, b, c, d):
    """Batched functional Thomas (reference pcr_solve_t) on (B,K) arrays."""
    dtype = b.dtype
    a, b, c, d = (np.ascontiguousarray(t, dtype=dtype) for t in (a, b, c, d))
    B, K = b.shape
    x = np.empty_like(d)
    getattr(lib(), "orc_thomas_batched" + _sfx(dtype))(
        B, K, _ptr(a), _ptr(b), _ptr(c), _ptr(d), _ptr(x))
    return x


def pcr(a, b, c, d):
    """Batched PCR (reference pcr_solve_parallel_t) on (B,K) arrays."""
    dtype = b.dtype
    a, b, c, d = (np.ascontiguousarray(t, dtype=dtype) for t in (a, b, c, d))
    B, K = b.shape
    x = np.empty_like(d)
    f = getattr(lib(), "orc_pcr" + _sfx(dtype))
    for i in range(B):
        f(K, _ptr(a[i]), _ptr(b[i]), _ptr(c[i]), _ptr(d[i]), _ptr(x[i]))
    return x


def block3_solve(lower, main, upper, rhs):
    """Block Thomas on (B, K) systems of 3x3 blocks (diagonal off-diagonal blocks)."""
    dtype = rhs.dtype
    lower, main, upper, rhs = (np.ascontiguousarray(t, dtype=dtype)
                               for t in (lower, main, upper, rhs))
    B, K = rhs.shape[:2]
    x = np.empty_like(rhs)
    getattr(lib(), "orc_block3_thomas" + _sfx(dtype))(
        B, K, _ptr(lower), _ptr(main), _ptr(upper), _ptr(rhs), _ptr(x))
    return x


def dhs_solve(d, a, b, parent, order, layer_ptr):
    """Sequential DHS solve of (B,K) systems in solver order."""
    dtype = d.dtype
    d, a, b = (np.ascontiguousarray(t, dtype=dtype) for t in (d, a, b))
    parent = np.ascontiguousarray(parent, dtype=np.int32)
    order = np.ascontiguousarray(order, dtype=np.int32)
    layer_ptr = np.ascontiguousarray(layer_ptr, dtype=np.int32)
    B, K = d.shape
    x = np.zeros_like(d)
    getattr(lib(), "orc_dhs_solve_batched" + _sfx(dtype))(
        B, K, _ptr(d), _ptr(a), _ptr(b), _ptr(parent), _ptr(order), _ptr(layer_ptr),
        int(layer_ptr.size - 1), _ptr(x))
    return x


def cable_run(p: dict, n_steps: int, rec_every: int = 1, t0_ms: float = 0.0,
              gate_f32: bool = False, record_all: bool = False, raster=None,
              raster_cap: int = 64, step0: int = 0):
    """Run the HH cable update on a packed problem dict (see dendra_gb300.cable).

    ``p`` holds numpy arrays: cable_ptr, v, m, h, n (modified in place),
    g_right, g_left, scale, cm_inv, field (or None), gnabar, gkbar, gl, el,
    ve_amp/ve_delay/ve_pw (or None), in_idx/in_amp/in_delay/in_pw (or None),
    rec_idx, spk_idx, and scalars ena, ek, q10, dt_ms, dt_s, spk_thr.
    ``gate_f32`` evaluates the pulse gates on a float32 time grid (how a
    float32 model sees its pulses) while the arithmetic stays in p's dtype.
    Returns (trace, spk_count, spk_first, spk_below).

    record_all / raster: with either, a fifth element is returned, a dict with
    ``trace_all`` (1 + n_steps // rec_every, N) of every compartment's v and,
    for ``raster`` ((B, R) local checked compartments, -1 none), ``rast_count``
    (B, R), ``rast_steps`` (B, R, raster_cap) absolute crossing steps
    (step0 + s + 1; -1 unused) and ``rast_below`` (B, R) latches.
    """
    dtype = p["v"].dtype
    sfx = _sfx(dtype)
    B = int(p["cable_ptr"].size - 1)
    n_rec = 1 + n_steps // rec_every
    trace = np.full((B, n_rec), np.nan, dtype=dtype)
    spk_below = p.get("spk_below")
    if spk_below is None:
        spk_below = np.ones(B, dtype=np.int32)
    spk_count = np.zeros(B, dtype=np.int32)
    spk_first = np.full(B, -1, dtype=np.int32)

    def arr(name, dt=dtype):
        x = p.get(name)
        if x is None:
            return None
        y = np.ascontiguousarray(x, dtype=dt)
        return y

    keep = {k: arr(k) for k in ("g_right", "g_left", "scale", "cm_inv", "field", "gnabar",
                                  "gkbar", "gl", "el", "ve_amp", "ve_delay", "ve_pw",
                                  "in_amp", "in_delay", "in_pw")}
    for k in ("in_idx", "rec_idx", "spk_idx", "spk_idx2"):
        keep[k] = arr(k, np.int32)
    spk_below2 = np.ones(B, dtype=np.int32)
    cable_ptr = np.ascontiguousarray(p["cable_ptr"], dtype=np.int64)
    N = int(cable_ptr[-1])
    trace_all = np.full((n_rec, N), np.nan, dtype=dtype) if record_all else None
    if raster is not None:
        r_idx = np.ascontiguousarray(raster, dtype=np.int32).reshape(B, -1)
    else:
        r_idx = np.zeros((B, 0), dtype=np.int32)
    R = r_idx.shape[1]
    r_below = np.ones((B, R), dtype=np.int32)
    r_count = np.zeros((B, R), dtype=np.int32)
    r_steps = np.full((B, R, max(int(raster_cap), 0)), -1, dtype=np.int64)
    getattr(lib(), "orc_cable_run" + sfx)(
        B, int(n_steps), int(rec_every), _ptr(cable_ptr),
        _ptr(p["v"]), _ptr(p["m"]), _ptr(p["h"]), _ptr(p["n"]),
        _ptr(keep["g_right"]), _ptr(keep["g_left"]), _ptr(keep["scale"]),
        _ptr(keep["cm_inv"]), _ptr(keep["field"]), _ptr(keep["gnabar"]),
        _ptr(keep["gkbar"]), _ptr(keep["gl"]), _ptr(keep["el"]),
        float(p["ena"]), float(p["ek"]), float(p["q10"]), float(p["dt_ms"]),
        float(p["dt_s"]), float(t0_ms),
        _ptr(keep["ve_amp"]), _ptr(keep["ve_delay"]), _ptr(keep["ve_pw"]),
        _ptr(keep["in_idx"]), _ptr(keep["in_amp"]), _ptr(keep["in_delay"]),
        _ptr(keep["in_pw"]), _ptr(keep["rec_idx"]), _ptr(trace),
        _ptr(keep["spk_idx"]), float(p.get("spk_thr", 0.0)), _ptr(spk_below),
        _ptr(spk_count), _ptr(spk_first), int(bool(gate_f32)), _ptr(keep["spk_idx2"]),
        _ptr(spk_below2), _ptr(trace_all), int(R), _ptr(r_idx), _ptr(r_below), _ptr(r_count),
        int(raster_cap), _ptr(r_steps), int(step0),
    )
    if not record_all and raster is None:
        return trace, spk_count, spk_first, spk_below
    extra = {"trace_all": trace_all, "rast_count": r_count, "rast_steps": r_steps,
             "rast_below": r_below}
    return trace, spk_count, spk_first, spk_below, extra


def cable_grad(p: dict, n_steps: int, trace_grad, rec_every: int = 1, t0_ms: float = 0.0,
               gate_f32: bool = False):
    """Reverse mode of ``cable_run`` for a trace functional.

    ``trace_grad`` (B, 1 + n_steps // rec_every) is dLoss/dtrace for the trace
    ``cable_run`` records from the same state.  Returns a dict with lam_v,
    lam_m, lam_h, lam_n (adjoint of the initial state), g_gnabar, g_gkbar,
    g_gl and g_axial (per compartment; g_axial is lam_g * g over the axial
    bands, so dLoss/dRa of a cable = -sum of its g_axial / Ra).  ``p``'s state arrays end at
    the final state, as after ``cable_run``.
    """
    dtype = p["v"].dtype
    sfx = _sfx(dtype)
    B = int(p["cable_ptr"].size - 1)
    N = int(p["v"].size)

    def arr(name, dt=dtype):
        x = p.get(name)
        return None if x is None else np.ascontiguousarray(x, dtype=dt)

    keep = {k: arr(k) for k in ("g_right", "g_left", "scale", "cm_inv", "field", "gnabar",
                                  "gkbar", "gl", "el", "ve_amp", "ve_delay", "ve_pw",
                                  "in_amp", "in_delay", "in_pw")}
    for k in ("in_idx", "rec_idx"):
        keep[k] = arr(k, np.int32)
    tg = np.ascontiguousarray(trace_grad, dtype=dtype)
    assert tg.shape == (B, 1 + n_steps // rec_every)
    out = {k: np.zeros(N, dtype=dtype) for k in ("lam_v", "lam_m", "lam_h", "lam_n", "g_gnabar",
                                                  "g_gkbar", "g_gl", "g_axial")}
    cable_ptr = np.ascontiguousarray(p["cable_ptr"], dtype=np.int64)
    getattr(lib(), "orc_cable_grad" + sfx)(
        B, int(n_steps), int(rec_every), _ptr(cable_ptr),
        _ptr(p["v"]), _ptr(p["m"]), _ptr(p["h"]), _ptr(p["n"]),
        _ptr(keep["g_right"]), _ptr(keep["g_left"]), _ptr(keep["scale"]),
        _ptr(keep["cm_inv"]), _ptr(keep["field"]), _ptr(keep["gnabar"]),
        _ptr(keep["gkbar"]), _ptr(keep["gl"]), _ptr(keep["el"]),
        float(p["ena"]), float(p["ek"]), float(p["q10"]), float(p["dt_ms"]),
        float(p["dt_s"]), float(t0_ms),
        _ptr(keep["ve_amp"]), _ptr(keep["ve_delay"]), _ptr(keep["ve_pw"]),
        _ptr(keep["in_idx"]), _ptr(keep["in_amp"]), _ptr(keep["in_delay"]),
        _ptr(keep["in_pw"]), _ptr(keep["rec_idx"]), _ptr(tg), int(bool(gate_f32)),
        *(_ptr(out[k]) for k in ("lam_v", "lam_m", "lam_h", "lam_n", "g_gnabar", "g_gkbar",
                                  "g_gl", "g_axial")),
    )
    return out


def net_run(pd: dict, n_steps: int):
    """Run the network oracle on a TreeNetwork.problem_dict (arrays updated in place).

    Returns the spike raster (n_steps, n_cells) uint8.
    """
    dtype = pd["v"].dtype
    sfx = _sfx(dtype)
    P = pd["plan"]
    nodes, syn, conn, prm = pd["nodes"], pd["syn"], pd["conn"], pd["params"]
    c = lambda x, dt=None: np.ascontiguousarray(x if dt is None else np.asarray(x, dtype=dt))
    keep = dict(
        node_ptr=c(P["node_ptr"], np.int64), plan_of=c(P["plan_of"], np.int32),
        plan_node_ptr=c(P["plan_node_ptr"], np.int64), plan_layer_off=c(P["plan_layer_off"], np.int64),
        parent=c(P["parent"], np.int32), order=c(P["order"], np.int32),
        layer_ptr=c(P["layer_ptr"], np.int32), child_ptr=c(P["child_ptr"], np.int32),
        child_idx=c(P["child_idx"], np.int32),
        area=c(nodes["area"], dtype), cm_dt=c(nodes["cm_dt"], dtype), a_geom=c(nodes["a_geom"], dtype),
        gl=c(nodes["gl"], dtype), el=c(nodes["el"], dtype),
        syn_ptr=c(pd["syn_ptr"], np.int64), node_syn_ptr=c(pd["node_syn_ptr"], np.int32),
        factor=c(syn["factor"], dtype), decay_A=c(syn["decay_A"], dtype),
        decay_B=c(syn["decay_B"], dtype),
        bg=None if pd["bg_bits"] is None else c(pd["bg_bits"], np.uint64),
        pre=c(conn["pre"], np.int64), post=c(conn["post"], np.int64),
        delay=c(conn["delay"], np.int64), weight=c(conn["weight"], dtype))
    drive = {k: (None if pd.get(k) is None else c(pd[k], np.int32 if k == "in_node" else dtype))
             for k in ("ve_field", "ve_amp", "ve_delay", "ve_pw", "in_node", "in_amp",
                       "in_delay", "in_pw")}
    slot = np.array([pd["slot"]], dtype=np.int64)
    raster = np.zeros((n_steps, pd["n_cells"]), dtype=np.uint8)
    getattr(lib(), "orc_net_run" + sfx)(
        int(pd["n_cells"]), int(n_steps), int(pd["step"]), int(pd["depth"]), _ptr(slot),
        int(pd["n_syn"]), _ptr(keep["node_ptr"]), _ptr(keep["plan_of"]), _ptr(keep["plan_node_ptr"]),
        _ptr(keep["plan_layer_off"]), _ptr(keep["parent"]), _ptr(keep["order"]),
        _ptr(keep["layer_ptr"]), _ptr(keep["child_ptr"]), _ptr(keep["child_idx"]),
        _ptr(pd["v"]), _ptr(keep["area"]), _ptr(keep["cm_dt"]), _ptr(keep["a_geom"]),
        _ptr(keep["gl"]), _ptr(keep["el"]), _ptr(pd["m"]), _ptr(pd["h"]), _ptr(pd["n"]),
        float(prm["gnabar"]), float(prm["gkbar"]), float(prm["ena"]), float(prm["ek"]),
        float(prm["q10"]), float(prm["dt_ms"]), float(prm["spk_thr"]),
        _ptr(keep["syn_ptr"]), _ptr(keep["node_syn_ptr"]), _ptr(pd["A"]), _ptr(pd["B"]),
        _ptr(keep["factor"]), _ptr(keep["decay_A"]), _ptr(keep["decay_B"]), float(prm["e_syn"]),
        _ptr(pd["ring"]), _ptr(keep["bg"]), int(pd["bg_words"]), int(pd["bg_syn"]),
        float(pd["bg_weight"]), int(keep["pre"].size), _ptr(keep["pre"]), _ptr(keep["post"]),
        _ptr(keep["delay"]), _ptr(keep["weight"]), _ptr(pd["below"]), _ptr(pd["spike_count"]),
        _ptr(raster), *(_ptr(drive[k]) for k in ("ve_field", "ve_amp", "ve_delay", "ve_pw",
                                                  "in_node", "in_amp", "in_delay", "in_pw")),
        float(pd.get("t0_ms", 0.0)))
    pd["slot"] = int(slot[0])
    return raster


# ---------------------------------------------------------------------------
# Interpolated delay transport (networks/_two_tap_enqueue_cpu.cpp,
# networks/_event_delivery.py:229-308)
# ---------------------------------------------------------------------------
def _edges(dtype, weights, gates, fraction, pre_idx):
    w = np.ascontiguousarray(weights, dtype=dtype)
    g = np.ascontiguousarray(gates, dtype=dtype)
    f = np.ascontiguousarray(fraction, dtype=dtype)
    pre = None if pre_idx is None else np.ascontiguousarray(pre_idx, dtype=np.int64)
    n_src = 0 if pre is None else int(g.shape[-1])
    return w, g, f, pre, n_src


def two_tap_enqueue(queue, slot, weights, gates, fraction, lower, upper, pre_idx=None):
    """ordered_two_tap_enqueue: returns (new queue, delivered row of slot)."""
    ring = np.array(queue, copy=True, order="C")
    dtype = ring.dtype
    depth, width = ring.shape
    w, g, f, pre, n_src = _edges(dtype, weights, gates, fraction, pre_idx)
    lower = np.ascontiguousarray(lower, dtype=np.int64)
    upper = np.ascontiguousarray(upper, dtype=np.int64)
    payload = np.empty(width, dtype)
    rc = getattr(lib(), "orc_two_tap_enqueue" + _sfx(dtype))(
        depth, width, _ptr(ring), int(slot), w.size, _ptr(w), _ptr(g), _ptr(pre), n_src,
        _ptr(f), _ptr(lower), _ptr(upper), _ptr(payload))
    if rc:
        raise IndexError("two-tap address, source or slot outside the ring")
    return ring, payload


def three_tap_enqueue(queue, slot, weights, gates, coeff, offsets, post_idx, pre_idx=None):
    """Three-tap branch of dense_interpolated_delay_transition (edge-major order)."""
    ring = np.array(queue, copy=True, order="C")
    dtype = ring.dtype
    depth, width = ring.shape
    w, g, c, pre, n_src = _edges(dtype, weights, gates, coeff, pre_idx)
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    post = np.ascontiguousarray(post_idx, dtype=np.int64)
    payload = np.empty(width, dtype)
    rc = getattr(lib(), "orc_three_tap_enqueue" + _sfx(dtype))(
        depth, width, _ptr(ring), int(slot), w.size, _ptr(w), _ptr(g), _ptr(pre), n_src,
        _ptr(c), _ptr(offsets), _ptr(post), _ptr(payload))
    if rc:
        raise IndexError("three-tap post, source or slot outside the ring")
    return ring, payload


def two_tap_vjp(ring, offset, weights, gates, fraction, lower, upper, pre_idx=None):
    """delay_ring_two_tap_vjp: (grad_weights, grad_gates, grad_fraction)."""
    R = np.ascontiguousarray(ring)
    dtype = R.dtype
    w, g, f, pre, n_src = _edges(dtype, weights, gates, fraction, pre_idx)
    lower = np.ascontiguousarray(lower, dtype=np.int64)
    upper = np.ascontiguousarray(upper, dtype=np.int64)
    dw, df, dg = np.empty_like(w), np.empty_like(f), np.empty_like(g)
    getattr(lib(), "orc_two_tap_vjp" + _sfx(dtype))(
        R.size, _ptr(R), int(offset), w.size, _ptr(w), _ptr(g), _ptr(pre), n_src, _ptr(f),
        _ptr(lower), _ptr(upper), _ptr(dw), _ptr(dg), _ptr(df))
    return dw, dg, df


def two_tap_rollout(queue, slot0, weights, gates, fraction, lower, upper, pre_idx=None):
    """n_steps = len(gates) steps: returns (final queue, payload[n_steps][width])."""
    ring = np.array(queue, copy=True, order="C")
    dtype = ring.dtype
    depth, width = ring.shape
    w, g, f, pre, n_src = _edges(dtype, weights, gates, fraction, pre_idx)
    lower = np.ascontiguousarray(lower, dtype=np.int64)
    upper = np.ascontiguousarray(upper, dtype=np.int64)
    n_steps = g.shape[0]
    payload = np.empty((n_steps, width), dtype)
    rc = getattr(lib(), "orc_two_tap_rollout" + _sfx(dtype))(
        depth, width, _ptr(ring), int(slot0), n_steps, w.size, _ptr(w), _ptr(g), _ptr(pre),
        n_src, _ptr(f), _ptr(lower), _ptr(upper), _ptr(payload))
    if rc:
        raise IndexError("two-tap address, source or slot outside the ring")
    return ring, payload


def two_tap_rollout_vjp(grad_queue, slot0, weights, gates, fraction, lower, upper,
                        grad_payload, pre_idx=None):
    """Reverse of two_tap_rollout: (grad_queue0, grad_weights, grad_gates, grad_fraction)."""
    R = np.array(grad_queue, copy=True, order="C")
    dtype = R.dtype
    depth, width = R.shape
    w, g, f, pre, n_src = _edges(dtype, weights, gates, fraction, pre_idx)
    lower = np.ascontiguousarray(lower, dtype=np.int64)
    upper = np.ascontiguousarray(upper, dtype=np.int64)
    gp = np.ascontiguousarray(grad_payload, dtype=dtype)
    n_steps = g.shape[0]
    dw, df, dg = np.zeros_like(w), np.zeros_like(f), np.empty_like(g)
    getattr(lib(), "orc_two_tap_rollout_vjp" + _sfx(dtype))(
        depth, width, _ptr(R), int(slot0), n_steps, w.size, _ptr(w), _ptr(g), _ptr(pre), n_src,
        _ptr(f), _ptr(lower), _ptr(upper), _ptr(gp), _ptr(dw), _ptr(dg), _ptr(df))
    return R, dw, dg, df


# ---------------------------------------------------------------------------
# NetStim renewal (networks/_netstim_renewal.py:70-159)
# ---------------------------------------------------------------------------
def philox4x32_10(counter, key):
    """Philox4x32-10 block: 4 x uint32 counter, 2 x uint32 key -> 4 x uint32."""
    c = np.ascontiguousarray(counter, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.empty(4, np.uint32)
    lib().orc_philox4x32_10_f64(_ptr(c), _ptr(k), _ptr(out))
    return out


def series_log(x):
    return float(lib().orc_series_log_f64(float(x)))


def unit_exponential(seed, step, gen, stream=0, dtype=np.float64):
    return getattr(lib(), "orc_unit_exponential" + _sfx(dtype))(seed, step, gen, stream)


def netstim_init(interval, noise, start, seed=0, draws=None, dtype=np.float64):
    """(next_time, counts) of netstim_initial_state."""
    iv, nz, st = (np.ascontiguousarray(a, dtype=dtype) for a in (interval, noise, start))
    n = iv.size
    d = None if draws is None else np.ascontiguousarray(draws, dtype=dtype)
    nxt = np.empty(n, dtype)
    cnt = np.empty(n, np.int64)
    getattr(lib(), "orc_netstim_init" + _sfx(dtype))(
        n, _ptr(iv), _ptr(nz), _ptr(st), int(bool((nz > 0).any())), seed, _ptr(d), _ptr(nxt),
        _ptr(cnt))
    return nxt, cnt


def netstim_run(next_time, counts, n_steps, interval, noise, number=None, step0=0, t0=0.0,
                dt=0.025, seed=0, draws=None):
    """n_steps renewal steps: returns (next_time, counts, spikes[n_steps][n])."""
    nxt = np.array(next_time, copy=True)
    dtype = nxt.dtype
    cnt = np.array(counts, dtype=np.int64, copy=True)
    iv, nz = (np.ascontiguousarray(a, dtype=dtype) for a in (interval, noise))
    num = None if number is None else np.ascontiguousarray(number, dtype=np.int64)
    d = None if draws is None else np.ascontiguousarray(draws, dtype=dtype)
    n = nxt.size
    spikes = np.empty((n_steps, n), np.uint8)
    getattr(lib(), "orc_netstim_run" + _sfx(dtype))(
        n, n_steps, step0, float(t0), float(dt), _ptr(iv), _ptr(nz), _ptr(num), seed, _ptr(d),
        _ptr(nxt), _ptr(cnt), _ptr(spikes))
    return nxt, cnt, spikes


# ---------------------------------------------------------------------------
# 3x3 block tree solve (triton/dhs_kernel_bt.py: the matrix its kernel factors)
# ---------------------------------------------------------------------------
def dhs_block3_matrix(D, G, parent):
    """Dense (B, 3K, 3K) matrices: A_ii = D_i + diag(g_i) + sum_children diag(g_c),
    A_ic = A_ci = -diag(g_c)."""
    D = np.asarray(D, dtype=np.float64)
    G = np.asarray(G, dtype=np.float64)
    B, K = G.shape[:2]
    A = np.zeros((B, 3 * K, 3 * K))
    for i in range(K):
        A[:, 3 * i:3 * i + 3, 3 * i:3 * i + 3] += D[:, i] + np.einsum("bj,jk->bjk", G[:, i],
                                                                        np.eye(3))
    for c, p in enumerate(parent):
        if p < 0:
            continue
        for r in range(3):
            A[:, 3 * p + r, 3 * p + r] += G[:, c, r]
            A[:, 3 * c + r, 3 * p + r] -= G[:, c, r]
            A[:, 3 * p + r, 3 * c + r] -= G[:, c, r]
    return A


def dhs_block3_solve(D, G, b, parent):
    """Dense solve of the block tree systems, (B, K, 3) solutions (float64)."""
    A = dhs_block3_matrix(D, G, parent)
    B, K = np.asarray(b).shape[:2]
    return np.linalg.solve(A, np.asarray(b, dtype=np.float64).reshape(B, 3 * K, 1)).reshape(
        B, K, 3)


# ---------------------------------------------------------------------------
# SPD block Thomas (triton/bt_spd_kernel.py:9-370), restated in numpy
# ---------------------------------------------------------------------------
def _spd_mid(a, b, dt):
    fi = np.finfo(dt)
    hm, tt = fi.max / 2, 2 * fi.tiny
    bounded = (np.abs(a) <= hm) & (np.abs(b) <= hm)
    extreme = np.where(np.abs(a) < tt, a + 0.5 * b,
                       np.where(np.abs(b) < tt, 0.5 * a + b, 0.5 * a + 0.5 * b))
    return np.where(bounded, 0.5 * (a + b), extreme)


def _chol3(a):
    c0 = a[..., 0] > 0
    l00 = np.sqrt(np.where(c0, a[..., 0], 1.0))
    l10, l20 = a[..., 1] / l00, a[..., 2] / l00
    s11 = a[..., 4] - l10 * l10
    c1 = s11 > 0
    l11 = np.sqrt(np.where(c1, s11, 1.0))
    l21 = (a[..., 5] - l10 * l20) / l11
    s22 = a[..., 8] - l20 * l20 - l21 * l21
    c2 = s22 > 0
    l22 = np.sqrt(np.where(c2, s22, 1.0))
    z = np.zeros_like(l00)
    L = np.stack([l00, z, z, l10, l11, z, l20, l21, l22], -1)
    return L, c0 & c1 & c2


def _chol3_bumped(a, eps_rel, eps_abs):
    a = a.copy()
    for i, j in ((1, 3), (2, 6), (5, 7)):
        m = _spd_mid(a[..., i], a[..., j], a.dtype)
        a[..., i] = m
        a[..., j] = m
    L1, s1 = _chol3(a)
    tr = np.abs(a[..., 0]) + np.abs(a[..., 4]) + np.abs(a[..., 8])
    g = np.stack([a[..., 0] - (np.abs(a[..., 1]) + np.abs(a[..., 2])),
                  a[..., 4] - (np.abs(a[..., 3]) + np.abs(a[..., 5])),
                  a[..., 8] - (np.abs(a[..., 6]) + np.abs(a[..., 7]))], -1).min(-1)
    margin = np.maximum(eps_abs, eps_rel * tr)
    tau = np.where(g > 0, margin, -g + margin)
    b = a.copy()
    for q in (0, 4, 8):
        b[..., q] = a[..., q] + tau
    L2, s2 = _chol3(b)
    for q in (0, 4, 8):
        b[..., q] = b[..., q] + 10.0 * margin
    L3, s3 = _chol3(b)
    L = np.where(s1[..., None], L1, np.where(s2[..., None], L2, L3))
    return L, s1 | s2 | s3


def _chol_solve3(L, b):
    y0 = b[..., 0] / L[..., 0]
    y1 = (b[..., 1] - L[..., 3] * y0) / L[..., 4]
    y2 = (b[..., 2] - L[..., 6] * y0 - L[..., 7] * y1) / L[..., 8]
    x2 = y2 / L[..., 8]
    x1 = (y1 - L[..., 7] * x2) / L[..., 4]
    x0 = (y0 - L[..., 3] * x1 - L[..., 6] * x2) / L[..., 0]
    return np.stack([x0, x1, x2], -1)


def block3_spd_solve(lower, main, upper, rhs):
    """(x, info) of the SPD block Thomas with symmetrisation and diagonal shifts."""
    dt = np.asarray(rhs).dtype
    eps_rel, eps_abs = (1e-12, 1e-30) if dt == np.float64 else (1e-6, 1e-18)
    lower, upper, rhs = (np.asarray(t, dtype=dt) for t in (lower, upper, rhs))
    M = np.asarray(main, dtype=dt).reshape(rhs.shape[0], rhs.shape[1], 9)
    B, K = rhs.shape[:2]
    Ls, info, d = [], np.zeros((B, K), np.int32), [rhs[:, 0].copy()]
    L, ok = _chol3_bumped(M[:, 0], eps_rel, eps_abs)
    info[:, 0] = ~ok
    Ls.append(L)
    for k in range(1, K):
        u, lo = upper[:, k - 1], lower[:, k - 1]
        cols = [_chol_solve3(L, np.stack([u[:, 0] * (j == 0), u[:, 1] * (j == 1),
                                          u[:, 2] * (j == 2)], -1).astype(dt)) for j in range(3)]
        a = M[:, k].copy()
        for r in range(3):
            for c in range(3):
                a[:, r * 3 + c] = M[:, k, r * 3 + c] - lo[:, r] * cols[c][:, r]
        t = _chol_solve3(L, d[-1])
        d.append(rhs[:, k] - lo * t)
        L, ok = _chol3_bumped(a, eps_rel, eps_abs)
        info[:, k] = ~ok
        Ls.append(L)
    x = np.empty_like(rhs)
    xn = _chol_solve3(Ls[-1], d[-1])
    x[:, -1] = xn
    for k in range(K - 2, -1, -1):
        xn = _chol_solve3(Ls[k], d[k] - upper[:, k] * xn)
        x[:, k] = xn
    return x, info


def _schur(left, right, pivot):
    """small * (large / pivot) of the pair, by magnitude (the conductance-form
    Schur product of models/integrators/triton/tree_contraction.py:22-30)."""
    left_small = np.abs(left) < np.abs(right)
    small = np.where(left_small, left, right)
    large = np.where(left_small, right, left)
    return small * (large / pivot)


def tree_contract_solve(d, g, rhs, tables):
    """Tree-contraction solve of (B, K) Hines systems, numpy restatement.

    Follows models/integrators/triton/tree_contraction.py: segment
    condensation (_condense_segment_tile :237-287), endpoint gather
    (_gather_segment_tile :290-328), rounds of updates (_update :33-74,
    _solve_contracted_tree :110-178), recovery (_recover :77-107,
    _recover_segment_tile :331-361), on the plan tables of
    ``dendra_gb300.contraction.build_contraction_tables`` (the reference's
    plan comes from the dendra-solvers package, absent here).  Every
    operation is a single correctly rounded numpy operation in the input
    dtype, in the kernel's order.
    """
    d, g, rhs = (np.asarray(a) for a in (d, g, rhs))
    dt = d.dtype
    B, K = d.shape
    T = {k: np.asarray(v, dtype=np.int64) for k, v in tables.items()}
    seg, interior, retained = T["seg"], T["interior"], T["retained"]
    S, R = seg.shape[1], retained.shape[1]
    zero = np.zeros(B, dtype=dt)
    out = np.zeros((B, K), dtype=dt)
    saved = np.zeros((B, max(1, interior.size)), dtype=dt)
    pivots = np.ones_like(saved)
    bridges = np.zeros_like(saved)
    summ = np.zeros((5, B, max(1, S)), dtype=dt)
    for s in range(S):
        child, a0, a1 = retained[0, seg[1, s]], seg[2, s], seg[3, s]
        near = g[:, interior[a0]]
        left_d, left_r, carry_d, carry_r = zero, zero, zero, zero
        for pos in range(a0, a1):
            node = interior[pos]
            succ = interior[pos + 1] if pos + 1 < a1 else child
            far = g[:, succ]
            shunt = d[:, node] + carry_d
            value = rhs[:, node] + carry_r
            pivot = shunt + (near + far)
            saved[:, pos], pivots[:, pos], bridges[:, pos] = value, pivot, near
            left_d = left_d + _schur(near, shunt, pivot)
            left_r = left_r + (near / pivot) * value
            carry_d = _schur(far, shunt, pivot)
            carry_r = (far / pivot) * value
            near = _schur(near, far, pivot)
        summ[:, :, s] = (left_d, left_r, carry_d, carry_r, near)
    U = T["update"].shape[1]
    n_br = (T["incidence"][3].max() + 1 - R) if T["incidence"].size else 0
    st_s = np.zeros((B, R + U), dtype=dt)
    st_r = np.zeros((B, R + U), dtype=dt)
    edge = np.zeros((B, R + max(int(n_br), 0)), dtype=dt)
    ep = T["endpoint"]
    for r in range(R):
        node, inc, e0, ne = retained[:, r]
        diag, val = d[:, node], rhs[:, node]
        for e in range(e0, e0 + ne):
            s, side = ep[0, e], ep[1, e]
            diag = diag + summ[2 * side, :, s]
            val = val + summ[2 * side + 1, :, s]
        st_s[:, r], st_r[:, r] = diag, val
        edge[:, r] = summ[4, :, inc] if inc >= 0 else g[:, node]
    rp, upd, inc = T["round_ptr"], T["update"], T["incidence"]
    P = rp.shape[1] - 1
    for p in range(P):
        for u in range(rp[0, p], rp[0, p + 1]):
            src, q0, nq = upd[:, u]
            diag, val = st_s[:, src], st_r[:, src]
            for q in range(q0, q0 + nq):
                m, ns, fs, dest = inc[:, q]
                shunt, value, near = st_s[:, m], st_r[:, m], edge[:, ns]
                far = edge[:, fs] if fs >= 0 else zero
                pivot = shunt + (near + far)
                diag = diag + _schur(near, shunt, pivot)
                val = val + (near / pivot) * value
                if dest >= 0:
                    edge[:, dest] = _schur(near, far, pivot)
            st_s[:, R + u], st_r[:, R + u] = diag, val
    xr = np.zeros((B, R), dtype=dt)
    roots = T["roots"]
    for k in range(roots.shape[1]):
        r, st = roots[:, k]
        xr[:, r] = st_r[:, st] / (st_s[:, st] + edge[:, r])
    rec = T["recovery"]
    for p in range(P - 1, -1, -1):
        for e in range(rp[1, p], rp[1, p + 1]):
            node, st, a, c, ns, fs = rec[:, e]
            near = edge[:, ns]
            far = edge[:, fs] if fs >= 0 else zero
            xc = xr[:, c] if c >= 0 else zero
            pivot = st_s[:, st] + (near + far)
            xr[:, node] = ((st_r[:, st] + near * xr[:, a]) + far * xc) / pivot
    out[:, retained[0]] = xr
    for s in range(S):
        anc, succ = retained[0, seg[0, s]], retained[0, seg[1, s]]
        a0, a1 = seg[2, s], seg[3, s]
        xa, xs = out[:, anc], out[:, succ]
        for pos in range(a1 - 1, a0 - 1, -1):
            node = interior[pos]
            x = ((saved[:, pos] + bridges[:, pos] * xa) + g[:, succ] * xs) / pivots[:, pos]
            out[:, node] = x
            succ, xs = node, x
    return out


def hines_matrix(d, g, parent):
    """Dense matrix of one scalar Hines system (conductance form: shunt d_i,
    edge g_i to the parent, a root's g_i a second shunt)."""
    K = len(parent)
    A = np.diag(np.asarray(d, dtype=np.float64) + np.asarray(g, dtype=np.float64))
    for i in range(K):
        p = parent[i]
        if p >= 0:
            A[p, p] += g[i]
            A[i, p] -= g[i]
            A[p, i] -= g[i]
    return A
