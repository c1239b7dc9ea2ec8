"""ctypes binding of the C ABI in ``include/dendra_gb300.h``.

The library is the only compute path: if it cannot be built or loaded the
import of a kernel-facing function raises, there is no CPU fallback.
"""

from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None

F32 = 0
F64 = 1
THOMAS = 0
PCR = 1
CABLE_UNIFORM_CHANNELS = 1
CABLE_UNIFORM_GEOMETRY = 2
CABLE_FAST_MATH = 4
CABLE_STOP_ON_SPIKE = 8
CABLE_SPLIT_GATES = 16

_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_D = ctypes.c_double
_INT = ctypes.c_int


class DgbError(RuntimeError):
    """A dendra_gb300 C-ABI call returned an error code."""


class DgbTimeout(DgbError):
    """A bounded device-side wait gave up (DGB_ETIMEOUT)."""


class CableArgs(ctypes.Structure):
    """Mirror of ``dgb_cable_args`` (field order and types must match)."""

    _fields_ = [
        ("dtype", _I32), ("n_cables", _I32), ("n_steps", _I32), ("rec_every", _I32),
        ("cable_ptr", _P), ("order", _P),
        ("v", _P), ("m", _P), ("h", _P), ("n", _P),
        ("g_right", _P), ("g_left", _P), ("scale", _P), ("cm_inv", _P), ("field", _P),
        ("gnabar", _P), ("gkbar", _P), ("gl", _P), ("el", _P),
        ("ena", _D), ("ek", _D), ("q10", _D), ("dt_ms", _D), ("dt_s", _D), ("t0_ms", _D),
        ("step0", _I64),
        ("ve_amp", _P), ("ve_delay", _P), ("ve_pw", _P),
        ("in_idx", _P), ("in_amp", _P), ("in_delay", _P), ("in_pw", _P),
        ("rec_idx", _P), ("trace", _P),
        ("spk_idx", _P), ("spk_thr", _D), ("spk_below", _P), ("spk_count", _P),
        ("spk_first", _P), ("spk_idx2", _P), ("spk_below2", _P),
        ("max_k", _I32), ("flags", _I32), ("n_comp", _I64),
        ("comp_cable", _P), ("scratch", _P), ("warps_per_block", _I32), ("n_rast", _I32),
        ("rast_idx", _P), ("rast_below", _P), ("rast_count", _P), ("rast_steps", _P),
        ("rast_cap", _I32), ("lanes_mode", _I32), ("n_lanes32", _I32), ("n_lanes16", _I32),
        ("trace_all", _P),
    ]


class CableAdjointArgs(ctypes.Structure):
    """Mirror of ``dgb_cable_adjoint_args``."""

    _fields_ = [
        ("tape", _P), ("trace_grad", _P), ("trace_len", _I64),
        ("lam_v", _P), ("lam_m", _P), ("lam_h", _P), ("lam_n", _P),
        ("grad_gnabar", _P), ("grad_gkbar", _P), ("grad_gl", _P), ("grad_axial", _P),
    ]


# name -> (restype, argtypes); every symbol declared in include/dendra_gb300.h
SIGNATURES = {
    "dgb_version": (ctypes.c_char_p, []),
    "dgb_last_error": (ctypes.c_char_p, []),
    "dgb_cable_args_size": (ctypes.c_size_t, []),
    "dgb_tridiag_solve": (_INT, [_INT, _INT, _I64, _I64, _P, _P, _P, _P, _P, _P]),
    "dgb_tridiag_solve_lanes": (_INT, [_INT, _I64, _I64, _P, _P, _P, _P, _P, _I32, _P]),
    "dgb_tridiag_solve_transpose": (_INT, [_INT, _I64, _I64, _P, _P, _P, _P, _P, _P]),
    "dgb_tridiag_status": (_INT, [_P]),
    "dgb_tridiag_set_wait_limit": (_INT, [_I64]),
    "dgb_cable_adjoint_set_wait_limit": (_INT, [_I64]),
    "dgb_block3_solve": (_INT, [_INT, _I64, _I64, _P, _P, _P, _P, _P, _P, _I32, _P]),
    "dgb_block3_work_size": (ctypes.c_size_t, [_INT, _I64, _I64]),
    "dgb_cable_run": (_INT, [ctypes.POINTER(CableArgs), _P]),
    "dgb_cable_assemble": (_INT, [ctypes.POINTER(CableArgs), _I32, _P, _P, _P, _P, _P]),
    "dgb_cable_solve_update": (_INT, [ctypes.POINTER(CableArgs), _P, _P, _P, _P, _P]),
    "dgb_cable_step_static": (_INT, [ctypes.POINTER(CableArgs), _I32, _P]),
    "dgb_cable_run_taped": (_INT, [ctypes.POINTER(CableArgs), _P, _P]),
    "dgb_cable_adjoint": (_INT, [ctypes.POINTER(CableArgs), ctypes.POINTER(CableAdjointArgs), _P]),
    "dgb_cable_adjoint_args_size": (ctypes.c_size_t, []),
    "dgb_dhs_solve": (_INT, [_INT, _I64, _I64, _P, _P, _P, _P, _P, _P, _I32, _P, _P, _P, _P]),
    "dgb_dhs_solve_forest": (_INT, [_INT, _P, _P, _P, _P, _P, _P]),
    "dgb_detect_spikes": (_INT, [_INT, _P, _P, _I64, _D, _P, _P, _P]),
    "dgb_pack_source_spikes": (_INT, [_P, _I64, _P, _I64, _P, _P]),
    "dgb_build_delivery": (_INT, [_INT, _P, _P, _P, _P, _P, _P, _I64, _P, _P, _I64, _I64, _I64,
                                  _P]),
    "dgb_build_delivery_uniform": (_INT, [_INT, _P, _P, _I64, _P, _P, _P, _I64, _P, _P, _I64,
                                          _I64, _I64, _P]),
    "dgb_ring_enqueue": (_INT, [_INT, _P, _I64, _I64, _P, _P, _I64, _P, _P, _P, _P, _P, _P]),
    "dgb_net_window": (_INT, [_P, _P]),
    "dgb_net_enqueue": (_INT, [_INT, _P, _I64, _I64, _I64, _P, _I64, _P, _P, _P, _P, _P, _P]),
    "dgb_net_args_size": (ctypes.c_size_t, []),
    "dgb_mlp_gemm": (_INT, [_I32, _I32, _I32, _P, _I64, _I64, _P, _I64, _I64, _P, _I32, _P, _P,
                            _P, _P]),
    "dgb_mlp_gemm_path": (_INT, [_I32, _I32, _I32, _P, _I64, _I64, _P, _I64, _I64]),
    "dgb_mlp_gemm_status": (_INT, [_P]),
    "dgb_mlp_gemm_set_wait_limit": (_INT, [_I64]),
    "dgb_colsum": (_INT, [_I32, _I32, _P, _P, _P]),
    "dgb_adam": (_INT, [_I64, _I32, _I32, _P, _P, _P, _P, ctypes.c_float, ctypes.c_float,
                        ctypes.c_float, ctypes.c_float, _I32, _P, _P, _P]),
    "dgb_mse_grad": (_INT, [_I64, _P, _P, ctypes.c_float, _P, _P, _P]),
    "dgb_two_tap_enqueue": (_INT, [_INT, _P, _I64, _I64, _P, _I64, _P, _P, _P, _I64, _P, _P,
                                   _P, _P, _P, _P, _P, _P, _P]),
    "dgb_three_tap_enqueue": (_INT, [_INT, _P, _I64, _I64, _P, _I64, _P, _P, _P, _I64, _P, _P,
                                     _P, _P, _P, _P, _P]),
    "dgb_two_tap_gather": (_INT, [_INT, _P, _I64, _P, _I64, _P, _P, _P, _P, _P]),
    "dgb_two_tap_vjp": (_INT, [_INT, _P, _I64, _P, _I64, _P, _P, _P, _I64, _P, _P, _P, _P, _P,
                               _P, _P, _P, _P]),
    "dgb_three_tap_vjp": (_INT, [_INT, _P, _I64, _I64, _P, _I64, _P, _P, _P, _P, _P, _P, _P,
                                 _P, _P]),
    "dgb_two_tap_rollout": (_INT, [_INT, _P, _I64, _I64, _P, _I64, _I64, _P, _P, _I64, _P,
                                   _I64, _P, _P, _P, _P, _P, _I32, _P, _P]),
    "dgb_two_tap_rollout_vjp": (_INT, [_INT, _P, _I64, _I64, _P, _I64, _I64, _P, _P, _I64, _P,
                                       _I64, _P, _P, _P, _P, _P, _I32, _P, _P, _P, _I32, _P, _P,
                                       _P, _P, _P]),
    "dgb_gates_by_source": (_INT, [_INT, _I64, _I64, _P, _P, _I64, _P]),
    "dgb_delay_status": (_INT, [_P]),
    "dgb_block3_spd_solve": (_INT, [_INT, _I64, _I64, _P, _P, _P, _P, _P, _P, _P, _P]),
    "dgb_block3_spd_solve_chol": (_INT, [_INT, _I64, _I64, _P, _P, _P, _P, _P, _P]),
    "dgb_dhs_block3_solve": (_INT, [_INT, _I64, _I64, _P, _P, _P, _P, _P, _P, _I32, _P, _P, _P,
                                    _I32, _P]),
    "dgb_tree_contract_solve": (_INT, [_INT, _I64, _P, _P, _P, _P, _P, _P, ctypes.c_size_t, _P]),
    "dgb_tree_contract_work_size": (ctypes.c_size_t, [_INT, _P, _I64]),
    "dgb_contract_plan_size": (ctypes.c_size_t, []),
    "dgb_netstim_init": (_INT, [_INT, _I64, _P, _P, _P, _I32, ctypes.c_uint64, _P, _P, _P, _P]),
    "dgb_netstim_run": (_INT, [_INT, _I64, _I64, _I64, ctypes.c_double, ctypes.c_double, _P, _P,
                               _P, ctypes.c_uint64, _P, _P, _P, _P, _P, _I64, _P]),
}


def _declare(L):
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def path() -> str:
    return _build.LIB


def load():
    """Build (if stale) and load the CUDA library; raise if that fails."""
    global _lib
    with _lock:
        if _lib is None:
            try:
                so = _build.build()
            except Exception as exc:  # no silent fallback: the kernels are the product
                raise DgbError(f"dendra_gb300 CUDA library could not be built: {exc}") from exc
            if not os.path.exists(so):
                raise DgbError(f"dendra_gb300 CUDA library missing at {so}")
            L = ctypes.CDLL(so)
            _declare(L)
            _lib = L
    return _lib


def check(rc: int, what: str) -> None:
    if rc != 0:
        msg = load().dgb_last_error().decode(errors="replace")
        kind = {-1: ValueError, -4: ValueError}.get(rc)
        if kind is not None:
            raise kind(f"{what}: {msg}")
        if rc == -3:
            raise DgbTimeout(f"{what} timed out (code {rc}): {msg}")
        raise DgbError(f"{what} failed (code {rc}): {msg}")


def stream_ptr(device=None) -> int:
    import torch

    return torch.cuda.current_stream(device).cuda_stream


def dtype_code(dtype) -> int:
    import torch

    if dtype == torch.float32:
        return F32
    if dtype == torch.float64:
        return F64
    raise TypeError("dendra_gb300 kernels support only float32 and float64")
