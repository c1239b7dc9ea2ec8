"""The C-ABI library builds, loads and exports every declared symbol (CPU only)."""

import ctypes
import os
import re
import subprocess

import pytest

import dendra_gb300
from dendra_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))
           if f.endswith(".h")]


def _declared():
    names = set()
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(dgb_\w+)\s*\(", text))
    return sorted(names)


def test_header_declares_entry_points():
    names = _declared()
    assert "dgb_tridiag_solve" in names and "dgb_cable_run" in names


def test_library_exports_every_declared_symbol():
    L = dendra_gb300.load()
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.path()], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\b(dgb_\w+)\b", out))
    missing = [n for n in _declared() if n not in exported]
    assert not missing, missing
    for n in _declared():
        assert hasattr(L, n)
    # every declared function has a ctypes signature in the binding
    assert set(_declared()) <= set(_lib.SIGNATURES)


def test_cable_args_mirror_matches_c_layout():
    L = dendra_gb300.load()
    assert L.dgb_cable_args_size() == ctypes.sizeof(_lib.CableArgs)


def test_cable_adjoint_args_mirror_matches_c_layout():
    L = dendra_gb300.load()
    assert L.dgb_cable_adjoint_args_size() == ctypes.sizeof(_lib.CableAdjointArgs)


def test_net_args_mirror_matches_c_layout():
    from dendra_gb300.network import NetArgs

    L = dendra_gb300.load()
    assert L.dgb_net_args_size() == ctypes.sizeof(NetArgs)


def test_library_has_no_torch_dependency():
    out = subprocess.run(["readelf", "-d", _lib.path()], capture_output=True, text=True,
                         check=True).stdout
    assert "torch" not in out and "c10" not in out


def test_argument_errors_are_reported_without_touching_a_device():
    L = dendra_gb300.load()
    rc = L.dgb_tridiag_solve(7, 0, 1, 4, None, None, None, None, None, None)
    assert rc == -1
    assert b"dtype" in L.dgb_last_error()
    rc = L.dgb_tridiag_solve(0, 0, 1, 0, None, None, None, None, None, None)
    assert rc == -1 and b"K >= 1" in L.dgb_last_error()
    args = _lib.CableArgs()
    args.dtype = 3
    assert L.dgb_cable_run(ctypes.byref(args), None) == -1
    with pytest.raises(ValueError):
        _lib.check(-1, "probe")


def test_taped_run_and_adjoint_reject_bad_arguments_on_the_host():
    """Validation happens before any device work (the pointers are never read)."""
    L = dendra_gb300.load()
    a = _lib.CableArgs()
    a.dtype, a.n_cables, a.n_steps, a.rec_every, a.max_k, a.n_comp = 0, 1, 4, 1, 11, 11
    for name in ("cable_ptr", "v", "m", "h", "n", "g_right", "g_left", "scale", "cm_inv",
                 "gnabar", "gkbar", "gl", "el", "scratch"):
        setattr(a, name, 4096)
    a.flags = _lib.CABLE_STOP_ON_SPIKE
    assert L.dgb_cable_run_taped(ctypes.byref(a), 4096, None) == -1
    assert b"not accepted" in L.dgb_last_error()
    adj = _lib.CableAdjointArgs()
    assert L.dgb_cable_adjoint(ctypes.byref(a), ctypes.byref(adj), None) == -1
    a.flags = 0
    assert L.dgb_cable_adjoint(ctypes.byref(a), ctypes.byref(adj), None) == -1
    assert b"tape" in L.dgb_last_error()
    adj.tape = 4096
    assert L.dgb_cable_adjoint(ctypes.byref(a), ctypes.byref(adj), None) == -1
    assert b"lam_v" in L.dgb_last_error()


def test_block3_contract_errors_on_the_host():
    import torch

    from dendra_gb300.solvers import validate_block_tridiagonal

    lo = torch.zeros(2, 4, 3)
    mn = torch.zeros(2, 5, 3, 3)
    rhs = torch.zeros(2, 5, 3)
    with pytest.raises(ValueError, match="rhs must have shape"):
        validate_block_tridiagonal(lo, mn, lo, torch.zeros(2, 5))
    with pytest.raises(ValueError, match="lower must have shape"):
        validate_block_tridiagonal(torch.zeros(2, 5, 3), mn, lo, rhs)
    with pytest.raises(ValueError, match="main must have shape"):
        validate_block_tridiagonal(lo, torch.zeros(2, 5, 9), lo, rhs)
    with pytest.raises(ValueError, match="CUDA"):
        validate_block_tridiagonal(lo, mn, lo, rhs)
    L = dendra_gb300.load()
    assert L.dgb_block3_work_size(0, 10, 7) == 0
    assert L.dgb_block3_solve(0, 0, 4, None, None, None, None, None, None, 0, None) == -1


def test_delay_contract_errors_on_the_host():
    """Argument errors of the interpolated-delay entry points come back before
    any launch (dummy pointers are never dereferenced)."""
    L = dendra_gb300.load()
    p = 16  # a non-null address that is never touched
    # dtype
    assert L.dgb_two_tap_enqueue(7, p, 4, 4, p, 1, p, p, None, 0, p, p, p, p, p, p, p, None,
                                 None) == -1
    # an empty ring cannot receive edges
    assert L.dgb_two_tap_enqueue(0, p, 4, 0, p, 3, p, p, None, 0, p, p, p, p, p, p, p, None,
                                 None) == -1
    assert b"Empty ring" in L.dgb_last_error()
    # missing column plan
    assert L.dgb_two_tap_enqueue(0, p, 4, 4, p, 3, p, p, None, 0, p, p, p, None, p, p, p, None,
                                 None) == -1
    # source indices without sources
    assert L.dgb_two_tap_rollout(0, p, 4, 4, p, 2, 3, p, p, 0, p, 0, p, p, p, p, p, 0, None,
                                 None) == -1
    # negative step count
    assert L.dgb_two_tap_rollout_vjp(1, p, 4, 4, p, -1, 3, p, p, 0, None, 0, p, p, p, p, p, 0,
                                     None, None, None, 0, p, p, p, None, None) == -1
    # a rollout plan is required
    assert L.dgb_two_tap_rollout(0, p, 4, 4, p, 2, 3, p, p, 0, None, 0, p, None, p, p, p, 0,
                                 None, None) == -1
    # gates by source need source indices
    assert L.dgb_two_tap_rollout(0, p, 4, 4, p, 2, 3, p, p, 8, None, 0, p, p, p, p, p, 8 | 16,
                                 None, None) == -1
    assert L.dgb_gates_by_source(0, 10, 3, p, p, 9, None) == -1
    # gather of an empty ring
    assert L.dgb_two_tap_gather(0, p, 0, p, 3, p, p, p, p, None) == -1
    assert L.dgb_three_tap_vjp(0, p, 0, 4, p, 2, p, p, p, p, p, p, p, p, None) == -1


def test_block_tree_contract_errors_on_the_host():
    import torch

    from dendra_gb300.tree import validate_tree_block

    rhs = torch.zeros(2, 5, 3)
    main = torch.zeros(2, 5, 3, 3)
    edge = torch.zeros(2, 5, 3)
    i = torch.zeros(5, dtype=torch.int64)
    lp = torch.tensor([0, 5])
    with pytest.raises(ValueError, match="rhs must have shape"):
        validate_tree_block(main, edge, torch.zeros(2, 5), i, i, lp, 16)
    with pytest.raises(ValueError, match="edge must have shape"):
        validate_tree_block(main, torch.zeros(2, 5, 2), rhs, i, i, lp, 16)
    with pytest.raises(ValueError, match="main must have shape"):
        validate_tree_block(torch.zeros(2, 5, 9), edge, rhs, i, i, lp, 16)
    with pytest.raises(ValueError, match="CUDA"):  # data must live on the GPU
        validate_tree_block(main, edge, rhs, i, i, lp, 16)
    L = dendra_gb300.load()
    p = 16
    assert L.dgb_dhs_block3_solve(0, 0, 4, p, p, p, p, p, p, 1, p, p, p, 0, None) == -1
    assert L.dgb_dhs_block3_solve(0, 2, 4, p, p, p, p, p, p, 1, p, p, p, 0, None) == -1  # alias


def test_cable_flag_constants_match_the_header():
    text = open(os.path.join(ROOT, "include", "dendra_gb300.h")).read()
    defined = {m.group(1): int(m.group(2))
               for m in re.finditer(r"#define DGB_(CABLE_\w+) (\d+)", text)}
    assert "CABLE_SPLIT_GATES" in defined
    for name, value in defined.items():
        assert getattr(_lib, name) == value, name


def test_cable_run_flag_checks_on_the_host():
    """Unknown flag bits and a split-gate run with lane classes are refused
    before any device work (the pointers are never read)."""
    L = dendra_gb300.load()
    a = _lib.CableArgs()
    a.dtype, a.n_cables, a.n_steps, a.rec_every, a.max_k, a.n_comp = 0, 1, 4, 1, 11, 11
    for name in ("cable_ptr", "v", "m", "h", "n", "g_right", "g_left", "scale", "cm_inv",
                 "gnabar", "gkbar", "gl", "el", "scratch"):
        setattr(a, name, 4096)
    a.flags = 32
    assert L.dgb_cable_run(ctypes.byref(a), None) == -1
    assert b"unknown flags" in L.dgb_last_error()
    a.flags = _lib.CABLE_SPLIT_GATES
    a.lanes_mode, a.n_lanes32, a.n_lanes16 = 1, 1, 0
    assert L.dgb_cable_run(ctypes.byref(a), None) == -1
    assert b"lanes_mode 0" in L.dgb_last_error()
