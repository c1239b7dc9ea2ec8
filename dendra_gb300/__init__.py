"""dendra_gb300 — GB300-native (sm_103a) kernels for Dendra's per-timestep cable update.

Drop-in pieces for the reference's solver-dispatch and run APIs:

* ``solvers``  — ``thomas_solve_cuda_t`` / ``pcr_solve_cuda_t`` (batched tridiagonal)
* ``cable``    — ``CablePopulation``: packed HH cable populations, persistent
                 multi-step runs and the unfused per-step path
* ``tree``     — DHS/Hines tree solve ``dhs_solve_cuda`` and its topology plan
* ``netcon``   — spike bit-packing and deterministic delayed delivery

All compute runs in ``_build/libdendra_gb300.so`` through the C ABI declared in
``include/dendra_gb300.h``; there is no CPU fallback.
"""

from . import _lib  # noqa: F401
from .solvers import pcr_solve_cuda_t, thomas_solve_cuda_t  # noqa: F401

__version__ = "0.1.0"


def library_path() -> str:
    return _lib.path()


def load():
    """Build if needed and load the CUDA library (raises if unavailable)."""
    return _lib.load()
