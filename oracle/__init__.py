"""CPU oracle for the Dendra cable update — TEST INFRASTRUCTURE ONLY.

This package restates the reference algorithms on the CPU so that tests,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` can check
and time the CUDA path.  Nothing in ``dendra_gb300`` imports it: the product
path has no CPU fallback.

Parity status: pinned.  ``tests/golden/`` holds vectors produced by running the
reference implementation itself (``tests/golden/make_golden.py``), and
``tests/test_oracle_golden.py`` checks this oracle against them.

Layers:
  * ``oracle.c`` / ``oracle_impl.h``  float64 and float32 C restatements of the
    HH rates, cnexp, the backward-Euler cable update, Thomas, PCR and DHS,
    and the reverse mode of the cable update (``cable_grad``: full state
    tape, transposed Thomas solve, gate partials on the forward's branches).
  * ``events.py``  numpy restatement of NetCon delay rounding, the dense delay
    ring and bit-packed delivery (integer/index work).
  * ``trees.py``   numpy restatement of the tree topology plan and the DHS
    right-hand-side assembly.
"""

from .core import (  # noqa: F401
    build,
    lib,
    vtrap,
    phi1,
    hh_rates,
    hh_steady,
    cnexp,
    thomas,
    pcr,
    cable_run,
    cable_grad,
    dhs_solve,
    net_run,
    num_threads,
)
