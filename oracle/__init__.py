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
    HH rates, cnexp, the backward-Euler cable update, Thomas, PCR, 3x3 block
    Thomas, DHS and the
    branched-cell network step (``orc_net_run``: Exp2Syn delivery, soma HH,
    tree solve, delay ring), and the reverse mode of the cable update
    (``cable_grad``: full state tape, transposed Thomas solve, gate partials
    on the forward's branches), and the interpolated delay transport
    (``two_tap_enqueue`` / ``three_tap_enqueue`` / ``two_tap_vjp`` and their
    multi-step rollouts: the reference's ordered CPU op, sequential adds), and
    the NetStim renewal with counter-based draws (Philox4x32-10, a series
    logarithm in rounded operations).
  * ``core.py``  ctypes bindings; builds the C library with gcc on first use;
    numpy restatements of the 3x3 block tree and SPD solves and of the tree
    contraction solve (``tree_contract_solve``: the reference kernel's
    operation order on a given plan).
  The integer/index event primitives (delay rounding, bit packing, sequential
  delivery) are restated inline in ``tests/test_netcon.py``, next to the
  reference known answers they are checked against.
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
    block3_solve,
    cable_run,
    cable_grad,
    dhs_solve,
    net_run,
    num_threads,
    two_tap_enqueue,
    three_tap_enqueue,
    two_tap_vjp,
    two_tap_rollout,
    two_tap_rollout_vjp,
    philox4x32_10,
    series_log,
    unit_exponential,
    netstim_init,
    netstim_run,
    dhs_block3_matrix,
    dhs_block3_solve,
    block3_spd_solve,
    tree_contract_solve,
    hines_matrix,
)
