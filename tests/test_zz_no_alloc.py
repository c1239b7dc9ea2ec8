"""The allocation-free cable step (dgb_cable_step_static) through the C ABI.

Callers that cannot allocate device memory on their call path (a host that
preallocates all GPU memory at start-up, a plugin running while another
runtime owns the CUDA allocator) use dgb_cable_step_static: the step's band
scratch lives in a fixed array inside the library.  These tests check that
two calls in a row give the same state as the allocating entry points
(dgb_cable_assemble + dgb_cable_solve_update with caller-allocated bands), and
that populations beyond the array's capacity are rejected.  The file is
collected last so that a failure here leaves every other test already run.
"""

import ctypes

import numpy as np
import pytest
import torch

from dendra_gb300 import _lib
from tests._cases import synthetic_population

pytestmark = pytest.mark.gpu

# Both paths run the same two kernels on the same inputs; only the band
# scratch lives elsewhere, so the states must agree bit for bit.


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_static_step_matches_allocating_step(cuda, dtype):
    ref = synthetic_population(21, 48, 1, 401, dtype, cuda, intra=True)
    new = synthetic_population(21, 48, 1, 401, dtype, cuda, intra=True)
    L = _lib.load()
    for _ in range(2):  # two calls in a row share and reuse the static scratch
        ref.step_plain()
        args = new._args(1)
        rc = L.dgb_cable_step_static(ctypes.byref(args), 0, _lib.stream_ptr(cuda))
        _lib.check(rc, "dgb_cable_step_static")
        new.step_index += 1
        new.t += new.dt
        torch.cuda.synchronize()
        for name in ("v", "m", "h", "n"):
            assert torch.equal(getattr(new, name), getattr(ref, name)), name
    assert bool(torch.isfinite(new.v).all())


def test_static_step_rejects_populations_beyond_capacity(cuda):
    pop = synthetic_population(3, 4, 51, 101, torch.float64, cuda)
    args = pop._args(1)
    args.n_comp = 131072 + 1  # float64 capacity of the 4 MiB array is 131,072 compartments
    L = _lib.load()
    rc = L.dgb_cable_step_static(ctypes.byref(args), 0, _lib.stream_ptr(cuda))
    assert rc == -4
    assert b"static scratch holds" in L.dgb_last_error()
