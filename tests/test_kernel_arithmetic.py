"""CPU checks of two pieces of the cable kernels' arithmetic, restated here.

* The state-tape walk of the persistent run (``rows_store_state`` in
  csrc/cable_rows.cuh) advances (lane, slot) by (P // ch, P % ch) with one
  carry instead of dividing per row; it must visit the same (row, lane, slot)
  triples as row i -> (lane0 + i // ch, i % ch).
* ``div_c`` in csrc/common.cuh divides by the rate constants 10, 18, 20 and 80
  in float64 as q = RN(x rc), rc = RN(1/c), corrected once by the FMA
  remainder, RN(q + rc RN(x - q c)).  It must equal the correctly rounded
  quotient x / c for every finite x in the rates' range.  The FMAs are
  evaluated here in exact rational arithmetic and rounded once, as the
  hardware does.
"""

from fractions import Fraction

import numpy as np
import pytest


def _walk(r, lane0, P, ch, K):
    L, j = lane0 + r // ch, r % ch
    dl, dj = P // ch, P % ch
    out = []
    for i in range(r, K, P):
        out.append((i, L, j))
        L += dl
        j += dj
        if j >= ch:
            j -= ch
            L += 1
    return out


@pytest.mark.parametrize("P", [8, 16, 32])
def test_tape_walk_visits_the_same_rows_as_the_division_form(P):
    for ch in range(1, 33):
        for K in sorted({1, P * ch // 2 + 1, P * ch - 1, P * ch}):
            for lane0 in (0, 32 - P):
                for r in range(P):
                    want = [(i, lane0 + i // ch, i % ch) for i in range(r, K, P)]
                    assert _walk(r, lane0, P, ch, K) == want, (P, ch, K, lane0, r)


def _rn(q):
    """Fraction -> nearest float64 (ties to even): Python's int true division
    is correctly rounded."""
    return q.numerator / q.denominator


def _fma(a, b, c):
    return _rn(Fraction(a) * Fraction(b) + Fraction(c))


def _div_c(x, c):
    rc = 1.0 / c
    q = x * rc
    return _fma(_fma(-q, c, x), rc, q)


@pytest.mark.parametrize("c", [10.0, 18.0, 20.0, 80.0])
def test_constant_division_is_the_correctly_rounded_quotient(c):
    rng = np.random.default_rng(int(c))
    # the rates divide v + 35, v + 40, v + 55 or v + 65 (mV): voltages from
    # -200 to 200 mV, plus values near 0, binade edges, multiples of c and the
    # doubles just above them
    xs = list(rng.uniform(-265.0, 265.0, 4000))
    xs += list(rng.uniform(-1e-3, 1e-3, 500))
    xs += [float(c) * k for k in range(-40, 41)]
    xs += [np.nextafter(float(c) * k, np.inf) for k in range(-40, 41)]
    xs += [2.0 ** e for e in range(-20, 9)] + [-(2.0 ** e) for e in range(-20, 9)]
    xs += [5e-324, -5e-324, 0.0]
    corrected = 0
    for x in xs:
        x = float(x)
        got = _div_c(x, c)
        want = x / c
        assert got == want, (x, c, got, want)
        corrected += x * (1.0 / c) != want
    # the plain product x RN(1/c) misses the quotient often (about a third of
    # the uniform samples): the correction is doing the work
    assert corrected > len(xs) // 5
