"""Tree-contraction plan and oracle on the CPU; the C ABI's host-side checks.

The oracle restates the reference kernel's arithmetic
(models/integrators/triton/tree_contraction.py) on this package's plan; here it
is checked against dense solves of the Hines matrix for every plan shape
(segment caps, fine contraction, forests, arbitrary node order) and the
planner's invariants are checked directly.
"""

import ctypes

import numpy as np
import pytest

import oracle
from dendra_gb300 import _lib
from dendra_gb300.contraction import (DgbContractPlan, TreeContractionPlan,
                                      build_contraction_tables)

# the reference's integration-test morphology
# (tests/func/test_tree_contraction_integration.py:20-35): edges parent -> child
REF_EDGES = ((7, 1), (1, 2), (2, 3), (3, 4), (4, 0), (4, 5), (7, 6))


def ref_parent():
    p = np.full(8, -1)
    for a, b in REF_EDGES:
        p[b] = a
    return p


def random_tree(rng, K, branch):
    """Random tree in a shuffled node order (parents need not precede children)."""
    p = np.full(K, -1)
    for i in range(1, K):
        p[i] = i - 1 if rng.random() > branch else rng.integers(0, i)
    perm = rng.permutation(K)
    q = np.full(K, -1)
    for i in range(K):
        q[perm[i]] = perm[p[i]] if p[i] >= 0 else -1
    return q


def systems(rng, B, K, dtype=np.float64):
    d = rng.uniform(0.05, 2.0, (B, K)).astype(dtype)
    g = rng.uniform(0.5, 20.0, (B, K)).astype(dtype)
    b = rng.normal(size=(B, K)).astype(dtype)
    return d, g, b


def dense(d, g, b, parent):
    return np.stack([np.linalg.solve(oracle.hines_matrix(d[r], g[r], parent), b[r].astype(np.float64))
                     for r in range(d.shape[0])])


@pytest.mark.parametrize("cap", [None, 1, 2, 3, 16])
@pytest.mark.parametrize("K,branch", [(1, 0.0), (2, 0.0), (3, 0.5), (9, 0.3), (64, 0.0),
                                      (64, 0.15), (150, 0.6)])
def test_oracle_matches_dense_solve(cap, K, branch):
    rng = np.random.default_rng(K * 31 + (cap or 0))
    parent = random_tree(rng, K, branch)
    tables, _ = build_contraction_tables(parent, cap)
    d, g, b = systems(rng, 3, K)
    x = oracle.tree_contract_solve(d, g, b, tables)
    np.testing.assert_allclose(x, dense(d, g, b, parent), rtol=1e-12, atol=1e-13)


@pytest.mark.parametrize("cap", [None, 2])
def test_reference_morphology_and_forest(cap):
    rng = np.random.default_rng(5)
    for parent in (ref_parent(), np.array([-1, 0, 0, -1, 3, 4, 5, -1])):
        tables, counts = build_contraction_tables(parent, cap)
        assert counts["n_roots"] == int((parent < 0).sum())
        d, g, b = systems(rng, 2, parent.size)
        x = oracle.tree_contract_solve(d, g, b, tables)
        np.testing.assert_allclose(x, dense(d, g, b, parent), rtol=1e-12, atol=1e-13)


def test_float32_oracle_is_float32_accurate():
    rng = np.random.default_rng(2)
    parent = random_tree(rng, 300, 0.05)
    tables, _ = build_contraction_tables(parent, 16)
    d, g, b = systems(rng, 2, 300, np.float32)
    x = oracle.tree_contract_solve(d, g, b, tables)
    assert x.dtype == np.float32
    np.testing.assert_allclose(x, dense(d, g, b, parent), rtol=2e-5, atol=2e-6)


def test_segments_respect_the_cap_and_rounds_are_logarithmic():
    K = 1025
    chain = np.arange(K) - 1  # an unbranched cable as a tree
    tables, c = build_contraction_tables(chain, None)
    assert c["n_segments"] == 0 and c["n_retained"] == K
    assert c["n_rounds"] <= 2 * int(np.ceil(np.log2(K)))
    for cap in (1, 4, 16):
        tables, c = build_contraction_tables(chain, cap)
        seg = tables["seg"]
        assert (seg[3] - seg[2]).max() <= cap
        assert c["n_interior"] + c["n_retained"] == K
    # a balanced binary tree needs no segments and contracts in O(log K) rounds
    K = 1023
    binary = np.array([-1] + [(i - 1) // 2 for i in range(1, K)])
    tables, c = build_contraction_tables(binary, 16)
    assert c["n_segments"] == 0 and c["n_rounds"] <= 2 * 10


@pytest.mark.parametrize("cap", [False, 0, -1, 2.5, "auto"])
def test_invalid_cap_is_rejected(cap):
    # the reference's messages (integrators/__init__.py:82-91)
    with pytest.raises((TypeError, ValueError), match="max_segment_interior_nodes"):
        TreeContractionPlan(np.array([-1, 0, 1]), cap)


@pytest.mark.parametrize("parent,msg", [([0, 0], "own parent"), ([1, 0], "root"),
                                         ([-1, 2, 1], "cycle"), ([-1, 5], "must be in"),
                                         ([], "non-empty")])
def test_invalid_topology_is_rejected(parent, msg):
    with pytest.raises(ValueError, match=msg):
        TreeContractionPlan(np.asarray(parent, dtype=np.int64))


def test_struct_mirror_and_host_errors():
    L = _lib.load()
    assert L.dgb_contract_plan_size() == ctypes.sizeof(DgbContractPlan)
    plan = DgbContractPlan()
    plan.size = 4
    p = 16
    # bad dtype, null plan, inconsistent counts: rejected before any device work
    assert L.dgb_tree_contract_solve(7, 1, ctypes.byref(plan), p, p, p, 32, None, 0, None) == -1
    assert L.dgb_tree_contract_solve(0, 1, None, p, p, p, 32, None, 0, None) == -1
    assert L.dgb_tree_contract_solve(0, 1, ctypes.byref(plan), p, p, p, 32, None, 0, None) == -1
    assert L.dgb_tree_contract_solve(0, 1, ctypes.byref(plan), p, p, p, p, None, 0,
                                     None) == -1  # alias
    assert L.dgb_tree_contract_solve(0, 0, ctypes.byref(plan), None, None, None, None, None, 0,
                                     None) == 0  # empty batch
    assert L.dgb_tree_contract_work_size(0, None, 4) == 0
