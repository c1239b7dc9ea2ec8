"""Host-side tree planning against the reference's own plans (CPU only)."""

import numpy as np
import pytest

from dendra_gb300.tree import build_dhs_layers, build_morphology, children_csr


@pytest.mark.parametrize("threads", [1, 8, 32])
def test_layers_match_reference_plan(golden, threads):
    g = golden("dhs.npz")
    _, _, depth = build_morphology(g["parity_parent"].tolist())
    order, layer_ptr = build_dhs_layers(depth, threads)
    np.testing.assert_array_equal(order.numpy(), g[f"parity_order_t{threads}"])
    np.testing.assert_array_equal(layer_ptr.numpy(), g[f"parity_layer_ptr_t{threads}"])


def test_random_tree_plan_matches_reference(golden):
    g = golden("dhs.npz")
    _, _, depth = build_morphology(g["rand_parent"].tolist())
    np.testing.assert_array_equal(depth.numpy(), g["rand_depth"])
    order, layer_ptr = build_dhs_layers(depth, 32)
    np.testing.assert_array_equal(order.numpy(), g["rand_order_t32"])
    np.testing.assert_array_equal(layer_ptr.numpy(), g["rand_layer_ptr_t32"])


def test_children_csr():
    ptr, idx = children_csr([-1, 0, 0, 1, 1, 2, 5])
    assert ptr.tolist() == [0, 2, 4, 5, 5, 5, 6, 6]
    assert idx.tolist() == [1, 2, 3, 4, 5, 6]


@pytest.mark.parametrize("bad,err", [([-1, -1], ValueError), ([0, -1, 5], ValueError),
                                     ([-1, 1], ValueError), ([-1, 2, 1], ValueError)])
def test_morphology_errors(bad, err):
    with pytest.raises(err):
        build_morphology(bad)


def test_threads_validation():
    with pytest.raises(ValueError):
        build_dhs_layers(np.array([0, 1]), 3)
    with pytest.raises(TypeError):
        build_dhs_layers(np.array([0, 1]), True)
