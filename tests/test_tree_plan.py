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


def test_forest_plan_offsets_match_kernel_indexing():
    """Replay the forest kernel's index arithmetic on the host for every plan."""
    from dendra_gb300.tree import ForestPlan

    rng = np.random.default_rng(3)
    parents = []
    for K in (1, 2, 5, 40, 300, 1, 77):
        p = [-1] + [int(rng.integers(0, i)) for i in range(1, K)]
        parents.append(p)
    plan = ForestPlan(parents, device="cpu")
    T = {k: v.numpy() for k, v in plan.tensors.items()}
    for pidx, parent in enumerate(parents):
        K = len(parent)
        pn = int(T["plan_node_ptr"][pidx])
        assert int(T["plan_node_ptr"][pidx + 1]) - pn == K
        cptr = T["child_ptr"][pn + pidx: pn + pidx + K + 1]
        cidx = T["child_idx"][pn: pn + K]
        assert cptr[-1] <= K - 1 + (1 if K == 1 else 0)
        for i in range(K):
            kids = sorted(cidx[cptr[i]:cptr[i + 1]].tolist())
            assert kids == [c for c in range(K) if parent[c] == i]
        assert T["parent"][pn: pn + K].tolist() == parent
        lo, hi = int(T["plan_layer_off"][pidx]), int(T["plan_layer_off"][pidx + 1])
        lptr = T["layer_ptr"][lo:hi]
        assert lptr[0] == 0 and lptr[-1] == K
        assert sorted(T["order"][pn: pn + K].tolist()) == list(range(K))
    assert T["child_idx"].size == int(T["plan_node_ptr"][-1])
