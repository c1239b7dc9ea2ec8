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


def test_chain_schedule_structure_and_same_elimination():
    """build_chains: a partition of the nodes into unbranched chains, levels
    after their child chains, and (replayed in numpy, one operation at a time)
    the same elimination and substitution as the depth-layer schedule."""
    import numpy as np

    from dendra_gb300.network import random_cell
    from dendra_gb300.tree import build_chains, build_dhs_layers, build_morphology

    rng = np.random.default_rng(4)
    for k in (1, 2, 7, 250, 1400):
        parent = random_cell(rng, k).parent if k > 2 else np.arange(k) - 1
        K = len(parent)
        cn, cp, cl = build_chains(parent)
        assert sorted(cn.tolist()) == list(range(K))
        kids = [[] for _ in range(K)]
        for i, p in enumerate(parent):
            if p >= 0:
                kids[p].append(i)
        chain_of, level_of = {}, {}
        for lv in range(cl.size - 1):
            for c in range(cl[lv], cl[lv + 1]):
                nodes = cn[cp[c]:cp[c + 1]]
                for q, n in enumerate(nodes):
                    chain_of[int(n)] = c
                    if q + 1 < len(nodes):
                        assert parent[n] == nodes[q + 1] and len(kids[nodes[q + 1]]) == 1
                assert len(kids[nodes[0]]) != 1
                top_parent = parent[nodes[-1]]
                assert top_parent < 0 or len(kids[top_parent]) >= 2
                level_of[c] = lv
        for c, lv in level_of.items():
            bottom = cn[cp[c]]
            assert all(level_of[chain_of[ch]] < lv for ch in kids[bottom])
        # replay both schedules
        d = rng.uniform(1.0, 2.0, K)
        g = rng.uniform(0.1, 1.0, K)
        b = rng.standard_normal(K)
        cptr = [0]
        cidx = []
        for i in range(K):
            cidx.extend(kids[i])
            cptr.append(len(cidx))

        def pull(i, D, B):
            Dv, Bv = D[i], B[i]
            for c in kids[i]:
                f = g[c] * (1.0 / (D[c] + g[c]))
                Dv = Dv + f * D[c]
                Bv = Bv + f * B[c]
            D[i], B[i] = Dv, Bv

        _, _, depth = build_morphology([int(v) for v in parent])
        order, lptr = build_dhs_layers(depth, 32)
        D1, B1 = d.copy(), b.copy()
        for lv in range(lptr.numel() - 1):
            for o in range(int(lptr[lv]), int(lptr[lv + 1])):
                pull(int(order[o]), D1, B1)
        for lv in range(lptr.numel() - 2, -1, -1):
            for o in range(int(lptr[lv]), int(lptr[lv + 1])):
                i = int(order[o])
                xp = B1[parent[i]] if parent[i] >= 0 else 0.0
                B1[i] = (B1[i] + g[i] * xp) / (D1[i] + g[i])
        D2, B2 = d.copy(), b.copy()
        for c in range(cp.size - 1):
            for n in cn[cp[c]:cp[c + 1]]:
                pull(int(n), D2, B2)
        for c in range(cp.size - 2, -1, -1):
            for n in cn[cp[c]:cp[c + 1]][::-1]:
                xp = B2[parent[n]] if parent[n] >= 0 else 0.0
                B2[n] = (B2[n] + g[n] * xp) / (D2[n] + g[n])
        np.testing.assert_array_equal(D1, D2)
        np.testing.assert_array_equal(B1, B2)
