"""Plan caches must never return the plan of a freed tensor whose address was reused."""

import gc

import numpy as np
import pytest
import torch

from dendra_gb300._cache import TensorKeyedCache


def test_identity_and_version_key():
    cache = TensorKeyedCache(4)
    built = []

    def build(tag):
        built.append(tag)
        return tag

    a = torch.arange(8)
    assert cache.get((a,), 1, lambda: build("a")) == "a"
    assert cache.get((a,), 1, lambda: build("again")) == "a"  # hit
    assert cache.get((a,), 2, lambda: build("a2")) == "a2"  # other extra key
    a.add_(1)  # in-place change bumps the version
    assert cache.get((a,), 1, lambda: build("a'")) == "a'"
    b = a.clone()  # equal contents, another tensor: never shares a's entry
    assert cache.get((b,), 1, lambda: build("b")) == "b"
    assert cache.get((None, a), 1, lambda: build("none")) == "none"
    assert built == ["a", "a2", "a'", "b", "none"]
    assert len(cache) == 4


def test_entry_keeps_address_alive():
    """While an entry exists its tensor cannot be freed, so a new tensor never
    lands on the cached address."""
    cache = TensorKeyedCache(8)
    x = torch.zeros(1 << 16, dtype=torch.int64)
    ptr = x.data_ptr()
    cache.get((x,), None, lambda: "x")
    del x
    gc.collect()
    ys = [torch.ones(1 << 16, dtype=torch.int64) for _ in range(4)]
    assert all(y.data_ptr() != ptr for y in ys)
    assert all(cache.get((y,), None, lambda: "y") == "y" for y in ys)


def test_lru_eviction():
    cache = TensorKeyedCache(2)
    ts = [torch.zeros(2) for _ in range(3)]
    for i, t in enumerate(ts):
        cache.get((t,), None, lambda i=i: i)
    assert len(cache) == 2
    assert cache.get((ts[0],), None, lambda: "rebuilt") == "rebuilt"


@pytest.mark.gpu
def test_dhs_new_topology_same_size(cuda):
    """Solve one tree, free its plan tensors, build a different tree with the same
    node count (the allocator tends to hand back the same addresses) and check
    the second solve against the dense matrix of the second tree."""
    from dendra_gb300.tree import build_dhs_layers, build_morphology, dhs_solve_cuda

    import oracle

    rng = np.random.default_rng(5)
    K, B = 64, 3

    def plan(parent):
        _, _, depth = build_morphology(list(parent))
        order, layer_ptr = build_dhs_layers(depth, 32)
        return (torch.as_tensor(np.asarray(parent), device=cuda), order.to(cuda).long(),
                layer_ptr.to(cuda).long())

    def solve_and_check(parent):
        d = 1.0 + rng.random((B, K))
        a = 0.5 * rng.random((B, K))
        a[:, 0] = 0.0
        b = rng.standard_normal((B, K))
        p = plan(parent)
        x = dhs_solve_cuda(*(torch.as_tensor(t, device=cuda) for t in (d, a, b)), *p, threads=32)
        ref = oracle.dhs_solve(d, a, b, np.asarray(parent), p[1].cpu().numpy(),
                               p[2].cpu().numpy())
        np.testing.assert_allclose(x.cpu().numpy(), ref, rtol=1e-11, atol=1e-12)

    chain = [-1] + list(range(K - 1))  # unbranched
    star = [-1] + [0] * (K - 1)  # every node on the root
    solve_and_check(chain)
    gc.collect()
    solve_and_check(star)


@pytest.mark.gpu
def test_build_delivery_new_targets_same_size(cuda):
    """Two connection lists of the same length with different targets, the
    first freed before the second is made."""
    from dendra_gb300.netcon import build_delivery, n_words_for, pack_source_spikes

    n_src, n_post, n_conn, depth = 10, 7, 40, 4
    rng = np.random.default_rng(1)
    hist = torch.zeros((depth, n_words_for(n_src)), dtype=torch.int64, device=cuda)
    step = torch.tensor([0], device=cuda)
    pack_source_spikes(torch.ones(n_src, dtype=torch.bool, device=cuda), hist, step)
    pre = rng.integers(0, n_src, n_conn)
    word = torch.as_tensor(pre // 63, device=cuda)
    mask = torch.as_tensor(np.left_shift(np.int64(1), pre % 63), device=cuda)
    delay = torch.zeros(n_conn, dtype=torch.int64, device=cuda)
    w = torch.as_tensor(rng.random(n_conn), device=cuda)
    for trial in range(2):
        post_np = rng.integers(0, n_post, n_conn)
        post = torch.as_tensor(post_np, device=cuda)
        out = torch.zeros(n_post, dtype=torch.float64, device=cuda)
        build_delivery(hist, step, delay, word, mask, post, w, out)
        ref = np.zeros(n_post)
        np.add.at(ref, post_np, w.cpu().numpy())
        np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=1e-14)
        del post, out
        gc.collect()
