"""Event transport: reference known answers (CPU) and GPU kernels vs oracles."""

import numpy as np
import pytest
import torch

from dendra_gb300.netcon import (DenseRing, build_delivery, detect_spikes, exp2syn_factor,
                                 inference_delay_steps, n_words_for, pack_source_spikes,
                                 source_word_and_mask)


def test_delay_rounding_known_answers(golden):
    """tests/networks/test_event_delivery_contract.py:103-116 values."""
    g = golden("events.npz")
    dt = 0.025
    steps, inference = inference_delay_steps(torch.as_tensor(g["round_ratios"]) * dt, dt)
    assert steps.tolist() == g["round_delay_steps"].tolist()
    assert inference.tolist() == g["round_inference_steps"].tolist()


def test_exp2syn_factor_matches_reference(golden):
    g = golden("events.npz")
    f = exp2syn_factor(g["exp2syn_tau1"], g["exp2syn_tau2"])
    np.testing.assert_allclose(f.numpy(), g["exp2syn_factor"], rtol=1e-15, atol=0)
    with pytest.raises(ValueError):
        exp2syn_factor([0.0], [1.0])


@pytest.mark.gpu
def test_ring_sequence_matches_reference_bit_exact(cuda, golden):
    """dense_fixed_delay_transition sequence recorded from the reference (float64)."""
    g = golden("events.npz")
    n_conn = g["post"].size
    ring = DenseRing(int(g["depth"]), int(g["width"]), np.arange(n_conn), g["post"], g["delay"],
                     g["weight"], device=cuda, dtype=torch.float64)
    for s in range(g["gates"].shape[0]):
        due = ring.due()
        np.testing.assert_array_equal(due.cpu().numpy(), g["delivered"][s])
        ring.transition(torch.as_tensor(g["gates"][s] > 0, device=cuda))
    np.testing.assert_array_equal(ring.ring.cpu().numpy(), g["final_queue"])
    assert int(ring.slot.item()) == int(g["final_slot"])


@pytest.mark.gpu
@pytest.mark.parametrize("n_source", [1, 62, 63, 64, 126, 127, 4096])
def test_pack_matches_int64_oracle(cuda, n_source):
    rng = np.random.default_rng(n_source)
    spikes = rng.random(n_source) < 0.3
    n_words = n_words_for(n_source)
    hist = torch.full((5, n_words), -1, dtype=torch.int64, device=cuda)
    step = torch.tensor([3], device=cuda)
    pack_source_spikes(torch.as_tensor(spikes, device=cuda), hist, step)
    words = np.zeros(n_words, dtype=np.int64)
    for s in np.nonzero(spikes)[0]:
        words[s // 63] |= np.int64(1) << np.int64(s % 63)
    np.testing.assert_array_equal(hist[3].cpu().numpy(), words)
    assert (hist[[0, 1, 2, 4]] == -1).all()  # other rows untouched
    assert (hist[3] >= 0).all()  # bit 63 never set


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_build_delivery_matches_sequential_oracle(cuda, dtype):
    rng = np.random.default_rng(11)
    n_source, n_post, n_conn, depth = 200, 37, 5000, 9
    pre = rng.integers(0, n_source, n_conn)
    post = rng.integers(0, n_post, n_conn)
    delay = rng.integers(1, depth, n_conn)
    weight = rng.lognormal(-7, 0.5, n_conn)
    hist_bits = rng.random((depth, n_source)) < 0.2
    n_words = n_words_for(n_source)
    hist = np.zeros((depth, n_words), dtype=np.int64)
    for r in range(depth):
        for s in np.nonzero(hist_bits[r])[0]:
            hist[r, s // 63] |= np.int64(1) << np.int64(s % 63)
    now = 4
    out0 = rng.standard_normal(n_post)
    ref = out0.astype(np.float64 if dtype == torch.float64 else np.float32).copy()
    for e in range(n_conn):  # reference semantics, sequential in connection order
        row = (now - delay[e]) % depth
        if hist_bits[row, pre[e]]:
            ref[post[e]] = ref[post[e]] + ref.dtype.type(weight[e])
    word, mask = source_word_and_mask(pre)
    out = torch.as_tensor(out0, dtype=dtype, device=cuda)
    t = lambda x: torch.as_tensor(x, device=cuda)
    build_delivery(t(hist), t([now]), t(delay), word.to(cuda), mask.to(cuda), t(post),
                   torch.as_tensor(weight, dtype=dtype, device=cuda), out)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


@pytest.mark.gpu
def test_detect_spikes_rising_edge(cuda):
    v = torch.tensor([-70.0, 0.0, 10.0, 5.0, -1.0], device=cuda)
    below = torch.tensor([1, 1, 0, 1, 0], dtype=torch.uint8, device=cuda)
    spikes = detect_spikes(v, below, 0.0)
    assert spikes.tolist() == [0, 1, 0, 1, 0]
    assert below.tolist() == [1, 0, 0, 0, 1]
