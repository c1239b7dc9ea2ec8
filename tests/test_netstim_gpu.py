"""NetStim renewal generators on the GPU, through the C ABI: bit-exact against
the reference's own trajectory (supplied draws) and against the oracle's
counter-based draws; packed spike words; split runs."""

import numpy as np
import pytest
import torch

import oracle
from dendra_gb300.netstim import NetStim

pytestmark = pytest.mark.gpu

TAGS = [("f64", np.float64, torch.float64), ("f32", np.float32, torch.float32)]


@pytest.mark.parametrize("tag,npt,tdt", TAGS)
def test_renewal_matches_reference(cuda, golden, tag, npt, tdt):
    z = golden(f"netstim_{tag}.npz")
    ns = NetStim(9, z["interval"], z["noise"], z["start"], z["number"], dtype=tdt, device=cuda)
    ns.initialize(draws=z["draws0"])
    np.testing.assert_array_equal(ns.next_stoch_time.cpu().numpy(), z["next_time"][0])
    spikes = ns.run(z["draws"].shape[0], float(z["dt"]), draws=z["draws"])
    np.testing.assert_array_equal(spikes.cpu().numpy(), z["spikes"])
    np.testing.assert_array_equal(ns.next_stoch_time.cpu().numpy(), z["next_time"][-1])
    np.testing.assert_array_equal(ns.spike_counts.cpu().numpy(), z["counts"][-1])


def _params(n, seed):
    rng = np.random.default_rng(seed)
    iv = rng.uniform(0.5, 30.0, n)
    nz = rng.choice([0.0, 0.25, 1.0], n)
    st = rng.uniform(0.0, 5.0, n)
    num = rng.integers(0, 40, n)
    return iv, nz, st, num


@pytest.mark.parametrize("tag,npt,tdt", TAGS)
def test_counter_draws_match_oracle(cuda, tag, npt, tdt):
    n, steps, dt = 1000, 700, 0.025
    iv, nz, st, num = _params(n, 3)
    ns = NetStim(n, iv, nz, st, num, seed=0xDEADBEEF12345, dtype=tdt, device=cuda)
    nxt0, cnt0 = oracle.netstim_init(iv, nz, st, seed=0xDEADBEEF12345, dtype=npt)
    np.testing.assert_array_equal(ns.next_stoch_time.cpu().numpy(), nxt0)
    spikes, bits = ns.run(steps, dt, t0=0.0, bits=True)
    nxt, cnt, ospk = oracle.netstim_run(nxt0, cnt0, steps, iv.astype(npt), nz.astype(npt), num,
                                        dt=dt, seed=0xDEADBEEF12345)
    np.testing.assert_array_equal(spikes.cpu().numpy(), ospk)
    np.testing.assert_array_equal(ns.next_stoch_time.cpu().numpy(), nxt)
    np.testing.assert_array_equal(ns.spike_counts.cpu().numpy(), cnt)
    # packed words: bit g % 64 of word g // 64
    words = bits.cpu().numpy().view(np.uint64)
    unpacked = ((words[:, :, None] >> np.arange(64, dtype=np.uint64)) & 1).reshape(steps, -1)
    np.testing.assert_array_equal(unpacked[:, :n].astype(np.uint8), ospk)
    assert not unpacked[:, n:].any()


def test_split_runs_continue_identically(cuda):
    n = 300
    iv, nz, st, num = _params(n, 4)
    a = NetStim(n, iv, nz, st, None, seed=9, device=cuda)
    b = NetStim(n, iv, nz, st, None, seed=9, device=cuda)
    whole = a.run(500, 0.025)
    parts = torch.cat([b.run(123, 0.025), b.run(377, 0.025)])
    torch.testing.assert_close(whole, parts, rtol=0, atol=0)
    torch.testing.assert_close(a.next_stoch_time, b.next_stoch_time, rtol=0, atol=0)


def test_background_rate(cuda):
    """The 4,096-cell network's background: 4,096 Poisson generators at 5 Hz over 200 ms."""
    ns = NetStim(4096, interval=200.0, noise=1.0, start=0.0, seed=2024, device=cuda)
    spikes = ns.run(8000, 0.025)
    total = int(spikes.sum())
    # first clock E*200 ms plus renewals: expected count 4096 * (1 - e^-1) + ... ~ 4096
    assert 3600 < total < 4600


def test_deterministic_initialisation_keeps_start_for_nonfinite_intervals(cuda):
    """Without noise the first clock is start itself (the reference's
    netstim_initial_state: no inf * 0, a negative zero stays negative)."""
    ns = NetStim(2, interval=[float("inf"), float("nan")], noise=0.0, start=[-0.0, 2.0],
                 dtype=torch.float64, device=cuda)
    clock = ns.next_stoch_time.cpu()
    assert clock[1].item() == 2.0 and clock[0].item() == 0.0
    assert torch.signbit(clock[0])
