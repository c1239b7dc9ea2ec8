"""NetStim renewal: the oracle against the reference's own trajectory (CPU only).

``netstim_{f64,f32}.npz`` hold netstim_initial_state and 600 steps of
netstim_renewal (networks/_netstim_renewal.py) run by the reference with a
supplied table of unit-exponential draws.
"""

import math

import numpy as np
import pytest

import oracle

TAGS = [("f64", np.float64), ("f32", np.float32)]


def _golden_run(z, dt):
    nxt, cnt = oracle.netstim_init(z["interval"], z["noise"], z["start"], draws=z["draws0"],
                                   dtype=dt)
    return nxt, cnt, oracle.netstim_run(nxt, cnt, z["draws"].shape[0], z["interval"].astype(dt),
                                        z["noise"].astype(dt), z["number"], dt=float(z["dt"]),
                                        draws=z["draws"].astype(dt))


@pytest.mark.parametrize("tag,dt", TAGS)
def test_oracle_renewal_matches_reference(golden, tag, dt):
    z = golden(f"netstim_{tag}.npz")
    nxt0, cnt0, (nxt, cnt, spikes) = _golden_run(z, dt)
    np.testing.assert_array_equal(nxt0, z["next_time"][0])
    np.testing.assert_array_equal(cnt0, z["counts"][0])
    np.testing.assert_array_equal(spikes, z["spikes"])
    np.testing.assert_array_equal(nxt, z["next_time"][-1])
    np.testing.assert_array_equal(cnt, z["counts"][-1])
    # the caps hold: generator 8 has number 0, generators 1 and 5 stop at 3 and 2
    assert spikes[:, 8].sum() == 0 and spikes[:, 1].sum() <= 3 and spikes[:, 5].sum() <= 2


@pytest.mark.parametrize("tag,dt", TAGS)
def test_split_runs_continue_identically(golden, tag, dt):
    z = golden(f"netstim_{tag}.npz")
    nxt0, cnt0 = oracle.netstim_init(z["interval"], z["noise"], z["start"], seed=5, dtype=dt)
    iv, nz = z["interval"].astype(dt), z["noise"].astype(dt)
    a = oracle.netstim_run(nxt0, cnt0, 500, iv, nz, z["number"], seed=5)
    b1 = oracle.netstim_run(nxt0, cnt0, 200, iv, nz, z["number"], seed=5)
    b2 = oracle.netstim_run(b1[0], b1[1], 300, iv, nz, z["number"], step0=200, seed=5)
    np.testing.assert_array_equal(a[2], np.concatenate([b1[2], b2[2]]))
    np.testing.assert_array_equal(a[0], b2[0])


def test_philox_known_answers():
    """Philox4x32-10 known-answer vectors of the published algorithm."""
    cases = [
        ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
        ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
        ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
         [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
    ]
    for ctr, key, want in cases:
        np.testing.assert_array_equal(oracle.philox4x32_10(ctr, key), np.array(want, np.uint32))


def test_series_log_is_accurate():
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.random(20000), np.exp(-rng.random(2000) * 700), [1.0, 0.5, 2e-300]])
    for x in xs:
        want = math.log(x)
        got = oracle.series_log(x)
        assert abs(got - want) <= 4e-16 * max(1.0, abs(want)), (x, got, want)


@pytest.mark.parametrize("dt_", [np.float64, np.float32])
def test_device_generator_statistics(dt_):
    """Poisson (noise 1) and periodic (noise 0) generators with the counter draws."""
    n, steps, dt = 200, 40000, 0.025  # 1 s
    iv = np.full(n, 10.0)
    nz = np.where(np.arange(n) < n // 2, 1.0, 0.0)
    st = np.zeros(n)
    nxt, cnt = oracle.netstim_init(iv, nz, st, seed=11, dtype=dt_)
    _, cnt, spikes = oracle.netstim_run(nxt, cnt, steps, iv.astype(dt_), nz.astype(dt_),
                                        seed=11, dt=dt)
    poisson = spikes[:, : n // 2]
    isi = np.concatenate([np.diff(np.flatnonzero(poisson[:, g])) for g in range(n // 2)]) * dt
    assert abs(isi.mean() - 10.0) < 0.3
    assert abs(isi.std() / isi.mean() - 1.0) < 0.05
    # periodic generators fire every 400 steps from step 0
    periodic = spikes[:, n // 2:]
    assert (periodic.sum(0) == steps // 400).all()
    np.testing.assert_array_equal(np.flatnonzero(periodic[:, 0]), np.arange(0, steps, 400))
