"""Host-side pieces of bench.py on CPU: the clock-sample summary that decides
whether a timed run is kept, and the synthetic system generators."""

import numpy as np
import torch

import bench
import oracle


def _summary(lines):
    s = bench.ClockSampler(0)
    s.lines = list(lines)
    return s.summary()


def test_clock_summary_median_and_reasons():
    ok = "0, {mhz}, 2070, 900.0, 0x0, Not Active, Not Active, Not Active, {cap}"
    lines = [ok.format(mhz=m, cap="Not Active") for m in (2070, 2070, 1965)]
    lines.append(ok.format(mhz=1800, cap="Active"))
    lines.append("garbage line")
    out = _summary(lines)
    assert out["samples"] == 4
    assert out["sm_mhz"] == float(np.median([2070, 2070, 1965, 1800]))
    assert out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"]


def test_clock_summary_flags_thermal_slowdown_and_empty_runs():
    line = "0, 1500, 2070, 1390.0, 0x40, Not Active, Active, Active, Not Active"
    assert _summary([line])["reasons"] == ["hw_thermal_slowdown", "sw_thermal_slowdown"]
    empty = _summary([])
    assert empty["samples"] == 0 and empty["sm_mhz"] is None


def test_tridiagonal_workload_is_diagonally_dominant_and_solvable():
    a, b, c, d = bench._tridiag_system(8, 401, 11, torch.float64)
    assert a.shape == (8, 400) and b.shape == (8, 401)
    off = torch.zeros_like(b)
    off[:, 1:] += a.abs()
    off[:, :-1] += c.abs()
    assert bool((b > off).all())
    x = oracle.thomas(*(t.numpy() for t in (a, b, c, d)))
    A = np.diag(b[0].numpy()) + np.diag(a[0].numpy(), -1) + np.diag(c[0].numpy(), 1)
    assert np.abs(A @ x[0] - d[0].numpy()).max() < 1e-12


def test_reference_arm_of_single_solve_workloads_runs_on_the_host():
    """``bench.py --impl reference`` for the solver workloads times the
    oracle's CPU solve and prints one reference line, without a GPU."""
    import json
    import os
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for workload, unit in (("tridiag", "row-solves/s"), ("bt", "compartment-solves/s"),
                           ("tree", "node-solves/s")):
        out = subprocess.run(
            [sys.executable, "bench.py", "--workload", workload, "--impl", "reference",
             "--steps", "1", "--warmup", "0", "--cables", "64"],
            cwd=root, capture_output=True, text=True, timeout=300, check=True)
        line = json.loads(out.stdout.strip().splitlines()[-1])
        assert line["impl"] == "reference" and line["unit"] == unit
        assert line["value"] > 0 and line["cpu_baseline"]["kind"] == "port"
        assert line["e2e"]["h2d_bytes_per_step"] == 0


def test_launch_override_sets_cables_per_cta_or_split_gates():
    from types import SimpleNamespace

    pop = SimpleNamespace(warps_per_block=0, split_gates=False)
    bench._apply_launch(pop, "-1")
    assert pop.split_gates and pop.warps_per_block == 0
    bench._apply_launch(pop, "2,0,0")
    assert not pop.split_gates and pop.warps_per_block == 2
    bench._apply_launch(pop, "")
    assert not pop.split_gates and pop.warps_per_block == 2
