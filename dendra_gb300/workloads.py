"""Seeded synthetic workloads with the shapes and distributions of the benchmark configs.

``cable_population_c1``: 64 HH cables x 101 compartments (Unmyelinated,
L = 1000 um, dx = 10 um, diam 1 um, Ra 100 ohm cm), float64, somatic
1 ms current pulse at 5 ms of U[0.05, 0.5] nA, dt 0.025 ms, 2000 steps.

``cable_population_c2``: 16,384 HH cables, odd compartment counts uniform in
[51, 401], diameter U[0.5, 4] um, length U[500, 5000] um (dx = L/K), Ra 100,
float32; each cable sees a point source in a homogeneous medium
(sigma = 0.3 S/m -> rho_e = 333.33 ohm cm) at distance U[0.5, 3] mm from its
centre, delivering a cathodic 0.1 ms pulse of U[0.1, 2] mA at t = 0;
dt 0.005 ms for 10 ms (2000 steps).

``cable_population_c4``: 1,024 HH cables of 201 compartments (Unmyelinated,
L = 2010 um, dx = 10 um -> K = 201, diam 1 um), float32, dt 0.025 ms for
20,000 steps (500 ms); a somatic step current of U[0.1, 0.4] nA from 5 ms to
485 ms drives repetitive firing.  ``c4_spec`` also draws the hidden per-cable
gnabar, gkbar, gl and Ra (defaults x U[0.7, 1.3]) whose somatic traces are the
fit targets; the initial guesses are the defaults.

No public dataset is involved; the generators stand in for the reference's
configurations with the stated distributions.
"""

from __future__ import annotations

import numpy as np
import torch

from .cable import HH_DEFAULTS, CablePopulation, unmyelinated_K

RHOE_OHM_CM = 1.0 / 0.3 * 100.0  # sigma = 0.3 S/m


def c2_spec(n_cables=16384, seed=2024, kmin=51, kmax=401):
    rng = np.random.default_rng(seed)
    ks = 2 * rng.integers((kmin - 1) // 2, (kmax - 1) // 2 + 1, n_cables) + 1
    return dict(
        ks=ks,
        diam=rng.uniform(0.5, 4.0, n_cables),
        length=rng.uniform(500.0, 5000.0, n_cables),
        dist=rng.uniform(500.0, 3000.0, n_cables),
        amp=-rng.uniform(0.1, 2.0, n_cables),
    )


def cable_population_c2(n_cables=16384, seed=2024, dtype=torch.float32, device="cuda",
                        subset=None, fast_math=False):
    """The 16,384-cable population (K 51-401, point-source pulse), optionally only
    the cables listed in ``subset``."""
    s = c2_spec(n_cables, seed)
    idx = np.arange(n_cables) if subset is None else np.asarray(subset)
    ks = s["ks"][idx]
    dx = s["length"][idx] / ks
    pop = CablePopulation(ks.tolist(), torch.as_tensor(s["diam"][idx]), torch.as_tensor(dx),
                          rhoa=100.0, celsius=6.3, v_init=-65.0, dtype=dtype, device=device,
                          fast_math=fast_math)
    x = pop.positions()
    cab = np.repeat(np.arange(len(idx)), ks)
    r_cm = torch.sqrt(x ** 2 + torch.as_tensor(s["dist"][idx][cab]) ** 2) * 1e-4
    field = RHOE_OHM_CM / (4 * torch.pi * r_cm)
    pop.set_extracellular(field, torch.as_tensor(s["amp"][idx]), 0.0, 0.1)
    return pop.initialize(0.005)


C2_STEPS = 2000


def cable_population_c1(seed=1, dtype=torch.float64, device="cuda", n_cables=64):
    rng = np.random.default_rng(seed)
    amp_na = rng.uniform(0.05, 0.5, n_cables)
    pop = CablePopulation([101] * n_cables, 1.0, 10.0, rhoa=100.0, celsius=6.3, v_init=-65.0,
                          dtype=dtype, device=device)
    pop.inject(0, torch.as_tensor(amp_na * 1e-6), 5.0, 1.0)
    return pop.initialize(0.025)


C1_STEPS = 2000


C4_STEPS = 20000
C4_CHECKPOINT = 500


def c4_spec(n_cables=1024, seed=4):
    rng = np.random.default_rng(seed)
    amp_na = rng.uniform(0.1, 0.4, n_cables)
    defaults = dict(gnabar=HH_DEFAULTS["gnabar"], gkbar=HH_DEFAULTS["gkbar"],
                    gl=HH_DEFAULTS["gl"], ra=100.0)
    hidden = {k: v * rng.uniform(0.7, 1.3, n_cables) for k, v in defaults.items()}
    guess = {k: np.full(n_cables, v) for k, v in defaults.items()}
    return dict(K=unmyelinated_K(2010.0, 10.0), amp_ma=amp_na * 1e-6, delay=5.0, pw=480.0,
                hidden=hidden, guess=guess)


def cable_population_c4(n_cables=1024, seed=4, dtype=torch.float32, device="cuda",
                        fast_math=False):
    """The 1,024 × 201 gradient-fit population at the default parameters (the
    guesses)."""
    s = c4_spec(n_cables, seed)
    pop = CablePopulation([s["K"]] * n_cables, 1.0, 10.0, rhoa=100.0, celsius=6.3,
                          v_init=-65.0, dtype=dtype, device=device, fast_math=fast_math)
    pop.inject(0, torch.as_tensor(s["amp_ma"]), s["delay"], s["pw"])
    return pop.initialize(0.025), s
