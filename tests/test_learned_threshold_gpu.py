"""The learned bracket: same accepted thresholds as plain bisection, fewer trials."""

import numpy as np
import pytest
import torch

from dendra_gb300.mlp import BF16MLP, fibre_features
from dendra_gb300.threshold import (Thresholder, fibre_params, fibre_population, horizon_steps,
                                    learned_thresholds)

pytestmark = pytest.mark.gpu


def _plain(p, cuda):
    pop = fibre_population(p, device=cuda)
    th = Thresholder(pop, lb=0.0, ub=0.1, rtol=0.01)
    ub, lb = th.calculate_thresholds(horizon_steps(p["pw"].max()))
    return ub, lb, th


def test_learned_bracket_gains_over_plain_bisection(cuda):
    train = fibre_params(8192, seed=11)
    ub, lb, _ = _plain(train, cuda)
    ok = torch.isfinite(ub).cpu()
    X = fibre_features(train)[ok]
    y = torch.log(ub.cpu()[ok]).float()
    mlp = BF16MLP(device=cuda, seed=0)
    mlp.train(X, y, epochs=40, batch=512, lr=2e-3)
    # margin from held-out error
    val = fibre_params(1024, seed=12)
    vub, _, _ = _plain(val, cuda)
    vok = torch.isfinite(vub).cpu()
    err = (mlp.predict(fibre_features(val)).cpu().double() - torch.log(vub.cpu()))[vok].abs()
    margin = float(torch.quantile(err, 0.95))
    test = fibre_params(1024, seed=13)
    pub, plb, th_plain = _plain(test, cuda)
    pop = fibre_population(test, device=cuda)
    th = Thresholder(pop, lb=0.0, ub=0.1, rtol=0.01)
    pred = torch.exp(mlp.predict(fibre_features(test)).double())
    lub, llb = learned_thresholds(th, pred, margin, horizon_steps(test["pw"].max()))
    fin = torch.isfinite(pub) & torch.isfinite(lub)
    assert int(fin.sum()) >= 0.95 * int(torch.isfinite(pub).sum())
    # both are accepted brackets (width < 1%) of the same threshold
    assert bool((((lub - llb) / lub)[fin] < 0.01).all())
    assert bool(((llb[fin] <= pub[fin]) & (plb[fin] <= lub[fin])).all())
    print(f"median |log err| {float(err.median()):.4f}, margin {margin:.4f}; trials plain "
          f"{th_plain.trials} ({th_plain.fibre_steps:.3e} fibre-steps), learned {th.trials} "
          f"({th.fibre_steps:.3e} fibre-steps)")
    assert th.fibre_steps < 0.6 * th_plain.fibre_steps
