"""The oracle's reverse mode against the reference's autograd gradient and
against central finite differences (CPU only)."""

import numpy as np
import torch

from tests._cases import golden_adjoint_population, oracle_param_grads


def _problem(pop, rhoa):
    p = pop.problem_dict()
    p["rhoa_per_cable"] = np.asarray(rhoa, dtype=np.float64)
    return p


def test_oracle_gradient_matches_reference_autograd(golden):
    g = golden("adjoint_f64.npz")
    steps = int(g["steps"])
    pop = golden_adjoint_population(g, torch.float64)
    trace, loss, grads, _ = oracle_param_grads(_problem(pop, g["guess_rhoa"]), steps, g["target"])
    # the forward itself matches the reference's recorded somatic trace
    np.testing.assert_allclose(trace, g["trace"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(loss, g["loss"], rtol=1e-9)
    for k in ("gnabar", "gkbar", "gl", "rhoa"):
        np.testing.assert_allclose(grads[k], g[f"grad_{k}"], rtol=1e-7, err_msg=k)


def test_oracle_gradient_matches_central_differences(golden):
    """h = 1e-4 relative central differences of the oracle's own forward."""
    g = golden("adjoint_f64.npz")
    steps = int(g["steps"])
    pop = golden_adjoint_population(g, torch.float64)
    p0 = _problem(pop, g["guess_rhoa"])
    _, loss0, grads, _ = oracle_param_grads(p0, steps, g["target"])
    h = 1e-4
    B = loss0.size

    def loss_at(name, factor):
        p = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in p0.items()}
        if name == "rhoa":  # the axial bands scale as 1/Ra
            p["g_right"] = p["g_right"] / factor
            p["g_left"] = p["g_left"] / factor
        else:
            p[name] = p[name] * factor
        return oracle_param_grads(p, steps, g["target"])[1]

    for name in ("gnabar", "gkbar", "gl", "rhoa"):
        base = g[f"guess_{name}"]
        fd = (loss_at(name, 1 + h) - loss_at(name, 1 - h)) / (2 * h * base)
        # O(h^2) truncation: relative to the largest component of this gradient
        np.testing.assert_allclose(grads[name], fd, rtol=1e-5, atol=1e-5 * np.abs(fd).max(),
                                   err_msg=name)
    assert B == 3
