"""Pathwise adjoint against central finite differences over a longer horizon.

The short adjoint tests (600 steps) resolve only the fast parameters.  Here
the golden mesh runs 20,000 steps (0.18 ms at dt = 9 ns) of its spark source
with gating off (RyR 4 held open, so the trajectory is deterministic and the
loss differentiable), the x line scan sampled every 500 steps, loss
  L = 1/2 sum_k sum_i (F_ki / F0_i - 1 - target_ki)^2.
The adjoint runs on the FP32 resident engine (checkpoints every 1000
steps); the finite differences are central, h = 1e-4 |theta|, on the FP64
engine.  Every parameter of the gradient must agree to 1e-3 relative,
among them SERCA A_P, the calmodulin / troponin / SL-site kon, koff and
capacity, which the short horizon leaves below rounding.
"""
import numpy as np
import pytest

from conftest import GOLDEN_MESH, LINESCAN_DESC, params_from_golden

pytestmark = pytest.mark.gpu

N_STEPS, TICK, K = 20000, 500, 1000


def _params(srs):
    p, _ = params_from_golden(srs, "spark")
    p.ints[srs.I["FLAG_NO_FLUX_BOUNDARY"]] = 1
    p.ints[srs.I["FLAG_NO_GATING"]] = 1
    return p


def _sim(srs, p, precision, engine):
    g = srs.Grid(p, GOLDEN_MESH)
    sim = srs.Simulation(g, p, 1, precision, engine, seeds=[5])
    sim.reset()
    sim.linescan_setup(**LINESCAN_DESC)
    return sim


def test_adjoint_matches_finite_differences_over_20000_steps(srs):
    p0 = _params(srs)
    sim = _sim(srs, p0, srs.FP32, srs.ENGINE_RESIDENT)
    _, f0 = sim.linescan()
    rng = np.random.default_rng(7)
    target = rng.standard_normal((N_STEPS // TICK, len(f0))) * 0.01
    start = sim.get_state(0)
    loss, grad, _ = sim.adjoint(N_STEPS, TICK, f0, target[None], checkpoint_every=K)

    # the gradient is taken at a fixed initial state (the reset state of the
    # unperturbed parameters: the equilibrium buffer levels depend on kon and
    # koff), so every finite-difference run starts from that same state
    def loss_of(p):
        s = _sim(srs, p, srs.FP64, srs.ENGINE_PLAIN)
        s.set_state(0, start["states"], start["ryr"], start["lcc"], start["lccv"], start["residuals"])
        L = 0.0
        for k in range(N_STEPS // TICK):
            s.explicit_step(TICK)
            F, _ = s.linescan()
            e = F[0] / f0 - 1.0 - target[k]
            L += 0.5 * float((e * e).sum())
        return L

    L0 = loss_of(p0)
    assert abs(loss[0] - L0) <= 1e-5 * L0
    report = {}
    for k, name in enumerate(srs.ADJ_PARAMS):
        idx = srs.R[name]
        h = 1e-4 * abs(p0.reals[idx])
        hi, lo = p0.copy(), p0.copy()
        hi.reals[idx] += h
        lo.reals[idx] -= h
        fd = (loss_of(hi) - loss_of(lo)) / (2 * h)
        report[name] = (float(grad[0, k]), fd)
    bad = {n: v for n, v in report.items() if not abs(v[0] - v[1]) <= 1e-3 * abs(v[1])}
    assert not bad, (bad, report)
    # the parameters the short horizon cannot resolve are resolved here
    for name in ("A_P", "K_ON_CMDN", "K_OFF_CMDN", "K_ON_TRPN", "K_OFF_TRPN", "B_TOT_SL_HI",
                 "K_D_SL_HI"):
        assert report[name][1] != 0.0, name
