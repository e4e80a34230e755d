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


def test_large_mesh_plain_adjoint_matches_finite_differences(srs, tmp_path):
    """The plain engine's adjoint on a mesh of 65,536 elements and more (the
    split forward form; the forward state and lambda keep their compensation
    terms as halves on every mesh):
    1024 steps of the spark source with gating off against central
    differences of the FP64 engine (h = 1e-4 |theta|), 1e-3 relative on every
    parameter the horizon resolves."""
    base = str(tmp_path / "big")
    rep = srs.write_box_mesh(base, box_x=3.0, box_y=3.0, box_z=3.0, foot_half_x=0.3,
                             foot_half_y=0.3, n_foot_x=10, n_foot_y=10, n_out_x=6, n_out_y=6,
                             n_above_z=22)
    assert rep["n_tets"] >= 65536
    n, te = 1024, 128
    desc = dict(axis=0, offset1=0.0, offset2=0.1, x_min=-1.0, x_max=1.0, res=0.05, var_x=0.0289,
                var_y=0.1154, var_z=0.0289, r_thresh=1.0, f0_pad=0.0, pad_res=0.0, pad_min=0.0,
                pad_max=0.0, domain=(0, 0, 0, 0, 0, 0))
    p0 = srs.default_parameters().set(T_STEP=9e-6, FLAG_CLOCK_SEED=0, INIT_RYR=24, FLAG_NO_GATING=1)

    def make(p, prec):
        s = srs.Simulation(srs.Grid(p, base), p, 1, prec, srs.ENGINE_PLAIN, seeds=[3])
        s.reset()
        s.linescan_setup(**desc)
        return s

    sim = make(p0, srs.FP32)
    _, f0 = sim.linescan()
    start = sim.get_state(0)
    target = np.random.default_rng(9).standard_normal((n // te, len(f0))) * 0.01
    loss, grad, _ = sim.adjoint(n, te, f0, target[None], checkpoint_every=256)

    def loss_of(p):
        s = make(p, srs.FP64)
        s.set_state(0, start["states"], start["ryr"], start["lcc"], start["lccv"], start["residuals"])
        L = 0.0
        for k in range(n // te):
            s.explicit_step(te)
            F, _ = s.linescan()
            e = F[0] / f0 - 1.0 - target[k]
            L += 0.5 * float((e * e).sum())
        return L

    L0 = loss_of(p0)
    assert abs(loss[0] - L0) <= 1e-5 * L0
    checked, bad = [], {}
    for k, name in enumerate(srs.ADJ_PARAMS):
        idx = srs.R[name]
        h = 1e-4 * abs(p0.reals[idx])
        hi, lo = p0.copy(), p0.copy()
        hi.reals[idx] += h
        lo.reals[idx] -= h
        Lp, Lm = loss_of(hi), loss_of(lo)
        if abs(Lp - Lm) < 1e-9 * L0:
            continue  # below the loss's rounding over this horizon
        fd = (Lp - Lm) / (2 * h)
        if not abs(grad[0, k] - fd) <= 1e-3 * abs(fd):
            bad[name] = (float(grad[0, k]), fd)
        checked.append(name)
    assert not bad, bad
    assert {"D_CA", "K_ON_DYE", "K_OFF_DYE", "V_RYR"} <= set(checked), checked
