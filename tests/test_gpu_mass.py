"""Total Ca per compartment (srs_sim_total_ca), FP64 accumulation.

With SERCA, refill and boundary fluxes off, gating off and RyR 4 held open,
Ca only moves from the JSR to the cleft and through the cytosol.  The total
over both compartments is then conserved by the explicit step up to the
scheme's own O(dt^2) error of the rapid-buffer Euler update (2e-8 relative
after 20k steps on the golden mesh, measured with the FP64 oracle).
"""
import numpy as np
import pytest

from conftest import GOLDEN_MESH, params_from_golden

pytestmark = pytest.mark.gpu

STEPS, CHUNKS = 5000, 4


def _params(srs):
    p, _ = params_from_golden(srs, "spark")
    p.ints[srs.I["FLAG_NO_FLUX_BOUNDARY"]] = 1
    p.ints[srs.I["FLAG_NO_GATING"]] = 1
    p.reals[srs.R["A_P"]] = 0.0
    p.reals[srs.R["V_REFILL"]] = 0.0
    return p


def _numpy_total(srs, g, p, S):
    el = g.elements()
    N = g.n_ele
    c = S[:N]
    bound = S[N:].reshape(5, N).sum(axis=0)
    bhi = el["TT"] * p.reals[srs.R["B_TOT_SL_HI"]] / (el["V0"] * 1e-15)
    blo = el["TT"] * p.reals[srs.R["B_TOT_SL_LO"]] / (el["V0"] * 1e-15)
    t = el["V0"] * (c + bound + bhi * c / (p.reals[srs.R["K_D_SL_HI"]] + c) +
                    blo * c / (p.reals[srs.R["K_D_SL_LO"]] + c))
    return np.array([t[el["domain"] == 0].sum(), t[el["domain"] == 1].sum()])


def _run(srs, precision, engine):
    p = _params(srs)
    g = srs.Grid(p, GOLDEN_MESH)
    sim = srs.Simulation(g, p, 2, precision, engine, seeds=[1, 2])
    sim.reset()
    out = [sim.total_ca()]
    states = [sim.get_state(0)["states"]]
    for _ in range(CHUNKS):
        sim.explicit_step(STEPS)
        out.append(sim.total_ca())
        states.append(sim.get_state(0)["states"])
    return p, g, np.array(out), states


def test_total_ca_fp64_engine_matches_numpy_and_is_conserved(srs):
    p, g, tot, states = _run(srs, srs.FP64, srs.ENGINE_PLAIN)
    for k, S in enumerate(states):
        assert np.allclose(tot[k, 0], _numpy_total(srs, g, p, S), rtol=1e-13, atol=0)
    both = tot.sum(axis=2)
    assert np.all(np.abs(both - both[0]) <= 1e-7 * both[0])
    assert tot[-1, 0, 0] > tot[0, 0, 0] and tot[-1, 0, 1] < tot[0, 0, 1]  # JSR -> cleft


@pytest.mark.parametrize("engine", [0, 1])
def test_total_ca_fp32_engines_match_fp64(srs, engine):
    _, _, t64, _ = _run(srs, srs.FP64, srs.ENGINE_PLAIN)
    _, _, t32, _ = _run(srs, srs.FP32, engine)
    assert np.all(np.abs(t32 - t64) <= 1e-6 * np.abs(t64))
