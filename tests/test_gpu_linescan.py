"""Device line scan against a numpy restatement of linescan/main.cpp:160-225."""
import numpy as np
import pytest

from conftest import GOLDEN_MESH, LINESCAN_DESC as DESC, linescan_weights, params_from_golden

pytestmark = pytest.mark.gpu


def restated(srs, grid, states_by_r, d=DESC):
    W, pad = linescan_weights(grid, d)
    N = grid.n_ele
    return np.array([pad + W @ S[5 * N:6 * N] for S in states_by_r])


@pytest.mark.parametrize("prec,eng", [(64, 0), (32, 0), (32, 1)])
def test_linescan_matches_restatement(srs, prec, eng):
    p, _ = params_from_golden(srs, "spark")
    g = srs.Grid(p, GOLDEN_MESH)
    sim = srs.Simulation(g, p, 3, prec, eng, seeds=[1, 2, 3])
    ns = sim.linescan_setup(**DESC)
    F0, rest = sim.linescan()
    want0 = restated(srs, g, [g.initial_states(p)])
    assert np.allclose(rest, want0[0], rtol=1e-12, atol=0)
    assert np.allclose(F0, want0[0][None, :], rtol=1e-6 if prec == 32 else 1e-12)
    sim.explicit_step(2000)
    F, _ = sim.linescan()
    want = restated(srs, g, [sim.get_state(r)["states"] for r in range(3)])
    assert F.shape == (3, ns)
    assert np.allclose(F, want, rtol=1e-12, atol=0)
    assert (F > F0).any()  # the open RyR raised the bound dye somewhere on the line


def test_linescan_matches_reference_tool_output(srs):
    """The device line scan against the reference's own line-scan tool
    (linescan/main.cpp) on three states of the golden mesh whose grid files
    the reference wrote (tests/golden/linescan_tool.npz, from
    tests/golden/gen_linescan_tool.py).  The tool prints %g (six significant
    digits), so the bar is 5e-6 relative."""
    import json
    import os

    from conftest import GOLDEN
    d = np.load(os.path.join(GOLDEN, "linescan_tool.npz"))
    desc = json.loads(str(d["desc"]))
    states = d["states"]
    p, _ = params_from_golden(srs, "spark")
    g = srs.Grid(p, GOLDEN_MESH)
    sim = srs.Simulation(g, p, len(states), srs.FP64, srs.ENGINE_PLAIN, seeds=[1, 2, 3])
    for r, S in enumerate(states):
        sim.set_state(r, states=S)
    sim.linescan_setup(**desc)
    F, _ = sim.linescan()
    assert F.shape == d["tool_output"].shape
    assert np.allclose(F, d["tool_output"], rtol=5e-6, atol=0), np.abs(F / d["tool_output"] - 1).max()
